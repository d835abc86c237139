"""GPU parity of the binomial fill (mm_binomial through the package's ctypes layer) against the
reference's own outputs (tests/golden/binomial_golden.npz) and the CPU oracle.

Tolerances: amplitudes 1e-13 of max|G| (the GPU computes them with the vanilla kernels' fused
arithmetic), the stop weight exactly (identical zero pattern), the norm 1e-14 relative."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import mrmustard_gb300 as mm

pytestmark = pytest.mark.gpu


def rel(x, ref):
    return float(np.abs(np.asarray(x) - ref).max() / np.abs(ref).max())


def ket(M, seed, smax=0.6, sigma=0.6):
    from scipy.stats import unitary_group

    rng = np.random.default_rng(seed)
    U = unitary_group.rvs(M, random_state=seed) if M > 1 else np.exp(1j * rng.uniform(0, 6, (1, 1)))
    A = (U * rng.uniform(0.0, smax, M)) @ U.T
    b = sigma * (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / np.sqrt(2)
    return A, b, 0.5 + 0.1j


def test_golden_cases(cuda, binomial_golden):
    g = binomial_golden
    for n in g["names"]:
        l2, gc = g[f"{n}/params"]
        G, norm = mm.binomial(tuple(g[f"{n}/shape"]), g[f"{n}/A"], g[f"{n}/b"], g[f"{n}/c"], l2, int(gc))
        ref = g[f"{n}/G"]
        assert np.array_equal(G == 0, ref == 0), n
        assert rel(G, ref) < 1e-13, n
        assert abs(norm - float(g[f"{n}/norm"])) < 1e-14 * float(g[f"{n}/norm"]), n


@pytest.mark.parametrize("shape,l2", [((40,), 0.9), ((9000,), 0.99), ((30, 25), 0.95), ((12, 11, 10), 0.999),
                                      ((20, 20, 30), 0.9), ((6, 7, 5, 8), 0.99), ((4, 4, 3, 5, 3), 0.9)])
def test_vs_oracle(cuda, oracle_lib, shape, l2):
    A, b, c = ket(len(shape), 300 + sum(shape), smax=0.5, sigma=0.4)
    # scale c so the running norm crosses l2 part-way through the fill
    gc = sum(shape) - len(shape) + 1
    G, norm = mm.binomial(shape, A, b, c, l2, gc)
    ref, rnorm, stop = oracle_lib.binomial(shape, A, b, c, l2, gc)
    assert np.array_equal(G == 0, ref == 0)
    assert rel(G, ref) < 1e-13
    assert abs(norm - rnorm) < 1e-14 * rnorm


def test_no_early_stop_is_vanilla_up_to_global_cutoff(cuda, oracle_lib):
    A, b, c = ket(3, 77)
    shape = (8, 9, 7)
    G, _ = mm.binomial(shape, A, b, c, None, 12)
    V = oracle_lib.vanilla(shape, A, b, c)
    w = np.add.outer(np.add.outer(np.arange(8), np.arange(9)), np.arange(7))
    V[w >= 12] = 0
    assert np.array_equal(G == 0, V == 0)
    assert rel(G, V) < 1e-13


def test_backend_defaults_and_device_mode(cuda, oracle_lib):
    A, b, c = ket(2, 78)
    shape = (15, 12)
    G = mm.hermite_renormalized_binomial(A, b, c, shape)
    ref, _, _ = oracle_lib.binomial(shape, A, b, c, mm.settings.AUTOSHAPE_PROBABILITY, sum(shape) - 2 + 1)
    assert rel(G, ref) < 1e-13 and np.array_equal(G == 0, ref == 0)
    Gd, norm = mm.binomial(shape, torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                           torch.tensor(c, dtype=torch.complex128, device=cuda), 0.9, 20)
    assert Gd.is_cuda and isinstance(norm, float)
    ref, rnorm, _ = oracle_lib.binomial(shape, A, b, c, 0.9, 20)
    assert rel(Gd.cpu().numpy(), ref) < 1e-13
    assert mm.BackendGB300().hermite_renormalized_binomial(A, b, c, shape, 0.9, 20).shape == shape

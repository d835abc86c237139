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


@pytest.mark.parametrize("shape,gc", [((8, 9, 7), 12), ((6, 5, 7, 4), 19), ((30,), 40), ((12, 13), 5)])
def test_no_early_stop_norm(cuda, oracle_lib, shape, gc):
    """max_l2 = None: the fill is the vanilla one up to global_cutoff - 1 (the mask and the norm of
    the kept amplitudes come from the no-stop kernels)."""
    A, b, c = ket(len(shape), 900 + sum(shape), smax=0.5, sigma=0.4)
    G, norm = mm.binomial(shape, A, b, c, None, gc)
    ref, rnorm, _ = oracle_lib.binomial(shape, A, b, c, float("inf"), gc)
    assert np.array_equal(G == 0, ref == 0)
    assert rel(G, ref) < 1e-13
    assert abs(norm - rnorm) < 1e-14 * rnorm


def test_wave_launch_split_is_invisible(cuda, oracle_lib, monkeypatch):
    """The waves' split over one CTA, one cluster and the cooperative grid (picked from the wave
    sizes) changes only the order of the norm's additions: every split gives the oracle's tensor."""
    A, b, c = ket(3, 4242, smax=0.6, sigma=0.5)
    shape = (20, 20, 30)
    ref, rnorm, _ = oracle_lib.binomial(shape, A, b, c, 0.99999, sum(shape) - 2)
    for env in ({}, {"MM_BINOMIAL_TEAM": "0"}, {"MM_BINOMIAL_GRID": "0"}, {"MM_BINOMIAL_CTA_ITEMS": "16"},
                {"MM_BINOMIAL_TEAM_ITEMS": "300"}, {"MM_BINOMIAL_STAGE": "0"}, {"MM_BINOMIAL_BLOCK": "64"},
                {"MM_BINOMIAL_PERM": "0"}, {"MM_BINOMIAL_PERM": "0", "MM_BINOMIAL_STAGE": "0"}):
        for k in ("MM_BINOMIAL_TEAM", "MM_BINOMIAL_GRID", "MM_BINOMIAL_CTA_ITEMS", "MM_BINOMIAL_TEAM_ITEMS",
                  "MM_BINOMIAL_STAGE", "MM_BINOMIAL_BLOCK", "MM_BINOMIAL_PERM"):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        G, norm = mm.binomial(shape, A, b, c, 0.99999, sum(shape) - 2)
        assert np.array_equal(G == 0, ref == 0), env
        assert rel(G, ref) < 1e-13, env
        assert abs(norm - rnorm) < 1e-14 * rnorm, env


@pytest.mark.parametrize("mode_env", [{}, {"MM_BINOMIAL_TEAM": "0", "MM_BINOMIAL_GRID": "0"},
                                      {"MM_BINOMIAL_CTA_ITEMS": "8", "MM_BINOMIAL_TEAM_ITEMS": "40"}])
def test_stop_test_at_the_threshold(cuda, oracle_lib, monkeypatch, mode_env):
    """max_l2 within 1e-12 of the running norm after a weight: the per-weight FP32 estimate cannot
    settle the test there, so the exact norm decides; the fill must stop after that weight when
    max_l2 is just below the norm, after the next one when it is just above."""
    for k, v in mode_env.items():
        monkeypatch.setenv(k, v)
    A, b, c = ket(3, 515, smax=0.5, sigma=0.5)
    shape = (10, 11, 12)
    gc = sum(shape) - 2
    full, _, _ = oracle_lib.binomial(shape, A, b, c, float("inf"), gc)
    w = np.indices(shape).sum(axis=0)
    cum = np.cumsum([np.sum(np.abs(full[w == k]) ** 2) for k in range(gc)])
    for w0 in (3, 7, 12):
        for scale, stop in ((1 - 1e-12, w0), (1 + 1e-12, w0 + 1)):
            G, norm = mm.binomial(shape, A, b, c, float(cum[w0] * scale), gc)
            assert int(w[G != 0].max()) == stop, (w0, scale)
            assert abs(norm - cum[stop]) < 1e-13 * cum[stop]


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

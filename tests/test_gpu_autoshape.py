"""GPU parity of autoshape (mm_autoshape_batched, through the package's ctypes layer) against the
reference's own outputs (tests/golden/autoshape_golden.npz) and the CPU oracle.

The outputs are integers (cutoffs), so parity is exact equality.  The kernel follows the
reference's arithmetic term by term without fused multiply-adds; its complex exp, sqrt and |z|
come from the CUDA math library and may differ from the host's in the last bit, which could move
a cutoff only if a running sum landed within ~1e-15 of max_prob."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import mrmustard_gb300 as mm
from mrmustard_gb300 import _lib

pytestmark = pytest.mark.gpu


def random_dm_triples(B, M, seed, mixed=False):
    """Density-matrix triples of random pure Gaussian states (Takagi A, s < 0.6), optionally with a
    Hermitian bra-ket block added (mixed-state style)."""
    from scipy.stats import unitary_group

    rng = np.random.default_rng(seed)
    As, bs, cs = [], [], []
    for k in range(B):
        U = unitary_group.rvs(M, random_state=seed * 1000 + k) if M > 1 else np.exp(1j * rng.uniform(0, 6, (1, 1)))
        A = (U * rng.uniform(0.0, 0.6, M)) @ U.T
        b = rng.uniform(0.1, 1.0) * (rng.standard_normal(M) + 1j * rng.standard_normal(M)) / np.sqrt(2)
        Adm, bdm, cdm = mm.ket_dm_triple(A, b, rng.uniform(0.2, 0.9))
        if mixed:
            C = U @ np.diag(rng.uniform(0.05, 0.3, M)) @ U.conj().T
            Adm[:M, M:] = C.T
            Adm[M:, :M] = C
        As.append(Adm)
        bs.append(bdm)
        cs.append(cdm)
    return np.array(As), np.array(bs), np.array(cs)


def test_golden_cases(cuda, autoshape_golden):
    g = autoshape_golden
    for n in g["names"]:
        p, hi, lo = g[f"{n}/params"]
        got = mm.autoshape_numba(g[f"{n}/A"], g[f"{n}/b"], g[f"{n}/c"], p, int(hi), int(lo))
        assert got.dtype == np.int64
        assert np.array_equal(got, g[f"{n}/shape"]), (n, got, g[f"{n}/shape"])


def test_known_answers(cuda):
    """Coherent(alpha=1) -> (8,) (test_ket.py:98-100), the vacuum -> (1,) (test_coherent.py:74-75),
    with the reference's default settings (AUTOSHAPE_PROBABILITY 0.99999, MAX 50, MIN 1)."""
    A, b, c = mm.ket_dm_triple(np.zeros((1, 1)), np.array([1.0]), np.exp(-0.5))
    assert tuple(mm.autoshape_numba(A, b, c)) == (8,)
    A, b, c = mm.ket_dm_triple(np.zeros((1, 1)), np.zeros(1), 1.0)
    assert tuple(mm.autoshape_numba(A, b, c)) == (1,)


@pytest.mark.parametrize("M", [1, 2, 3, 4, 5, 6, 7, 8])
@pytest.mark.parametrize("mixed", [False, True])
def test_batched_vs_oracle(cuda, oracle_lib, M, mixed):
    A, b, c = random_dm_triples(64 if M <= 4 else 16, M, 40 + M, mixed)
    for p, hi, lo in ((0.99999, 50, 1), (0.99, 25, 3)):
        got = mm.autoshape_batched(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                                   torch.as_tensor(c, device=cuda), p, hi, lo).cpu().numpy()
        ref = np.array([oracle_lib.autoshape(A[k], b[k], c[k], p, hi, lo) for k in range(len(c))])
        assert np.array_equal(got, ref)


def test_clip_order_and_empty(cuda, oracle_lib):
    """np.clip(k, min_shape, max_shape) with min > max gives max (autoshape.py:154)."""
    A, b, c = mm.ket_dm_triple(np.zeros((1, 1)), np.array([0.7 + 0.2j]), 0.3)
    assert tuple(mm.autoshape_numba(A, b, c, 0.99999, 2, 5)) == tuple(oracle_lib.autoshape(A, b, c, 0.99999, 2, 5))
    out = mm.autoshape_batched(torch.zeros((0, 4, 4), dtype=torch.complex128, device=cuda),
                               torch.zeros((0, 4), dtype=torch.complex128, device=cuda),
                               torch.zeros(0, dtype=torch.complex128, device=cuda))
    assert out.shape == (0, 2)


def test_singular_reduction_raises(cuda):
    """A_nn - X singular (the reference's np.linalg.inv raises LinAlgError)."""
    A = np.zeros((4, 4), np.complex128)
    A[1, 3] = A[3, 1] = 1.0  # mode 1's block equals X, so reducing to mode 0 inverts a zero matrix
    with pytest.raises(np.linalg.LinAlgError):
        mm.autoshape_numba(A, np.zeros(4), 1.0)


def test_too_many_modes_and_launch_count(cuda):
    lib = _lib.load()
    n0 = mm.launch_count()
    A, b, c = random_dm_triples(3, 2, 7)
    mm.autoshape_batched(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                         torch.as_tensor(c, device=cuda))
    assert mm.launch_count() == n0 + 1
    x = torch.zeros((1, 18, 18), dtype=torch.complex128, device=cuda)
    rc = lib.mm_autoshape_batched(1, 9, x.data_ptr(), x.data_ptr(), x.data_ptr(), 0.9, 10, 1, x.data_ptr(), 0)
    assert rc == 2  # MM_ERR_UNSUPPORTED


def test_division_by_reciprocal_is_correctly_rounded(cuda):
    """The recurrence divides by sqrt(k) with three FP64 operations from the correctly rounded
    reciprocal (Markstein's theorem); 2^28 seeded quotients match the correctly rounded division
    bit for bit (exponents 2^-1000..2^1000, both signs, zeros; divisors sqrt(1..100000))."""
    from mrmustard_gb300 import _lib

    lib = _lib.load()
    bad = torch.zeros(1, dtype=torch.int64, device=cuda)
    for seed in (1, 2):
        _lib.check(lib.mm_probe_division(1 << 27, seed, bad.data_ptr(), torch.cuda.current_stream().cuda_stream),
                   "mm_probe_division")
    torch.cuda.synchronize()
    assert int(bad.item()) == 0

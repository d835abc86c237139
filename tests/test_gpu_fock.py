"""GPU parity of the Fock contraction (FP64 DFMA, FP64 MMA and Ozaki-split BF16 paths) against the
FP64 CPU oracle (numpy @ -> BLAS zgemm, the arithmetic ArrayAnsatz.contract reaches through einsum).

Error metric: max|Y - Y_ref| / max|Y_ref|.  FP64 kernels (DFMA and MMA): 1e-14.  Ozaki split with 7 slices
(balanced 8-bit digits, 55 bits per operand, pairs with slice order <= 8): 1e-13; fewer slices give coarser
results (checked to shrink monotonically)."""

from __future__ import annotations

import numpy as np
import pytest
import torch

import mrmustard_gb300 as mm

pytestmark = pytest.mark.gpu


def rel(x, ref):
    x = x.cpu().numpy() if isinstance(x, torch.Tensor) else np.asarray(x)
    return float(np.abs(x - ref).max() / np.abs(ref).max())


def cn(shape, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


# (40, 300, 64): N spans several 128-column tiles with a ragged last one (one lane of CTAs per column
# tile); (64, 8200, 70): 65 column tiles, too many for lanes (one sequence over every tile); K = 9345
# and 30100 take the int64 slice-order sums (K padded beyond 9344), K = 9344 the int32 ones at their
# bound, as every other case; K = 1025 and 4200 end in a partial 1024-value unit.
@pytest.mark.parametrize("M,N,K", [(1, 1, 1), (37, 5, 300), (300, 64, 200), (129, 33, 4200), (40, 300, 64),
                                   (64, 8200, 70), (70, 41, 1025), (20, 9, 9344), (20, 9, 9345), (24, 12, 30100)])
def test_gemm_random(cuda, oracle_lib, M, N, K):
    U, X = cn((M, K), M + K), cn((K, N), N)
    ref = oracle_lib.fock_gemm(U, X)
    # FP64 sums of K random products (the kernels' and BLAS's, in different orders) drift apart like
    # sqrt(K) unit roundoffs: 1e-14 up to K ~ 500, 2^-52 sqrt(K) beyond
    tol64 = max(1e-14, 2.0 ** -52 * np.sqrt(K))
    assert rel(mm.fock_gemm(U, X, "fp64"), ref) < tol64
    assert rel(mm.fock_gemm(U, X, "dmma"), ref) < tol64
    assert rel(mm.fock_gemm(U, X, "ozaki"), ref) < 1e-13


def test_gemm_wide_dynamic_range(cuda, oracle_lib):
    """Rows and columns spanning many decades (per-row / per-column scaling)."""
    rng = np.random.default_rng(5)
    U = cn((96, 160), 6) * (10.0 ** rng.uniform(-30, 5, (96, 1)))
    X = cn((160, 40), 7) * (10.0 ** rng.uniform(-8, 8, (1, 40)))
    ref = oracle_lib.fock_gemm(U, X)
    Y = mm.fock_gemm(U, X, "ozaki")
    # per-element check against each row/column's own scale
    scale = np.abs(U).max(axis=1, keepdims=True) * np.abs(X).max(axis=0, keepdims=True) * U.shape[1]
    assert (np.abs(Y - ref) / scale).max() < 1e-15
    assert rel(mm.fock_gemm(U, X, "fp64"), ref) < 1e-14
    assert rel(mm.fock_gemm(U, X, "dmma"), ref) < 1e-14


def test_gemm_slices_converge(cuda, oracle_lib):
    U, X = cn((64, 512), 8), cn((512, 32), 9)
    ref = oracle_lib.fock_gemm(U, X)
    errs = [rel(mm.fock_gemm(U, X, "ozaki", slices=s), ref) for s in (2, 3, 5, 7)]
    assert errs[0] > errs[1] > errs[2] >= errs[3]
    assert errs[3] < 1e-13


def test_cfg5_unitary_on_kets(cuda, oracle_lib):
    """Gate tensor from the recurrence (4x4 complex symmetric A, spectral norm 0.95, cutoff 50)
    applied to 256 normalised 2-mode kets, as one 2500 x 2500 by 2500 x 256 contraction."""
    rng = np.random.default_rng(55)
    Xa = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    A = Xa + Xa.T
    A *= 0.95 / np.linalg.norm(A, 2)
    b = 0.3 * (rng.standard_normal(4) + 1j * rng.standard_normal(4)) / np.sqrt(2)
    Ut = mm.device_fwd(torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda),
                       torch.tensor(1.0 + 0j, device=cuda), (50, 50, 50, 50))  # complex64 c: converted
    assert Ut[0, 0, 0, 0].item() == 1.0 and Ut.abs().max().item() >= 1.0
    kets = cn((256, 50, 50), 56)
    kets /= np.linalg.norm(kets.reshape(256, -1), axis=1)[:, None, None]
    kt = torch.as_tensor(kets, device=cuda)
    U = Ut.cpu().numpy()
    ref = np.einsum("abcd,ncd->nab", U, kets)
    for mode, tol in (("fp64", 1e-14), ("dmma", 1e-14), ("ozaki", 1e-13)):
        Y = mm.apply_unitary(Ut, kt, mode=mode)
        assert Y.shape == (256, 50, 50)
        assert rel(Y, ref) < tol, mode


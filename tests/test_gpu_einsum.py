"""GPU parity of the Fock-space einsum (permutation, inner sums, batched FP64 GEMM / GEMV kernels)
against the FP64 CPU oracle (numpy einsum, BLAS underneath), and ArrayAnsatz.contract semantics."""

from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TOL = 1e-13  # relative to max |reference|: FP64 with a different summation order


def _rel(x, ref):
    x, ref = np.asarray(x), np.asarray(ref)
    den = np.abs(ref).max() if ref.size else 0.0
    return float(np.abs(x - ref).max() / den) if den > 0 else float(np.abs(x - ref).max() if x.size else 0.0)


def _rand(rng, *shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


CASES = [
    ("ab,bc->ac", [(37, 23), (23, 41)]),
    ("abcd,cd->ab", [(12, 11, 12, 11), (12, 11)]),             # gate on one 2-mode ket (GEMV)
    ("c,abcd->abd", [(13,), (9, 10, 13, 7)]),                  # row vector times matrix (M = 1)
    ("zab,zbc->zac", [(5, 17, 19), (5, 19, 8)]),               # batch label
    ("zcd,abcd->zab", [(16, 9, 8), (10, 11, 9, 8)]),           # batch of kets through a gate
    ("a,b->ab", [(33,), (40,)]),                               # outer product (K = 1)
    ("ab->ba", [(300, 200)]),                                  # tiled transpose
    ("abcd->dbca", [(20, 7, 9, 33)]),
    ("abc->cab", [(3, 4, 5)]),
    ("aa->a", [(17, 17)]),                                     # diagonal
    ("aa->", [(17, 17)]),                                      # trace
    ("abab->ab", [(6, 5, 6, 5)]),
    ("abc->b", [(7, 9, 11)]),                                  # sums inside one operand
    ("abc,cd->ad", [(6, 7, 8), (8, 9)]),                       # b summed in A only
    ("ab,bc,cd->ad", [(9, 10), (10, 11), (11, 12)]),           # three operands
    ("a,cdab,b->cd", [(15,), (14, 13, 15, 16), (16,)]),        # ket0, BS, ket1 network
    ("ab,bc", [(8, 9), (9, 10)]),                              # implicit output
    ("a,a->", [(50,), (50,)]),                                 # scalar result
    ("ijk,jkl,lm->im", [(6, 7, 8), (7, 8, 9), (9, 10)]),
    ("abc,abc->abc", [(4, 5, 6), (4, 5, 6)]),                  # Hadamard (all batch)
]


@pytest.mark.parametrize("sub,shapes", CASES)
def test_einsum_vs_oracle(cuda, sub, shapes):
    import mrmustard_gb300 as gb

    rng = np.random.default_rng(abs(hash(sub)) % 2**32)
    ops = [_rand(rng, *s) for s in shapes]
    got = gb.einsum(sub, *ops)
    ref = oracle.einsum(sub, *ops)
    assert np.shape(got) == np.shape(ref)
    assert _rel(got, ref) <= TOL, _rel(got, ref)


def test_einsum_gate_on_kets_large(cuda):
    """A 2-mode Gaussian-like gate at cutoff 40 on 64 two-mode kets (GEMM 1600 x 1600 x 64), FP64 and
    the Ozaki tcgen05 path on one ket batch flattened (unbatched product)."""
    import mrmustard_gb300 as gb

    rng = np.random.default_rng(5)
    U = _rand(rng, 40, 40, 40, 40) / 1600
    kets = _rand(rng, 64, 40, 40)
    ref = oracle.einsum("abcd,zcd->zab", U, kets)
    assert _rel(gb.einsum("abcd,zcd->zab", U, kets), ref) <= TOL
    assert _rel(gb.einsum("abcd,zcd->zab", U, kets, mode="ozaki"), ref) <= 1e-12


def test_einsum_zero_sizes(cuda):
    import mrmustard_gb300 as gb

    rng = np.random.default_rng(6)
    A, B = _rand(rng, 4, 0), _rand(rng, 0, 5)
    got = gb.einsum("ab,bc->ac", A, B)  # empty sum
    assert got.shape == (4, 5) and np.all(got == 0)
    assert gb.einsum("ab,bc->ac", _rand(rng, 0, 3), _rand(rng, 3, 5)).shape == (0, 5)


def test_einsum_errors(cuda):
    import mrmustard_gb300 as gb

    with pytest.raises(ValueError):
        gb.einsum("ab,bc->ad", np.ones((2, 2)), np.ones((2, 2)))
    with pytest.raises(ValueError):
        gb.einsum("ab,bc->ac", np.ones((2, 3)), np.ones((2, 2)))
    with pytest.raises(ValueError):
        gb.einsum("ab->ab", np.ones((2, 2)), np.ones((2, 2)))
    with pytest.raises(ValueError):
        gb.einsum("...a->a", np.ones((2, 2)))


def test_contract_semantics(cuda):
    """ArrayAnsatz.contract (array_ansatz.py:159-226): str batch labels and int core labels,
    contracted labels sliced to the smaller dimension, output order from idx_out."""
    import mrmustard_gb300 as gb

    rng = np.random.default_rng(7)
    a1 = _rand(rng, 3, 10, 12)   # ['b', 0, 1]
    a2 = _rand(rng, 3, 9, 7)     # ['b', 1, 2]: label 1 has dims 12 and 9 -> sliced to 9
    got = gb.contract(a1, ["b", 0, 1], a2, ["b", 1, 2], ["b", 2, 0])
    ref = np.einsum("bxy,byz->bzx", a1[:, :, :9], a2)
    assert got.shape == (3, 7, 10) and _rel(got, ref) <= TOL
    with pytest.raises(ValueError, match="expected len"):
        gb.contract(a1, ["b", 0], a2, ["b", 1, 2], ["b"])
    with pytest.raises(ValueError, match="Output labels"):
        gb.contract(a1, ["b", 0, 1], a2, ["b", 1, 2], [5])


def test_mm_einsum_network_example(cuda):
    """The mm_einsum docstring network (physics/mm_einsum.py:85-98) in Fock space: ket0 [0], ket1 [1],
    BS [2, 3, 0, 1] -> [2, 3], contracted pair by pair as ArrayAnsatz.contract does."""
    import mrmustard_gb300 as gb

    rng = np.random.default_rng(8)
    k0, k1 = _rand(rng, 20), _rand(rng, 20)
    bs = _rand(rng, 10, 10, 20, 20)
    r1 = gb.contract(k0, [0], bs, [2, 3, 0, 1], [2, 3, 1])
    r2 = gb.contract(r1, [2, 3, 1], k1, [1], [2, 3])
    ref = np.einsum("a,cdab,b->cd", k0, bs, k1)
    assert r2.shape == (10, 10) and _rel(r2, ref) <= TOL


def test_einsum_device_in_device_out(cuda):
    import torch

    import mrmustard_gb300 as gb

    rng = np.random.default_rng(9)
    A, B = _rand(rng, 30, 20), _rand(rng, 20, 10)
    n0 = gb.launch_count()
    got = gb.einsum("ab,bc->ca", torch.tensor(A, device=cuda), torch.tensor(B, device=cuda))
    assert isinstance(got, torch.Tensor) and got.is_cuda
    assert gb.launch_count() > n0
    assert _rel(got.cpu().numpy(), (A @ B).T) <= TOL

"""GPU parity of the diagonal strategies (compactFock diagonal amplitudes and Jacobians,
fast_diagonal) against fixtures made from the reference source and against the C oracle."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from conftest import diagonal_cases

pytestmark = pytest.mark.gpu

TOL = 1e-13       # relative to max |reference|; FMA and summation order differ from the reference's BLAS dots
TOL_JAC = 1e-12


def _rel(x, ref):
    x, ref = np.asarray(x), np.asarray(ref)
    den = np.abs(ref).max()
    return float(np.abs(x - ref).max() / den) if den > 0 else float(np.abs(x - ref).max())


def _dm_triple(M, seed, r_max=0.6, t_max=0.3, beta=0.4):
    from scipy.stats import unitary_group

    rng = np.random.default_rng(seed)
    U = unitary_group.rvs(M, random_state=rng) if M > 1 else np.exp(1j * rng.uniform(0, 6, (1, 1)))
    V = unitary_group.rvs(M, random_state=rng) if M > 1 else np.ones((1, 1))
    K = (U * np.tanh(rng.uniform(0.05, r_max, M))) @ U.T
    Cm = (V * rng.uniform(0.0, t_max, M)) @ V.conj().T
    A = np.block([[K.conj(), Cm.T], [Cm, K]])
    bk = beta * (rng.standard_normal(M) + 1j * rng.standard_normal(M))
    b = np.concatenate([bk.conj(), bk])
    return np.conj(-A), np.conj(b), np.complex128(0.7)


def _interleave(A, b):
    o = np.arange(A.shape[0]).reshape(2, -1).T.flatten()
    return A[o][:, o], b[o]


def test_diagonal_amps_golden(cuda, diagonal_golden):
    """hermite_multidimensional_diagonal on the device: all five arrays of the reference source,
    with and without a batch axis on B, and the same elements written (zero pattern)."""
    import mrmustard_gb300 as gb

    g = diagonal_golden
    for n in diagonal_cases(g, "amps"):
        got = gb.hermite_multidimensional_diagonal(g[f"{n}/A"], g[f"{n}/B"], g[f"{n}/G0"], tuple(g[f"{n}/cutoffs"]))
        for name, x in zip(("arr0", "arr2", "arr1010", "arr1001", "arr1"), got):
            ref = g[f"{n}/{name}"]
            assert x.shape == ref.shape, (n, name)
            assert np.array_equal(x == 0, ref == 0), (n, name)
            assert _rel(x, ref) <= TOL, (n, name, _rel(x, ref))


def test_diagonal_grad_golden(cuda, diagonal_golden):
    """grad_hermite_multidimensional_diagonal on the device against the reference source's Jacobians."""
    import mrmustard_gb300 as gb

    g = diagonal_golden
    for n in diagonal_cases(g, "grad"):
        A, B, G0, cut = g[f"{n}/A"], g[f"{n}/B"], g[f"{n}/G0"], tuple(g[f"{n}/cutoffs"])
        arrs = gb.hermite_multidimensional_diagonal(A, B, G0, cut)
        got = gb.grad_hermite_multidimensional_diagonal(A, B, G0, *arrs)
        for name, x in zip(("dG0", "dA", "dB"), got):
            ref = g[f"{n}/{name}"]
            assert x.shape == ref.shape, (n, name)
            assert _rel(x, ref) <= TOL_JAC, (n, name, _rel(x, ref))


def test_fast_diagonal_golden(cuda, diagonal_golden):
    """fast_diagonal (vanilla and stable first block) against the reference source, including an
    output cutoff of 0, where the reference's weight loop stops early and leaves zeros."""
    import mrmustard_gb300 as gb

    g = diagonal_golden
    for n in diagonal_cases(g, "fd"):
        got = gb.fast_diagonal(g[f"{n}/A"], g[f"{n}/b"], g[f"{n}/c"], int(g[f"{n}/oc"]), tuple(g[f"{n}/pnr"]),
                               bool(g[f"{n}/stable"]))
        ref = g[f"{n}/out"]
        assert got.shape == ref.shape, n
        assert np.array_equal(got == 0, ref == 0), n
        assert _rel(got, ref) <= TOL, (n, _rel(got, ref))


@pytest.mark.parametrize("M,cut,nb", [(4, (8, 8, 8, 8), 1), (3, (14, 12, 10), 1), (2, (40, 30), 1), (5, (4, 5, 4, 3, 4), 1),
                                      (3, (8, 8, 8), 16), (1, (200,), 1), (6, (3, 3, 3, 3, 3, 3), 1)])
def test_diagonal_amps_vs_oracle(cuda, M, cut, nb):
    """Larger lattices than the fixtures (multi-CTA wavefronts), against the C oracle."""
    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(M, 40 + M + nb)
    Ai, bi = _interleave(A, b)
    B = bi if nb == 1 else bi[:, None] * np.linspace(0.5, 1.5, nb)[None, :]
    got = gb.hermite_multidimensional_diagonal(Ai, B, c, cut)
    ref = oracle.diagonal_amps(Ai, B, c, cut)
    for name, x, r in zip(("arr0", "arr2", "arr1010", "arr1001", "arr1"), got, ref):
        assert np.array_equal(x == 0, r == 0), name
        assert _rel(x, r) <= TOL, (name, _rel(x, r))


@pytest.mark.parametrize("M,cut", [(3, (6, 5, 4)), (2, (12, 10)), (4, (3, 4, 3, 3))])
def test_diagonal_jacobian_vs_oracle(cuda, M, cut):
    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(M, 70 + M)
    Ai, bi = _interleave(A, b)
    arrs = gb.hermite_multidimensional_diagonal(Ai, bi, c, cut)
    got = gb.grad_hermite_multidimensional_diagonal(Ai, bi, c, *arrs)
    ref = oracle.diagonal_grad(Ai, bi, c, cut)
    for x, r in zip(got, ref):
        assert _rel(x, r) <= TOL_JAC


@pytest.mark.parametrize("L,oc,pnr,stable", [(3, 10, (8, 8), False), (3, 6, (10, 6), True), (4, 5, (4, 4, 4), False),
                                             (2, 30, (25,), False), (5, 3, (2, 3, 2, 2), True), (2, 0, (6,), False)])
def test_fast_diagonal_vs_oracle(cuda, L, oc, pnr, stable):
    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(L, 90 + L + oc)
    got = gb.fast_diagonal(A, b, c, oc, pnr, stable)
    ref = oracle.fast_diagonal(A, b, c, oc, pnr, stable)
    assert np.array_equal(got == 0, ref == 0)
    assert _rel(got, ref) <= TOL, _rel(got, ref)


def test_facade_diagonal_equals_vanilla(cuda):
    """tests/test_math/test_compactFock.py:19-43: the backend method (A, B in Bargmann order,
    reorderedAB=True) gives G[k, k] of the vanilla tensor with shape cutoffs * 2."""
    import mrmustard_gb300 as gb

    cut = (5, 5, 5)
    A, b, c = _dm_triple(3, 5)
    G = gb.vanilla_numba(cut * 2, A, b, c)
    ref = np.zeros(cut, np.complex128)
    for idx in np.ndindex(*cut):
        ref[idx] = G[idx + idx]
    got = gb.BackendGB300().hermite_renormalized_diagonal(A, b, c, cut)
    assert np.allclose(got, ref, rtol=1e-10, atol=1e-14)


def test_facade_1leftover_equals_vanilla(cuda):
    """tests/test_math/test_fast_diagonal.py:24-31 and test_compactFock.py:46-69: the backend method's
    (oc+1, oc+1, pnr+1 ...) blocks equal the vanilla tensor's entries."""
    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(2, 6)
    fd = gb.hermite_renormalized_1leftoverMode(A, b, c, 5, (10,))
    control = gb.vanilla_numba((6, 11, 6, 11), A, b, c)
    control = control[:, np.arange(11), :, np.arange(11)]
    assert np.allclose(fd, np.transpose(control, (1, 2, 0)))
    A, b, c = _dm_triple(3, 7)
    fd = gb.BackendGB300().hermite_renormalized_1leftoverMode(A, b, c, 3, (1, 2), True)
    G = gb.vanilla_numba((4, 2, 3, 4, 2, 3), A, b, c)
    expected = np.diagonal(np.diagonal(G, axis1=1, axis2=4), axis1=1, axis2=3)
    assert np.allclose(expected, fd)


def test_diagonal_autograd_matches_jacobian_contraction(cuda):
    """DiagonalFn.backward = conj(sum_k conj(g_k) J_k) for PyTorch's convention, J the reference's
    Jacobians (the contraction of hermite_renormalized_diagonal_jax_bwd, jax_vjps/hermite.py:292-329)."""
    import torch

    import mrmustard_gb300 as gb

    cut = (5, 4, 3)
    A, b, c = _dm_triple(3, 8)
    At = torch.tensor(A, device=cuda, requires_grad=True)
    bt = torch.tensor(b, device=cuda, requires_grad=True)
    ct = torch.tensor(c, device=cuda, requires_grad=True)
    rng = np.random.default_rng(3)
    w = rng.standard_normal(cut) + 1j * rng.standard_normal(cut)
    out = gb.hermite_renormalized_diagonal_autograd(At, bt, ct, cut)
    loss = torch.real(torch.sum(torch.tensor(w, device=cuda) * out))
    loss.backward()
    Ai, bi = _interleave(A, b)
    dG0, dA, dB = oracle.diagonal_grad(Ai, bi, c, cut)
    g = np.conj(w)  # dL/dRe(out) + i dL/dIm(out) = conj(w)
    exp_A = np.conj(np.einsum("k,kpq->pq", np.conj(g).reshape(-1), dA.reshape(-1, 6, 6)))
    exp_B = np.conj(np.einsum("k,kp->p", np.conj(g).reshape(-1), dB.reshape(-1, 6)))
    exp_c = np.conj(np.sum(np.conj(g) * dG0))
    o = np.arange(6).reshape(2, -1).T.flatten()
    inv = np.argsort(o)  # gradient w.r.t. the Bargmann-order A, B: undo the interleaving
    assert _rel(At.grad.cpu().numpy(), exp_A[inv][:, inv]) <= 1e-12
    assert _rel(bt.grad.cpu().numpy(), exp_B[inv]) <= 1e-12
    assert abs(ct.grad.item() - exp_c) <= 1e-12 * abs(exp_c)


def test_diagonal_validation_errors(cuda):
    """input_validation and the shape checks of compactFock/inputValidation.py:25-100."""
    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(2, 9)
    Ai, bi = _interleave(A, b)
    with pytest.raises(ValueError, match="symmetric"):
        gb.hermite_multidimensional_diagonal(Ai + np.triu(np.ones((4, 4)), 1), bi, c, (3, 3))
    with pytest.raises(ValueError, match="square"):
        gb.hermite_multidimensional_diagonal(Ai[:3], bi, c, (3, 3))
    with pytest.raises(ValueError, match="incompatible"):
        gb.hermite_multidimensional_diagonal(Ai, bi[:3], c, (3, 3))
    with pytest.raises(ValueError, match="cutoffs"):
        gb.hermite_multidimensional_diagonal(Ai, bi, c, (3, 3, 3))
    with pytest.raises(ValueError, match="unbactched"):
        gb.hermite_multidimensional_diagonal(Ai, bi[:, None, None], c, (3, 3))
    with pytest.raises(TypeError):
        gb.hermite_multidimensional_diagonal(Ai.tolist(), bi, c, (3, 3))


def test_diagonal_device_in_device_out(cuda):
    import torch

    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(2, 10)
    Ai, bi = _interleave(A, b)
    n0 = gb.launch_count()
    got = gb.hermite_multidimensional_diagonal(torch.tensor(Ai, device=cuda), torch.tensor(bi, device=cuda),
                                               torch.tensor(c, device=cuda), (6, 6))
    assert all(isinstance(x, torch.Tensor) and x.is_cuda for x in got)
    assert gb.launch_count() > n0
    fd = gb.fast_diagonal(torch.tensor(A, device=cuda), torch.tensor(b, device=cuda), torch.tensor(c, device=cuda), 4, (5,))
    assert fd.is_cuda and fd.shape == (6, 5, 5)
    ref = oracle.fast_diagonal(A, b, c, 4, (5,))
    assert _rel(fd.cpu().numpy(), ref) <= TOL


# ----------------------------------------------------------------- leftover mode (compactFock)
def test_leftover_golden(cuda, diagonal_golden):
    """hermite_multidimensional_1leftoverMode and its gradient on the device against the reference
    source: the five block arrays (zero patterns equal) and (dG0, dA, dB)."""
    import mrmustard_gb300 as gb

    g = diagonal_golden
    for n in diagonal_cases(g, "lo"):
        A, B, G0, cut = g[f"{n}/A"], g[f"{n}/B"], g[f"{n}/G0"], tuple(g[f"{n}/cutoffs"])
        arrs = gb.hermite_multidimensional_1leftoverMode(A, B, G0, cut)
        for name, x in zip(("arr0", "arr2", "arr1010", "arr1001", "arr1"), arrs):
            ref = g[f"{n}/{name}"]
            assert x.shape == ref.shape, (n, name)
            assert np.array_equal(x == 0, ref == 0), (n, name)
            assert _rel(x, ref) <= TOL, (n, name, _rel(x, ref))
        for name, x in zip(("dG0", "dA", "dB"), gb.grad_hermite_multidimensional_1leftoverMode(A, B, G0, *arrs)):
            ref = g[f"{n}/{name}"]
            assert x.shape == ref.shape, (n, name)
            assert _rel(x, ref) <= TOL_JAC, (n, name, _rel(x, ref))


@pytest.mark.parametrize("M,cut", [(2, (20, 15)), (3, (10, 6, 6)), (4, (6, 4, 4, 4)), (5, (4, 3, 3, 3, 3))])
def test_leftover_vs_oracle(cuda, M, cut):
    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(M, 120 + M)
    Ai, bi = _interleave(A, b)
    got = gb.hermite_multidimensional_1leftoverMode(Ai, bi, c, cut)
    ref = oracle.leftover_amps(Ai, bi, c, cut)
    for name, x, r in zip(("arr0", "arr2", "arr1010", "arr1001", "arr1"), got, ref):
        assert np.array_equal(x == 0, r == 0), name
        assert _rel(x, r) <= TOL, (name, _rel(x, r))


@pytest.mark.parametrize("M,cut", [(2, (6, 5)), (3, (4, 3, 3))])
def test_leftover_jacobian_vs_oracle(cuda, M, cut):
    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(M, 140 + M)
    Ai, bi = _interleave(A, b)
    arrs = gb.hermite_multidimensional_1leftoverMode(Ai, bi, c, cut)
    got = gb.grad_hermite_multidimensional_1leftoverMode(Ai, bi, c, *arrs)
    for x, r in zip(got, oracle.leftover_grad(Ai, bi, c, cut)):
        assert _rel(x, r) <= TOL_JAC


def test_leftover_jax_path_equals_vanilla(cuda):
    """tests/test_math/test_compactFock.py:46-69 under the JAX backend's path: output cutoff 3, PNR
    cutoffs (1, 2) on a Bargmann-order triple equal the vanilla tensor's diagonal blocks."""
    import torch

    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(3, 11)
    got = gb.hermite_renormalized_1leftoverMode_autograd(torch.tensor(A, device=cuda), torch.tensor(b, device=cuda),
                                                         torch.tensor(c, device=cuda), 3, (1, 2))
    G = gb.vanilla_numba((4, 2, 3, 4, 2, 3), A, b, c)
    expected = np.diagonal(np.diagonal(G, axis1=1, axis2=4), axis1=1, axis2=3)
    assert got.shape == (4, 4, 2, 3)
    assert np.allclose(expected, got.detach().cpu().numpy())


def test_leftover_autograd_matches_jacobian_contraction(cuda):
    import torch

    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(3, 12)
    At = torch.tensor(A, device=cuda, requires_grad=True)
    bt = torch.tensor(b, device=cuda, requires_grad=True)
    ct = torch.tensor(c, device=cuda, requires_grad=True)
    out = gb.hermite_renormalized_1leftoverMode_autograd(At, bt, ct, 3, (2, 1))
    rng = np.random.default_rng(4)
    w = rng.standard_normal(out.shape) + 1j * rng.standard_normal(out.shape)
    torch.real(torch.sum(torch.tensor(w, device=cuda) * out)).backward()
    Ai, bi = _interleave(A, b)
    dG0, dA, dB = oracle.leftover_grad(Ai, bi, c, (4, 3, 2))
    exp_A = np.einsum("k,kpq->pq", w.reshape(-1), dA.reshape(-1, 6, 6)).conj()
    exp_B = np.einsum("k,kp->p", w.reshape(-1), dB.reshape(-1, 6)).conj()
    exp_c = np.sum(w * dG0).conj()
    inv = np.argsort(np.arange(6).reshape(2, -1).T.flatten())
    assert _rel(At.grad.cpu().numpy(), exp_A[inv][:, inv]) <= 1e-12
    assert _rel(bt.grad.cpu().numpy(), exp_B[inv]) <= 1e-12
    assert abs(ct.grad.item() - exp_c) <= 1e-12 * abs(exp_c)


def test_leftover_validation(cuda):
    import mrmustard_gb300 as gb

    A, b, c = _dm_triple(1, 13)
    with pytest.raises(ValueError, match="greater than 1"):
        gb.hermite_multidimensional_1leftoverMode(A, b, c, (3,))
    A, b, c = _dm_triple(2, 13)
    with pytest.raises(ValueError, match="incompatible"):
        gb.hermite_multidimensional_1leftoverMode(A, b[:3], c, (3, 3))

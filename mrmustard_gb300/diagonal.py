"""Diagonal strategies on the GPU: PNR amplitudes, their gradients, leftover-mode density matrices.

Mirrors, with the same arguments, return values and errors:

* ``hermite_multidimensional_diagonal(A, B, G0, cutoffs)`` -> (arr0, arr2, arr1010, arr1001, arr1)
  (mrmustard/math/lattice/strategies/compactFock/inputValidation.py:61-79, diagonal_amps.py:217-248);
* ``grad_hermite_multidimensional_diagonal(A, B, G0, arr0, arr2, arr1010, arr1001, arr1)`` ->
  (arr0_dG0, arr0_dA, arr0_dB) (inputValidation.py:82-100, diagonal_grad.py:261-378);
* ``fast_diagonal(A, b, c, output_cutoff, pnr_cutoffs, stable)``
  (mrmustard/math/lattice/strategies/fast_diagonal.py:32-77);
* ``hermite_multidimensional_1leftoverMode`` / ``grad_hermite_multidimensional_1leftoverMode``
  (compactFock/inputValidation.py:103-142, singleLeftoverMode_amps.py, singleLeftoverMode_grad.py),
  the JAX backend's leftover-mode path, with ``hermite_renormalized_1leftoverMode_autograd``
  (``hermite_renormalized_1leftoverMode_jax``, jax_vjps/hermite.py:339-430);
* the backend methods ``hermite_renormalized_diagonal(A, B, C, cutoffs, reorderedAB)`` and
  ``hermite_renormalized_1leftoverMode(A, b, c, output_cutoff, pnr_cutoffs, stable, reorderedAB)``
  (mrmustard/math/backend_numpy.py:423-446), and a differentiable
  ``hermite_renormalized_diagonal_autograd`` (the counterpart of
  ``hermite_renormalized_diagonal_jax``, mrmustard/math/jax_vjps/hermite.py:248-335).

numpy in -> numpy out; CUDA tensors in -> CUDA tensors out.
"""

from __future__ import annotations

from collections.abc import Iterable

import numpy as np
import torch

from . import _lib
from .hermite import Workspace, _finish, _shape_arr, _stream, _to_dev, device_fwd, raw, require_cuda

__all__ = [
    "hermite_multidimensional_diagonal",
    "grad_hermite_multidimensional_diagonal",
    "hermite_renormalized_diagonal",
    "hermite_renormalized_diagonal_autograd",
    "fast_diagonal",
    "hermite_renormalized_1leftoverMode",
    "reorder_AB_bargmann",
    "device_diagonal_slots",
    "hermite_multidimensional_1leftoverMode",
    "grad_hermite_multidimensional_1leftoverMode",
    "hermite_renormalized_1leftoverMode_autograd",
]


def _is_dev(x) -> bool:
    return isinstance(x, torch.Tensor) and x.is_cuda


def _out(t: torch.Tensor, dev_mode: bool):
    return t if dev_mode else t.cpu().numpy()


def reorder_AB_bargmann(A, B):
    """(mode0 .. mode_{M-1}, mode0' ..) -> (mode0, mode0', mode1, ...) (backend_numpy.py:367-375)."""
    n = A.shape[0]
    o = np.arange(n).reshape(2, -1).T.flatten()
    if isinstance(A, torch.Tensor):
        oi = torch.as_tensor(o, device=A.device)
        return A[oi][:, oi], B[torch.as_tensor(o, device=B.device)]
    A, B = np.asarray(A), np.asarray(B)
    return A[o][:, o], B[o]


# ----------------------------------------------------------------- compactFock diagonal
def _split_slots(W: torch.Tensor, M: int, cut: tuple, nb_shape: tuple):
    P = int(np.prod(cut))
    nb = int(np.prod(nb_shape)) if nb_shape else 1
    W = W.reshape(-1, P * nb)
    m1 = M - 1
    arr0 = W[0].reshape(cut + nb_shape)
    arr2 = W[1:1 + M].reshape((M,) + cut + nb_shape)
    o = 1 + M
    if M == 1:
        z = torch.zeros((1, 1, 1) + nb_shape, dtype=W.dtype, device=W.device)
        arr1010, arr1001 = z, z.clone()
    else:
        arr1010 = W[o:o + M * m1].reshape((M, m1) + cut + nb_shape)
        arr1001 = W[o + M * m1:o + 2 * M * m1].reshape((M, m1) + cut + nb_shape)
    o += 2 * M * m1
    arr1 = W[o:o + 2 * M].reshape((2 * M,) + cut + nb_shape)
    return arr0, arr2, arr1010, arr1001, arr1


def _join_slots(M, cut, arr0, arr2, arr1010, arr1001, arr1, dev) -> torch.Tensor:
    parts = [arr0, arr2] + ([arr1010, arr1001] if M > 1 else []) + [arr1]
    return torch.cat([_to_dev(p, dev).reshape(-1) for p in parts]).contiguous()


def device_diagonal_slots(A, B, G0, cutoffs):
    """Device forward: returns the slot buffer (arr0, arr2, arr1010, arr1001, arr1 back to back) for
    A (2M, 2M), B (2M,) or (2M, nb) already in the interleaved order, and G0 (broadcast over nb)."""
    dev = A.device if _is_dev(A) else require_cuda()
    cut, sh = _shape_arr(cutoffs)
    M = len(cut)
    Ad, Bd = _to_dev(A, dev).contiguous(), _to_dev(B, dev)
    nb_shape = tuple(Bd.shape[1:])
    nb = int(np.prod(nb_shape)) if nb_shape else 1
    Bd = Bd.reshape(2 * M, nb).contiguous()
    g0 = _to_dev(G0, dev).reshape(-1)
    g0 = (g0.expand(nb) if g0.numel() == 1 else g0.reshape(nb)).contiguous()
    lib = _lib.load()
    W = torch.empty(int(lib.mm_diagonal_slots(M)) * int(np.prod(cut)) * nb, dtype=torch.complex128, device=dev)
    ws = Workspace(lib.mm_diagonal_workspace_bytes(M, sh, nb), dev)
    _lib.check(lib.mm_diagonal_amps(M, sh, nb, Ad.data_ptr(), Bd.data_ptr(), g0.data_ptr(), W.data_ptr(), ws.ptr,
                                    ws.nbytes, _stream()), "mm_diagonal_amps")
    _finish(ws, "diagonal")
    return W, nb_shape


def _input_validation(A, rtol=1e-05, atol=1e-08):
    """input_validation (compactFock/inputValidation.py:25-58)."""
    if not isinstance(A, (np.ndarray, torch.Tensor)):
        raise TypeError("Input matrix must be a NumPy array.")
    n = A.shape
    if n[0] != n[1]:
        raise ValueError("Input matrix must be square.")
    An = A.detach().cpu().numpy() if isinstance(A, torch.Tensor) else A
    if np.isnan(An).any():
        raise ValueError("Input matrix must not contain NaNs.")
    if not np.allclose(An, An.T, rtol=rtol, atol=atol):
        raise ValueError("Input matrix must be symmetric.")
    return True


def hermite_multidimensional_diagonal(A, B, G0, cutoffs, rtol=1e-05, atol=1e-08):
    """The five arrays of the diagonal strategy (A, B in the interleaved order)."""
    _input_validation(A, atol=atol, rtol=rtol)
    if B.ndim > 2:
        raise ValueError("B should be either unbactched or two dimensional (vector and batch dimension)")
    if A.shape[0] != B.shape[0]:
        raise ValueError("The matrix A and vector B have incompatible dimensions")
    if isinstance(cutoffs, Iterable):
        cutoffs = tuple(int(c) for c in cutoffs)
    else:
        raise ValueError("cutoffs should be array like of length M")
    M = len(cutoffs)
    if A.shape[0] // 2 != M:
        raise ValueError("The matrix A and cutoffs have incompatible dimensions")
    dev_mode = _is_dev(A)
    W, nb_shape = device_diagonal_slots(A, B, G0, cutoffs)
    return tuple(_out(x, dev_mode) for x in _split_slots(W, M, cutoffs, nb_shape))


def _jacobian(A, B, W, cut, dev):
    M = len(cut)
    n = 2 * M
    _, sh = _shape_arr(cut)
    lib = _lib.load()
    Ad, Bd = _to_dev(A, dev).contiguous(), _to_dev(B, dev).reshape(-1).contiguous()
    J = torch.empty(W.numel() * (n * n + n), dtype=torch.complex128, device=dev)
    ws = Workspace(lib.mm_diagonal_workspace_bytes(M, sh, 1), dev)
    _lib.check(lib.mm_diagonal_jacobian(M, sh, Ad.data_ptr(), Bd.data_ptr(), W.data_ptr(), J.data_ptr(), ws.ptr,
                                        ws.nbytes, _stream()), "mm_diagonal_jacobian")
    _finish(ws, "diagonal jacobian")
    return J


def grad_hermite_multidimensional_diagonal(A, B, G0, arr0, arr2, arr1010, arr1001, arr1):
    """(arr0_dG0, arr0_dA, arr0_dB) from the forward arrays (B unbatched)."""
    if A.shape[0] != B.shape[0]:
        raise ValueError("The matrix A and vector B have incompatible dimensions")
    M = A.shape[0] // 2
    dev_mode = _is_dev(A)
    dev = A.device if dev_mode else require_cuda()
    cut = tuple(int(x) for x in arr0.shape)
    W = _join_slots(M, cut, arr0, arr2, arr1010, arr1001, arr1, dev)
    J = _jacobian(A, B, W, cut, dev)
    n = 2 * M
    P = int(np.prod(cut))
    J0 = J[:P * (n * n + n)].reshape(P, n * n + n)
    g0 = _to_dev(G0, dev).reshape(-1)[0]
    dG0 = (W[:P] / g0).reshape(cut)
    return (_out(dG0, dev_mode), _out(J0[:, :n * n].reshape(cut + (n, n)), dev_mode),
            _out(J0[:, n * n:].reshape(cut + (n,)), dev_mode))


def hermite_renormalized_diagonal(A, B, C, cutoffs, reorderedAB: bool = True):
    """``BackendNumpy.hermite_renormalized_diagonal`` (backend_numpy.py:423-432): arr0 of the triple."""
    A, B = reorder_AB_bargmann(A, B) if reorderedAB else (A, B)
    return hermite_multidimensional_diagonal(A, B, C, cutoffs)[0]


class DiagonalFn(torch.autograd.Function):
    """arr0(A, B, C) with the reference's custom VJP (jax_vjps/hermite.py:284-329): the Jacobians of
    diagonal_grad.py contracted with the cotangent, on the device.  PyTorch's convention for a
    holomorphic map: grad_in = conj(vjp(conj(grad_out)))."""

    @staticmethod
    def forward(ctx, A, B, C, cutoffs):
        cut = tuple(cutoffs)
        W, _ = device_diagonal_slots(A.detach(), B.detach(), C.detach(), cut)
        Ad = raw(A.detach().to(torch.complex128)).contiguous()
        Bd = raw(B.detach().to(torch.complex128)).contiguous()
        cd = raw(C.detach().to(torch.complex128)).reshape(1).contiguous()
        ctx.save_for_backward(Ad, Bd, cd, W)
        ctx.cut = cut
        ctx.c_shape = C.shape
        P = int(np.prod(cut))
        return W[:P].reshape(cut).clone()

    @staticmethod
    def backward(ctx, grad):
        A, B, C, W = ctx.saved_tensors
        cut = ctx.cut
        M = len(cut)
        n = 2 * M
        J = _jacobian(A, B, W, cut, A.device)
        g = grad.conj().resolve_conj().to(torch.complex128).reshape(-1).contiguous()
        dA = torch.empty((n, n), dtype=torch.complex128, device=A.device)
        dB = torch.empty((n,), dtype=torch.complex128, device=A.device)
        dC = torch.empty((1,), dtype=torch.complex128, device=A.device)
        _, sh = _shape_arr(cut)
        _lib.check(_lib.load().mm_diagonal_vjp(M, sh, J.data_ptr(), W.data_ptr(), C.data_ptr(), g.data_ptr(),
                                               dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), _stream()),
                   "mm_diagonal_vjp")
        return dA.conj(), dB.conj(), dC.conj().reshape(ctx.c_shape), None


def hermite_renormalized_diagonal_autograd(A, B, C, cutoffs, reorderedAB: bool = True):
    """Differentiable arr0 for CUDA tensors (unbatched B), like ``math.hermite_renormalized_diagonal``
    under the JAX backend (backend_jax.py:513-522)."""
    A, B = reorder_AB_bargmann(A, B) if reorderedAB else (A, B)
    return DiagonalFn.apply(A, B, C, tuple(int(c) for c in cutoffs))


# ----------------------------------------------------------------- leftover mode (compactFock)
def _lo_split(W: torch.Tensor, M: int, cut: tuple):
    """Slot buffer [slot][m][n][P'] -> the reference's arrays with the block axes first
    (singleLeftoverMode_amps.py:385-408); views, no copies."""
    q, tail = cut[0], tuple(cut[1:])
    Mt = M - 1
    W = W.reshape((-1, q, q) + tail)
    mv = lambda x: x.movedim(0, 2)
    arr0 = W[0]
    arr2 = mv(W[1:1 + Mt])
    o = 1 + Mt
    if Mt == 1:
        z = torch.zeros((1, 1, 1, 1, 1), dtype=W.dtype, device=W.device)
        arr1010, arr1001 = z, z.clone()
    else:
        k = Mt * (Mt - 1)
        arr1010 = mv(W[o:o + k]).reshape((q, q, Mt, Mt - 1) + tail)
        arr1001 = mv(W[o + k:o + 2 * k]).reshape((q, q, Mt, Mt - 1) + tail)
    o += 2 * Mt * (Mt - 1)
    arr1 = mv(W[o:o + 2 * Mt])
    return arr0, arr2, arr1010, arr1001, arr1


def _lo_join(M, cut, arr0, arr2, arr1010, arr1001, arr1, dev) -> torch.Tensor:
    q, tail = cut[0], tuple(cut[1:])
    Mt = M - 1
    parts = [_to_dev(arr0, dev).reshape((1, q, q) + tail), _to_dev(arr2, dev).movedim(2, 0)]
    if Mt > 1:
        k = Mt * (Mt - 1)
        parts += [_to_dev(arr1010, dev).reshape((q, q, k) + tail).movedim(2, 0),
                  _to_dev(arr1001, dev).reshape((q, q, k) + tail).movedim(2, 0)]
    parts.append(_to_dev(arr1, dev).movedim(2, 0))
    return torch.cat([p.contiguous().reshape(-1) for p in parts]).contiguous()


def device_leftover_slots(A, B, G0, cutoffs):
    """Device forward of the leftover strategy: the slot buffer (A, B interleaved; cutoffs[0] the
    leftover mode's cutoff)."""
    dev = A.device if _is_dev(A) else require_cuda()
    cut, sh = _shape_arr(cutoffs)
    M = len(cut)
    Ad, Bd = _to_dev(A, dev).contiguous(), _to_dev(B, dev).reshape(-1).contiguous()
    g0 = _to_dev(G0, dev).reshape(-1)[:1].contiguous()
    lib = _lib.load()
    W = torch.empty(int(lib.mm_leftover_slots(M)) * cut[0] ** 2 * int(np.prod(cut[1:])), dtype=torch.complex128,
                    device=dev)
    ws = Workspace(lib.mm_leftover_workspace_bytes(M, sh), dev)
    _lib.check(lib.mm_leftover_amps(M, sh, Ad.data_ptr(), Bd.data_ptr(), g0.data_ptr(), W.data_ptr(), ws.ptr,
                                    ws.nbytes, _stream()), "mm_leftover_amps")
    _finish(ws, "leftover")
    return W


def hermite_multidimensional_1leftoverMode(A, B, G0, cutoffs, rtol=1e-05, atol=1e-08):
    """The five arrays of the leftover-mode strategy (inputValidation.py:103-119); A, B interleaved."""
    _input_validation(A, atol=atol, rtol=rtol)
    if A.shape[0] != B.shape[0]:
        raise ValueError("The matrix A and vector B have incompatible dimensions")
    if isinstance(cutoffs, Iterable):
        cutoffs = tuple(int(c) for c in cutoffs)
    else:
        raise ValueError("cutoffs should be array like of length M")
    M = len(cutoffs)
    if A.shape[0] // 2 != M:
        raise ValueError("The matrix A and cutoffs have incompatible dimensions")
    if M <= 1:
        raise ValueError("The number of modes should be greater than 1.")
    dev_mode = _is_dev(A)
    W = device_leftover_slots(A, B, G0, cutoffs)
    return tuple(_out(x, dev_mode) for x in _lo_split(W, M, cutoffs))


def _lo_jacobian(A, B, W, cut, dev):
    M = len(cut)
    n = 2 * M
    _, sh = _shape_arr(cut)
    lib = _lib.load()
    Ad, Bd = _to_dev(A, dev).contiguous(), _to_dev(B, dev).reshape(-1).contiguous()
    J = torch.empty(W.numel() * (n * n + n), dtype=torch.complex128, device=dev)
    ws = Workspace(lib.mm_leftover_workspace_bytes(M, sh), dev)
    _lib.check(lib.mm_leftover_jacobian(M, sh, Ad.data_ptr(), Bd.data_ptr(), W.data_ptr(), J.data_ptr(), ws.ptr,
                                        ws.nbytes, _stream()), "mm_leftover_jacobian")
    _finish(ws, "leftover jacobian")
    return J


def grad_hermite_multidimensional_1leftoverMode(A, B, G0, arr0, arr2, arr1010, arr1001, arr1):
    """(arr0_dG0, arr0_dA, arr0_dB) of the leftover strategy (inputValidation.py:122-142)."""
    if A.shape[0] != B.shape[0]:
        raise ValueError("The matrix A and vector B have incompatible dimensions")
    M = A.shape[0] // 2
    if M <= 1:
        raise ValueError("The number of modes should be greater than 1.")
    dev_mode = _is_dev(A)
    dev = A.device if dev_mode else require_cuda()
    cut = (int(arr0.shape[0]),) + tuple(int(x) for x in arr0.shape[2:])
    W = _lo_join(M, cut, arr0, arr2, arr1010, arr1001, arr1, dev)
    J = _lo_jacobian(A, B, W, cut, dev)
    n = 2 * M
    E = int(np.prod(arr0.shape))
    J0 = J[:E * (n * n + n)].reshape(tuple(arr0.shape) + (n * n + n,))
    g0 = _to_dev(G0, dev).reshape(-1)[0]
    dG0 = (W[:E] / g0).reshape(tuple(arr0.shape))
    return (_out(dG0, dev_mode), _out(J0[..., :n * n].reshape(tuple(arr0.shape) + (n, n)), dev_mode),
            _out(J0[..., n * n:], dev_mode))


class LeftoverFn(torch.autograd.Function):
    """arr0 (q, q, *tail) of the leftover strategy with the reference's custom VJP
    (jax_vjps/hermite.py:381-430), on the device; PyTorch's convention as DiagonalFn."""

    @staticmethod
    def forward(ctx, A, B, C, cutoffs):
        cut = tuple(cutoffs)
        W = device_leftover_slots(A.detach(), B.detach(), C.detach(), cut)
        Ad = raw(A.detach().to(torch.complex128)).contiguous()
        Bd = raw(B.detach().to(torch.complex128)).contiguous()
        cd = raw(C.detach().to(torch.complex128)).reshape(1).contiguous()
        ctx.save_for_backward(Ad, Bd, cd, W)
        ctx.cut = cut
        ctx.c_shape = C.shape
        E = cut[0] ** 2 * int(np.prod(cut[1:]))
        return W[:E].reshape((cut[0], cut[0]) + tuple(cut[1:])).clone()

    @staticmethod
    def backward(ctx, grad):
        A, B, C, W = ctx.saved_tensors
        cut = ctx.cut
        M = len(cut)
        n = 2 * M
        J = _lo_jacobian(A, B, W, cut, A.device)
        g = grad.conj().resolve_conj().to(torch.complex128).reshape(-1).contiguous()
        dA = torch.empty((n, n), dtype=torch.complex128, device=A.device)
        dB = torch.empty((n,), dtype=torch.complex128, device=A.device)
        dC = torch.empty((1,), dtype=torch.complex128, device=A.device)
        _, sh = _shape_arr(cut)
        _lib.check(_lib.load().mm_leftover_vjp(M, sh, J.data_ptr(), W.data_ptr(), C.data_ptr(), g.data_ptr(),
                                               dA.data_ptr(), dB.data_ptr(), dC.data_ptr(), _stream()),
                   "mm_leftover_vjp")
        return dA.conj(), dB.conj(), dC.conj().reshape(ctx.c_shape), None


def hermite_renormalized_1leftoverMode_autograd(A, B, C, output_cutoff, pnr_cutoffs, reorderedAB: bool = True):
    """Differentiable leftover-mode density matrices, ``math.hermite_renormalized_1leftoverMode`` under
    the JAX backend (backend_jax.py:524-534): (oc+1, oc+1, pnr_1+1, ...) for CUDA tensors."""
    A, B = reorder_AB_bargmann(A, B) if reorderedAB else (A, B)
    cutoffs = (int(output_cutoff) + 1, *(int(p) + 1 for p in pnr_cutoffs))
    return LeftoverFn.apply(A, B, C, cutoffs)


# ----------------------------------------------------------------- fast_diagonal
def fast_diagonal(A, b, c, output_cutoff, pnr_cutoffs, stable: bool = False):
    """Conditional density matrices of mode 0: (pnr_1+1, ..., oc+1, oc+1).

    With no detected mode (``pnr_cutoffs == ()``) the result is the first block alone, the
    (oc+1, oc+1) recurrence of mode 0 (where the reference returns it too, for oc <= 1; for
    larger oc its weight loop fails on the empty cutoff tuple)."""
    dev_mode = _is_dev(A)
    dev = A.device if dev_mode else require_cuda()
    pnr = tuple(int(p) for p in pnr_cutoffs)
    oc = int(output_cutoff)
    L = len(pnr) + 1
    Ad, bd = _to_dev(A, dev).contiguous(), _to_dev(b, dev).reshape(-1).contiguous()
    cd = _to_dev(c, dev).reshape(-1)[:1].contiguous()
    if Ad.shape != (2 * L, 2 * L) or bd.shape != (2 * L,):
        raise ValueError(f"fast_diagonal: A {tuple(Ad.shape)} / b {tuple(bd.shape)} do not match {L} modes")
    if L == 1:
        G = device_fwd(Ad, bd, cd.reshape(()), (oc + 1, oc + 1), bool(stable))
        return _out(G, dev_mode)
    lib = _lib.load()
    _, sh = _shape_arr(pnr)
    out = torch.empty(tuple(p + 1 for p in pnr) + (oc + 1, oc + 1), dtype=torch.complex128, device=dev)
    ws = Workspace(lib.mm_fast_diagonal_workspace_bytes(L, sh, oc), dev)
    _lib.check(lib.mm_fast_diagonal(L, sh, oc, Ad.data_ptr(), bd.data_ptr(), cd.data_ptr(), int(bool(stable)),
                                    out.data_ptr(), ws.ptr, ws.nbytes, _stream()), "mm_fast_diagonal")
    _finish(ws, "fast_diagonal")
    return _out(out, dev_mode)


def hermite_renormalized_1leftoverMode(A, b, c, output_cutoff, pnr_cutoffs, stable: bool = False,
                                       reorderedAB: bool = True):
    """``BackendNumpy.hermite_renormalized_1leftoverMode`` (backend_numpy.py:434-446): fast_diagonal
    with the two mode-0 axes moved to the front, (oc+1, oc+1, pnr_1+1, ...).  As there,
    ``reorderedAB`` is accepted and not used.  (``math.hermite_renormalized_1leftoverMode``,
    backend_manager.py:759-787, passes its ``reorderedAB`` positionally, so through the facade it
    lands in ``stable``.)"""
    r = fast_diagonal(A, b, c, output_cutoff, pnr_cutoffs, stable)
    K = len(tuple(pnr_cutoffs))
    perm = (K, K + 1, *range(K))
    if isinstance(r, torch.Tensor):
        return r.permute(perm)
    return np.transpose(r, perm)

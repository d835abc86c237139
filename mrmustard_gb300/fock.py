"""Fock-space contraction on the GB300 library.

The reference contracts Fock arrays with ``ArrayAnsatz.contract``
(mrmustard/physics/ansatz/array_ansatz.py:159-226): labels become an einsum string,
``math.einsum`` hands it to opt_einsum (mrmustard/math/backend_manager.py:526-548), which reduces
a gate-on-kets contraction to numpy ``tensordot`` -> BLAS zgemm.  With the reference's wire order
(bra_out, bra_in, ket_out, ket_in, modes ascending; mrmustard/physics/wires.py:100-105) a 2-mode
unitary's Fock tensor is (out0, out1, in0, in1) and the contraction with kets (n, in0, in1) is
one complex GEMM: U reshaped (c0*c1, c0'*c1') times the kets stacked as columns.

``fock_gemm(U, X, mode)`` computes Y = U X with the native FP64 kernel (``"fp64"``: DFMA), the
FP64 tensor-core kernel (``"dmma"``: mma.sync .f64) or the Ozaki-split BF16 tensor-core kernel
(``"ozaki"``); ``apply_unitary`` is the gate-on-kets wrapper.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .hermite import Workspace, _is_dev, _stream, raw, require_cuda

__all__ = ["fock_gemm", "apply_unitary"]

_MODES = {"fp64": 0, "ozaki": 1, "ozaki_bf16": 1, "dmma": 2, "fp64_dmma": 2}


def fock_gemm(U, X, mode: str = "fp64", slices: int = 7, out=None):
    """Y = U @ X for complex128 matrices (numpy in -> numpy out, CUDA tensors stay on device)."""
    lib = _lib.load()
    if mode not in _MODES:
        raise ValueError(f"mode must be one of {sorted(_MODES)}")
    dev_mode = _is_dev(U) or _is_dev(X)
    device = U.device if _is_dev(U) else (X.device if _is_dev(X) else require_cuda())
    Ud = raw(torch.as_tensor(U, dtype=torch.complex128, device=device))
    Xd = raw(torch.as_tensor(X, dtype=torch.complex128, device=device))
    if Ud.dim() != 2 or Xd.dim() != 2 or Ud.shape[1] != Xd.shape[0]:
        raise ValueError(f"shapes {tuple(Ud.shape)} and {tuple(Xd.shape)} do not chain")
    M, K = Ud.shape
    N = Xd.shape[1]
    Y = torch.empty((M, N), dtype=torch.complex128, device=device)
    m = _MODES[mode]
    nbytes = lib.mm_fock_gemm_workspace_bytes(m, M, N, K, slices)
    if nbytes == 0:
        raise ValueError("invalid contraction arguments")
    ws = Workspace(nbytes, device)
    _lib.check(lib.mm_fock_gemm(m, M, N, K, Ud.data_ptr(), Xd.data_ptr(), Y.data_ptr(), slices, ws.ptr, ws.nbytes,
                                _stream()), "mm_fock_gemm")
    if out is not None:
        if isinstance(out, torch.Tensor):
            out.copy_(Y)
        else:
            out[...] = Y.cpu().numpy()
        return out
    return Y if dev_mode else Y.cpu().numpy()


def apply_unitary(U, kets, mode: str = "fp64", slices: int = 7):
    """Apply an n-mode gate Fock tensor U (out..., in...) to kets (batch, in...) -> (batch, out...)."""
    Ut = U if isinstance(U, torch.Tensor) else np.asarray(U)
    nin = kets.ndim - 1
    out_shape = tuple(Ut.shape[: Ut.ndim - nin])
    in_shape = tuple(Ut.shape[Ut.ndim - nin:])
    if tuple(kets.shape[1:]) != in_shape:
        raise ValueError(f"kets {tuple(kets.shape)} do not match the gate's input axes {in_shape}")
    rows = int(np.prod(out_shape))
    cols = int(np.prod(in_shape))
    Um = Ut.reshape(rows, cols)
    X = kets.reshape(kets.shape[0], cols).T
    X = X.contiguous() if isinstance(X, torch.Tensor) else np.ascontiguousarray(X)
    Y = fock_gemm(Um, X, mode=mode, slices=slices)
    Y = Y.T.reshape((kets.shape[0],) + out_shape)
    return Y

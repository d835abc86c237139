"""Binomial fill of a Fock tensor (by total photon number, with an L2 early stop) on the GPU.

Mirrors ``binomial(local_cutoffs, A, b, c, max_l2, global_cutoff) -> (G, norm)``
(mrmustard/math/lattice/strategies/binomial.py:30-70) and the backend method
``hermite_renormalized_binomial(A, B, C, shape, max_l2, global_cutoff) -> G``
(mrmustard/math/backend_numpy.py:405-421: ``max_l2`` defaults to ``AUTOSHAPE_PROBABILITY`` and
``global_cutoff`` to ``sum(shape) - len(shape) + 1``).  The amplitudes kept are those of total
photon number up to the first one after which the running sum of |G|^2 exceeds ``max_l2``;
the rest are zero.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .hermite import Workspace, _finish, _shape_arr, _stream, _to_dev, require_cuda
from .settings import settings

__all__ = ["binomial", "hermite_renormalized_binomial", "device_binomial"]


def device_binomial(A, b, c, shape, max_l2, global_cutoff):
    """Device tensors in and out: returns (G, norm) with G on the device and norm a 0-d tensor."""
    dev = A.device if isinstance(A, torch.Tensor) and A.is_cuda else require_cuda()
    Ad, bd, cd = _to_dev(A, dev), _to_dev(b, dev), _to_dev(c, dev).reshape(-1)
    shape, sh = _shape_arr(shape)
    D = len(shape)
    if Ad.shape != (D, D) or bd.shape != (D,) or cd.numel() < 1:
        raise ValueError(f"binomial: A {tuple(Ad.shape)} / b {tuple(bd.shape)} do not match shape {shape}")
    lib = _lib.load()
    G = torch.empty(shape, dtype=torch.complex128, device=dev)
    norm = torch.empty((), dtype=torch.float64, device=dev)
    ws = Workspace(lib.mm_binomial_workspace_bytes(D, sh), dev)
    l2 = float("inf") if max_l2 is None else float(max_l2)
    _lib.check(lib.mm_binomial(D, sh, Ad.data_ptr(), bd.data_ptr(), cd.data_ptr(), l2, int(global_cutoff),
                               G.data_ptr(), norm.data_ptr(), ws.ptr, ws.nbytes, _stream()), "mm_binomial")
    _finish(ws, "binomial")
    return G, norm


def binomial(local_cutoffs, A, b, c, max_l2, global_cutoff):
    """The reference strategy: numpy in, (G numpy, norm float) out (device tensors in: device G)."""
    dev_mode = isinstance(A, torch.Tensor) and A.is_cuda
    G, norm = device_binomial(A, b, c, tuple(int(x) for x in local_cutoffs), max_l2, global_cutoff)
    if dev_mode:
        return G, float(norm)
    return G.cpu().numpy(), float(norm)


def hermite_renormalized_binomial(A, B, C, shape, max_l2=None, global_cutoff=None):
    """The backend method: the binomial-filled tensor of ``shape`` with the reference's defaults."""
    shape = tuple(int(x) for x in shape)
    max_l2 = max_l2 or settings.AUTOSHAPE_PROBABILITY
    global_cutoff = global_cutoff or sum(shape) - len(shape) + 1
    return binomial(shape, A, B, C, max_l2, global_cutoff)[0]

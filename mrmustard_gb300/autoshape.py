"""Per-mode Fock cutoffs of Gaussian states (autoshape) on the GPU.

Mirrors ``autoshape_numba(A, b, c, max_prob, max_shape, min_shape)``
(mrmustard/math/lattice/autoshape.py:23-154), which ``State.auto_shape``
(mrmustard/lab/states/base.py:383-430) calls on the density-matrix triple of a state
(``ansatz.conj & ansatz`` for a ket): A is 2M x 2M, b has 2M entries (bra copy first, then
ket copy), c is the vacuum amplitude.  The result is the int64 array of M cutoffs, each the
number of steps the reference's buffered single-mode recurrence takes to collect ``max_prob``
of the mode's marginal, clipped to [min_shape, max_shape].

``autoshape_batched`` runs many states with the same M in one launch (device tensors in and
out); ``ket_dm_triple`` builds the density-matrix triple of a ket the way the reference's
``conj & ansatz`` does.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _lib
from .hermite import _stream, _to_dev, ensure_device_ready, require_cuda
from .settings import settings

__all__ = ["autoshape_numba", "autoshape_batched", "ket_dm_triple"]


def _params(max_prob, max_shape, min_shape):
    # the reference's caller passes `x or settings.X` (base.py:421-423)
    return (float(max_prob or settings.AUTOSHAPE_PROBABILITY), int(max_shape or settings.AUTOSHAPE_MAX),
            int(min_shape or settings.AUTOSHAPE_MIN))


def autoshape_batched(A, b, c, max_prob=None, max_shape=None, min_shape=None) -> torch.Tensor:
    """Cutoffs of B states with M modes: A (B, 2M, 2M), b (B, 2M), c (B,) -> int64 (B, M) on the
    device.  A state whose reduction is singular gets -1 in every mode (the reference raises)."""
    dev = A.device if isinstance(A, torch.Tensor) and A.is_cuda else require_cuda()
    ensure_device_ready(dev)
    Ad, bd, cd = _to_dev(A, dev), _to_dev(b, dev), _to_dev(c, dev).reshape(-1)
    if Ad.dim() != 3 or Ad.shape[1] != Ad.shape[2] or Ad.shape[1] % 2 or bd.shape != Ad.shape[:2]:
        raise ValueError(f"autoshape_batched needs A (B, 2M, 2M), b (B, 2M), c (B,); got {tuple(Ad.shape)}, "
                         f"{tuple(bd.shape)}, {tuple(cd.shape)}")
    B, M = Ad.shape[0], Ad.shape[1] // 2
    if cd.shape[0] != B:
        raise ValueError("autoshape_batched: c needs one entry per state")
    p, hi, lo = _params(max_prob, max_shape, min_shape)
    out = torch.empty((B, M), dtype=torch.int64, device=dev)
    with torch.cuda.device(dev):
        _lib.check(_lib.load().mm_autoshape_batched(B, M, Ad.data_ptr(), bd.data_ptr(), cd.data_ptr(), p, hi, lo,
                                                    out.data_ptr(), _stream()), "mm_autoshape_batched")
    return out


def autoshape_numba(A, b, c, max_prob=None, max_shape=None, min_shape=None) -> np.ndarray:
    """The reference's ``autoshape_numba`` for one state: numpy int64 array of M cutoffs."""
    A = np.asarray(A.detach().cpu() if isinstance(A, torch.Tensor) else A, np.complex128)
    b = np.asarray(b.detach().cpu() if isinstance(b, torch.Tensor) else b, np.complex128).reshape(-1)
    c = np.asarray(c.detach().cpu() if isinstance(c, torch.Tensor) else c, np.complex128).reshape(-1)
    shape = autoshape_batched(A[None], b[None], c[:1], max_prob, max_shape, min_shape)[0].cpu().numpy()
    if (shape < 0).any():
        raise np.linalg.LinAlgError("autoshape: singular matrix in the reduction to one mode")
    return shape


def ket_dm_triple(A, b, c):
    """Density-matrix triple of a ket's triple, as ``ansatz.conj & ansatz``: A -> [[A*, 0], [0, A]],
    b -> [b*, b], c -> |c|^2 (numpy arrays)."""
    A = np.asarray(A, np.complex128)
    b = np.asarray(b, np.complex128).reshape(-1)
    M = b.shape[0]
    Adm = np.zeros((2 * M, 2 * M), np.complex128)
    Adm[:M, :M] = np.conj(A)
    Adm[M:, M:] = A
    return Adm, np.concatenate([np.conj(b), b]), np.complex128(abs(complex(np.asarray(c).reshape(-1)[0])) ** 2)

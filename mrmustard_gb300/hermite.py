"""Host-side mirror of MrMustard's ``hermite_renormalized`` path on the GB300 library.

Two layers, both with the reference's names, argument meaning and errors:

* kernel level (``mrmustard/math/lattice/strategies/vanilla/__init__.py:17-27``):
  ``vanilla``, ``stable``, ``vanilla_batch``, ``vanilla_vjp``, ``vanilla_batch_vjp`` and the
  drop-in aliases ``vanilla_numba``, ``stable_numba``, ``vanilla_batch_numba``,
  ``vanilla_vjp_numba``, ``vanilla_batch_vjp_numba``;
* facade level: ``hermite_renormalized(A, b, c, shape, stable=False, out=None)`` with the
  batching / broadcasting / ``out`` rules of ``BackendManager.hermite_renormalized``
  (``mrmustard/math/backend_manager.py:643-727``).

Arrays may be numpy arrays (host; results come back as numpy, like the reference's numpy
backend) or torch tensors on a CUDA device (results stay on the device).  All compute runs
in ``libmm_gb300.so``; without a CUDA device every call raises.
"""

from __future__ import annotations

import ctypes
import threading
from collections.abc import Sequence

import numpy as np
import torch

from . import _lib
from .settings import settings

__all__ = [
    "vanilla",
    "stable",
    "vanilla_batch",
    "vanilla_vjp",
    "vanilla_batch_vjp",
    "vanilla_numba",
    "stable_numba",
    "vanilla_batch_numba",
    "vanilla_vjp_numba",
    "vanilla_batch_vjp_numba",
    "hermite_renormalized",
    "hermite_renormalized_batched",
    "device_fwd",
    "device_vjp",
    "checkpoint_elems",
    "device_checkpoint_save",
    "device_vjp_checkpointed",
]


# ----------------------------------------------------------------- plumbing
def require_cuda() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("mrmustard_gb300 computes on a CUDA device only; no CUDA device is available")
    return torch.device("cuda", torch.cuda.current_device())


_SELFTESTED: set[int] = set()


def ensure_device_ready(device) -> None:
    """Run the library's device self-test once per device (raises if it fails)."""
    idx = torch.device(device).index
    idx = torch.cuda.current_device() if idx is None else idx
    if idx in _SELFTESTED:
        return
    lib = _lib.load()
    with torch.cuda.device(idx):
        buf = torch.zeros(8192, dtype=torch.uint8, device=torch.device("cuda", idx))
        nbad = ctypes.c_int(-1)
        _lib.check(lib.mm_selftest(buf.data_ptr(), 8192, torch.cuda.current_stream().cuda_stream, ctypes.byref(nbad)),
                   "mm_selftest")
    if nbad.value != 0:
        raise RuntimeError(f"libmm_gb300 device self-test failed ({nbad.value} view fields wrong): "
                           "the kernels were mis-compiled for this GPU; refusing to run them")
    _SELFTESTED.add(idx)


def raw(t: torch.Tensor) -> torch.Tensor:
    """Contiguous complex128 storage of a tensor (converted if needed, torch's lazy conj/neg bits
    resolved), so that its data pointer holds exactly its values in the library's layout."""
    if t.dtype != torch.complex128:
        t = t.to(torch.complex128)
    return t.resolve_conj().resolve_neg().contiguous()


def _is_dev(x) -> bool:
    return isinstance(x, torch.Tensor) and x.is_cuda


def _to_dev(x, device) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x.detach()
        if t.dtype != torch.complex128:
            t = t.to(torch.complex128)
        return raw(t.to(device))
    a = np.ascontiguousarray(np.asarray(x, dtype=np.complex128))
    return torch.from_numpy(a).to(device)


def _ptr(t: torch.Tensor) -> int:
    return t.data_ptr()


def _stream() -> int:
    return torch.cuda.current_stream().cuda_stream


def _shape_arr(shape: Sequence[int]):
    shape = tuple(int(s) for s in shape)
    return shape, (ctypes.c_int64 * max(1, len(shape)))(*shape)


class Workspace:
    """Per-call device scratch from torch's stream-ordered caching allocator."""

    def __init__(self, nbytes: int, device):
        lib = _lib.load()
        ensure_device_ready(device)
        self.nbytes = max(int(nbytes), 512)
        self.buf = torch.empty(self.nbytes, dtype=torch.uint8, device=device)
        _lib.check(lib.mm_workspace_init(self.ptr, self.nbytes, _stream()), "mm_workspace_init")

    @property
    def ptr(self) -> int:
        return self.buf.data_ptr()

    def check_status(self, where: str) -> None:
        st = ctypes.c_int(0)
        lib = _lib.load()
        _lib.check(lib.mm_workspace_status(self.ptr, _stream(), ctypes.byref(st)), "mm_workspace_status")
        if st.value != 0:
            raise _lib.MMError(st.value, where, "device status word")


def _finish(ws: Workspace, where: str) -> None:
    if settings.CHECK_DEVICE_STATUS:
        ws.check_status(where)


# ----------------------------------------------------------- device entry points
def device_fwd(A: torch.Tensor, b: torch.Tensor, c: torch.Tensor, shape, stable: bool = False,
               out: torch.Tensor | None = None) -> torch.Tensor:
    """Forward on device tensors.  A: (B,D,D) or (D,D); b: (B,D) or (D,); c: (B,) or ()."""
    lib = _lib.load()
    A, b, c = raw(A), raw(b), raw(c)
    batched = A.dim() == 3
    shape, sh = _shape_arr(shape)
    D = len(shape)
    B = A.shape[0] if batched else 1
    if A.shape[-1] != D or A.shape[-2] != D or b.shape[-1] != D:
        raise ValueError(f"A {tuple(A.shape)} / b {tuple(b.shape)} do not match the {D} axes of shape {shape}")
    full = ((B,) if batched else ()) + shape
    if out is None:
        out = torch.empty(full, dtype=torch.complex128, device=A.device)
    elif tuple(out.shape) != full or out.dtype != torch.complex128 or not out.is_contiguous() or not out.is_cuda:
        raise ValueError(f"out must be a contiguous complex128 CUDA tensor of shape {full}")
    if B == 0 or out.numel() == 0:
        return out
    ws = Workspace(lib.mm_hermite_workspace_bytes(D, sh, B), A.device)
    c = c.reshape(-1)
    if batched:
        rc = lib.mm_hermite_fwd_batched(B, D, sh, _ptr(A), _ptr(b), _ptr(c), int(bool(stable)), _ptr(out), ws.ptr,
                                        ws.nbytes, _stream())
    else:
        rc = lib.mm_hermite_fwd(D, sh, _ptr(A), _ptr(b), _ptr(c), int(bool(stable)), _ptr(out), ws.ptr, ws.nbytes,
                                _stream())
    _lib.check(rc, "mm_hermite_fwd")
    _finish(ws, "hermite forward")
    return out


def device_vjp(G: torch.Tensor, c: torch.Tensor, dLdG: torch.Tensor, batched: bool):
    """VJP on device tensors; returns (dA, db, dc) on the device."""
    lib = _lib.load()
    G, c, dLdG = raw(G), raw(c), raw(dLdG)
    shape = tuple(G.shape[1:]) if batched else tuple(G.shape)
    shape, sh = _shape_arr(shape)
    D = len(shape)
    B = G.shape[0] if batched else 1
    if tuple(dLdG.shape) != tuple(G.shape):
        raise ValueError(f"dLdG shape {tuple(dLdG.shape)} must equal G shape {tuple(G.shape)}")
    dev = G.device
    dA = torch.empty(((B,) if batched else ()) + (D, D), dtype=torch.complex128, device=dev)
    db = torch.empty(((B,) if batched else ()) + (D,), dtype=torch.complex128, device=dev)
    dc = torch.empty((B,) if batched else (), dtype=torch.complex128, device=dev)
    if B == 0:
        return dA, db, dc
    ws = Workspace(lib.mm_hermite_workspace_bytes(D, sh, B), dev)
    c = c.reshape(-1)
    if batched:
        rc = lib.mm_hermite_vjp_batched(B, D, sh, _ptr(G), _ptr(c), _ptr(dLdG), _ptr(dA), _ptr(db), _ptr(dc), ws.ptr,
                                        ws.nbytes, _stream())
    else:
        rc = lib.mm_hermite_vjp(D, sh, _ptr(G), _ptr(c), _ptr(dLdG), _ptr(dA), _ptr(db), _ptr(dc), ws.ptr, ws.nbytes,
                                _stream())
    _lib.check(rc, "mm_hermite_vjp")
    _finish(ws, "hermite vjp")
    return dA, db, dc


def checkpoint_elems(shape, K: int) -> int:
    """Complex values of the checkpoint buffer of one instance (mm_hermite_checkpoint_elems)."""
    shape, sh = _shape_arr(shape)
    n = int(_lib.load().mm_hermite_checkpoint_elems(len(shape), sh, int(K)))
    if n < 0:
        raise ValueError(f"checkpoint segments need K >= 2 and a valid shape (K={K}, shape={shape})")
    return n


def device_checkpoint_save(G: torch.Tensor, shape, K: int, batched: bool) -> torch.Tensor:
    """Checkpoint slabs of a forward's G (slab 0, then the two slabs before every K-th slab
    along axis 0): (checkpoint_elems,) or (B, checkpoint_elems) complex128 on G's device."""
    lib = _lib.load()
    G = raw(G)
    shape, sh = _shape_arr(shape)
    n = checkpoint_elems(shape, K)
    B = G.shape[0] if batched else 1
    ck = torch.empty(((B,) if batched else ()) + (n,), dtype=torch.complex128, device=G.device)
    Gf, ckf = G.reshape(B, -1), ck.reshape(B, n)
    for k in range(B):
        _lib.check(lib.mm_hermite_checkpoint_save(len(shape), sh, int(K), _ptr(Gf[k]), _ptr(ckf[k]), _stream()),
                   "mm_hermite_checkpoint_save")
    return ck


def device_vjp_checkpointed(A: torch.Tensor, b: torch.Tensor, c: torch.Tensor, ckpt: torch.Tensor,
                            dLdG: torch.Tensor, shape, K: int, batched: bool):
    """VJP from checkpoints (mm_hermite_vjp_checkpointed): G is recomputed K slabs at a time from
    the checkpoint slabs and A, b; never held whole.  Returns (dA, db, dc) on the device."""
    lib = _lib.load()
    A, b, c, ckpt, dLdG = raw(A), raw(b), raw(c), raw(ckpt), raw(dLdG)
    shape, sh = _shape_arr(shape)
    D = len(shape)
    B = A.shape[0] if batched else 1
    dev = A.device
    dA = torch.empty(((B,) if batched else ()) + (D, D), dtype=torch.complex128, device=dev)
    db = torch.empty(((B,) if batched else ()) + (D,), dtype=torch.complex128, device=dev)
    dc = torch.empty((B,) if batched else (), dtype=torch.complex128, device=dev)
    if B == 0:
        return dA, db, dc
    nbytes = lib.mm_hermite_vjp_checkpointed_workspace_bytes(D, sh, int(K))
    if nbytes == 0:
        raise ValueError(f"checkpointed VJP: bad shape {shape} or K={K}")
    ws = Workspace(nbytes, dev)
    Af, bf, cf = A.reshape(B, D, D), b.reshape(B, D), c.reshape(B)
    ckf, gf = ckpt.reshape(B, -1), dLdG.reshape(B, -1)
    dAf, dbf, dcf = dA.reshape(B, D, D), db.reshape(B, D), dc.reshape(B)
    for k in range(B):
        _lib.check(lib.mm_hermite_vjp_checkpointed(D, sh, int(K), _ptr(Af[k]), _ptr(bf[k]), _ptr(cf[k:k + 1]),
                                                   _ptr(ckf[k]), _ptr(gf[k]), _ptr(dAf[k]), _ptr(dbf[k]),
                                                   _ptr(dcf[k:k + 1]), ws.ptr, ws.nbytes, _stream()),
                   "mm_hermite_vjp_checkpointed")
    _finish(ws, "checkpointed hermite vjp")
    return dA, db, dc


# ------------------------------------------------------------ kernel-level API
def _host_or_dev(*xs):
    dev_mode = any(_is_dev(x) for x in xs if x is not None)
    device = next((x.device for x in xs if _is_dev(x)), None) or require_cuda()
    return dev_mode, device


def _deliver(res: torch.Tensor, out, dev_mode: bool):
    """Return like the reference: into `out` when given, numpy for host callers."""
    if out is not None:
        if isinstance(out, torch.Tensor):
            if out.data_ptr() != res.data_ptr():
                out.copy_(res.reshape(out.shape))
            return out
        out[...] = res.cpu().numpy().reshape(out.shape)
        return out
    return res if dev_mode else res.cpu().numpy()


def _np_c128(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.complex128))


_SCALARS = (complex, float, int, np.number)
_tls = threading.local()
_SHAPES: dict = {}


def _raw_stream(idx: int) -> int:
    """The current torch stream of device `idx` as a cudaStream_t value (the cheap accessor when
    this torch has it)."""
    f = getattr(torch._C, "_cuda_getCurrentRawStream", None)
    return f(idx) if f is not None else torch.cuda.current_stream(idx).cuda_stream


def _fwd_host_fast(shape, A, b, c, stable_flag):
    """The reference's most common call (numpy A (D, D), b (D,), scalar c, no ``out``) with as
    little Python as possible: the inputs go into this thread's reusable host buffers (their
    addresses cached), the result into a fresh array, and one mm_hermite_fwd_host call does the
    rest (staging, launches, one synchronisation)."""
    D = len(shape)
    if A.shape != (D, D) or b.shape != (D,):
        raise ValueError(f"A {A.shape} / b {b.shape} do not match the {D} axes of shape {shape}")
    stages = getattr(_tls, "stages", None)
    if stages is None:
        stages = _tls.stages = {}
    st = stages.get(D)
    if st is None:
        bufs = (np.empty((D, D), np.complex128), np.empty(D, np.complex128), np.empty(1, np.complex128))
        st = stages[D] = (bufs, tuple(x.ctypes.data for x in bufs))
    (Ab, bb, cb), (pA, pb, pc) = st
    np.copyto(Ab, A)
    np.copyto(bb, b)
    cb[0] = c
    sh = _SHAPES.get(shape)
    if sh is None:
        if any(x == 0 for x in shape):
            return np.empty(shape, np.complex128)
        sh = _SHAPES.setdefault(shape, (ctypes.c_int64 * D)(*shape))
    G = np.empty(shape, np.complex128)
    idx = torch.cuda.current_device()
    if idx not in _SELFTESTED:
        ensure_device_ready(torch.device("cuda", idx))
    _lib.check(_lib.load().mm_hermite_fwd_host(D, sh, pA, pb, pc, int(bool(stable_flag)), G.ctypes.data,
                                               _raw_stream(idx)), "mm_hermite_fwd_host")
    return G


def _fwd_host(shape, A, b, c, stable_flag, out):
    """Unbatched forward with host (numpy) buffers: one library call that stages the inputs and the
    result through its own pinned and device buffers (mm_hermite_fwd_host)."""
    shape, sh = _shape_arr(shape)
    D = len(shape)
    A_h, b_h = _np_c128(A), _np_c128(b)
    c_h = _np_c128(c).reshape(-1)[:1]
    if A_h.shape != (D, D) or b_h.shape != (D,) or c_h.size != 1:
        raise ValueError(f"A {A_h.shape} / b {b_h.shape} do not match the {D} axes of shape {shape}")
    direct = (isinstance(out, np.ndarray) and out.dtype == np.complex128 and out.flags.c_contiguous
              and out.size == int(np.prod(shape)))
    target = out if direct else np.empty(shape, np.complex128)
    if target.size:
        ensure_device_ready(require_cuda())
        _lib.check(_lib.load().mm_hermite_fwd_host(D, sh, A_h.ctypes.data, b_h.ctypes.data, c_h.ctypes.data,
                                                   int(bool(stable_flag)), target.ctypes.data, _stream()),
                   "mm_hermite_fwd_host")
    if out is not None and not direct:
        out[...] = target.reshape(out.shape)
        return out
    return target if out is None else out


def _fwd_common(shape, A, b, c, stable_flag, out, batched):
    dev_mode, device = _host_or_dev(A, b, c, out)
    if not dev_mode and not batched and not isinstance(out, torch.Tensor):
        return _fwd_host(shape, A, b, c, stable_flag, out)
    A_d, b_d, c_d = _to_dev(A, device), _to_dev(b, device), _to_dev(c, device)
    direct = (
        isinstance(out, torch.Tensor) and out.is_cuda and out.is_contiguous() and out.dtype == torch.complex128
        and tuple(out.shape) == ((A_d.shape[0],) if batched else ()) + tuple(int(s) for s in shape)
    )
    res = device_fwd(A_d, b_d, c_d, shape, stable_flag, out if direct else None)
    return _deliver(res, out, dev_mode)


def vanilla(shape, A, b, c, out=None):
    """``vanilla_numba`` (core.py:25-124) on the GPU: Fock amplitudes of shape ``shape``."""
    return _fwd_common(shape, A, b, c, False, out, batched=False)


def stable(shape, A, b, c, out=None):
    """``stable_numba`` (core.py:127-213) on the GPU."""
    return _fwd_common(shape, A, b, c, True, out, batched=False)


def vanilla_batch(shape, A, b, c, stable=False, out=None):
    """``vanilla_batch_numba`` (batch.py:27-61): batch on axis 0 of A, b and c."""
    return _fwd_common(shape, A, b, c, bool(stable), out, batched=True)


def _vjp_host(G, c, dLdG):
    """Unbatched VJP with host (numpy) buffers through mm_hermite_vjp_host."""
    G_h, g_h = _np_c128(G), _np_c128(dLdG)
    c_h = _np_c128(c).reshape(-1)[:1]
    if G_h.shape != g_h.shape:
        raise ValueError(f"dLdG shape {g_h.shape} must equal G shape {G_h.shape}")
    shape, sh = _shape_arr(G_h.shape)
    D = len(shape)
    dA = np.empty((D, D), np.complex128)
    db = np.empty(D, np.complex128)
    dc = np.empty(1, np.complex128)
    if G_h.size:
        ensure_device_ready(require_cuda())
        _lib.check(_lib.load().mm_hermite_vjp_host(D, sh, G_h.ctypes.data, c_h.ctypes.data, g_h.ctypes.data,
                                                   dA.ctypes.data, db.ctypes.data, dc.ctypes.data, _stream()),
                   "mm_hermite_vjp_host")
    else:
        dA[...] = 0
        db[...] = 0
        dc[...] = 0
    return dA, db, complex(dc[0])


def _vjp_common(G, c, dLdG, batched):
    dev_mode, device = _host_or_dev(G, c, dLdG)
    if not dev_mode and not batched:
        return _vjp_host(G, c, dLdG)
    G_d, c_d, g_d = _to_dev(G, device), _to_dev(c, device), _to_dev(dLdG, device)
    dA, db, dc = device_vjp(G_d, c_d, g_d, batched)
    if dev_mode:
        return dA, db, dc
    return dA.cpu().numpy(), db.cpu().numpy(), (dc.cpu().numpy() if batched else complex(dc.item()))


def vanilla_vjp(G, c, dLdG):
    """``vanilla_vjp_numba`` (gradients.py:25-82): returns dL/dA, dL/db, dL/dc."""
    return _vjp_common(G, c, dLdG, batched=False)


def vanilla_batch_vjp(G, c, dLdG):
    """``vanilla_batch_vjp_numba`` (gradients.py:85-116)."""
    return _vjp_common(G, c, dLdG, batched=True)


# drop-in aliases with the reference's names
vanilla_numba = vanilla
stable_numba = stable
vanilla_batch_numba = vanilla_batch
vanilla_vjp_numba = vanilla_vjp
vanilla_batch_vjp_numba = vanilla_batch_vjp


# ----------------------------------------------------------------- facade
def _ndim(x):
    return x.dim() if isinstance(x, torch.Tensor) else np.ndim(x)


def _shp(x):
    return tuple(x.shape) if isinstance(x, (torch.Tensor, np.ndarray)) else np.shape(x)


def _reshape(x, s):
    return x.reshape(s)


def _broadcast(x, s):
    if isinstance(x, torch.Tensor):
        return x.broadcast_to(s)
    return np.broadcast_to(np.asarray(x), s)


def hermite_renormalized_batched(A, b, c, shape, stable=False, out=None):
    """``BackendNumpy.hermite_renormalized_batched`` (backend_numpy.py:394-403)."""
    return vanilla_batch(tuple(shape), A, b, c, stable, out)


def hermite_renormalized(A, b, c, shape, stable=False, out=None):
    """``math.hermite_renormalized`` (backend_manager.py:643-727) on the GB300 library.

    1. A.ndim = 2, b.ndim = 1, c scalar: unbatched;
    2. A.ndim = 2, b.ndim > 1: b-batched, A and c broadcast over b's batch dims;
    3. A.ndim > 2, b.ndim > 1, c.ndim > 0: fully batched, batch dims flattened.
    ``stable`` is also switched on by ``settings.STABLE_FOCK_CONVERSION``.
    """
    shape = tuple(int(s) for s in shape)
    if (out is None and type(A) is np.ndarray and type(b) is np.ndarray and A.ndim == 2 and b.ndim == 1
            and isinstance(c, _SCALARS) and not (stable or settings.STABLE_FOCK_CONVERSION)
            and A.dtype == np.complex128 and b.dtype == np.complex128):
        return _fwd_host_fast(shape, A, b, c, False)

    def check_out_shape(batch_shape):
        if out is not None and any(d_out < d for d_out, d in zip(_shp(out), batch_shape + shape)):
            raise ValueError(f"batch+shape {batch_shape + shape} is too large for out.shape={_shp(out)}")

    stable = stable or settings.STABLE_FOCK_CONVERSION
    if _ndim(A) > 2 and _ndim(b) > 1 and _ndim(c) > 0:
        batch_shape = _shp(A)[:-2]
        check_out_shape(batch_shape)
        if _shp(b)[:-1] != batch_shape:
            raise ValueError(f"b.shape={_shp(b)} must match batch_shape={batch_shape}")
        if _shp(c)[: len(batch_shape)] != batch_shape:
            raise ValueError(f"c.shape={_shp(c)} must match batch_shape={batch_shape}")
        n = int(np.prod(batch_shape))
        A2 = _reshape(A, (n, *_shp(A)[-2:]))
        b2 = _reshape(b, (n, _shp(b)[-1]))
        c2 = _reshape(c, (n,))
        out2 = _reshape(out, (n, *shape)) if out is not None else None
        res = hermite_renormalized_batched(A2, b2, c2, shape, stable, out2)
        return out if out is not None else _reshape(res, batch_shape + shape)
    if _ndim(A) == 2 and _ndim(b) > 1:
        batch_shape = _shp(b)[:-1]
        check_out_shape(batch_shape)
        n = int(np.prod(batch_shape))
        b2 = _reshape(b, (n, _shp(b)[-1]))
        A2 = _broadcast(A, (n, *_shp(A)))
        c2 = _broadcast(c, (n,))
        out2 = _reshape(out, (n, *shape)) if out is not None else None
        res = hermite_renormalized_batched(A2, b2, c2, shape, stable, out2)
        return out if out is not None else _reshape(res, batch_shape + shape)
    check_out_shape(())
    if stable:
        return stable_numba(shape, A, b, c, out)
    return vanilla_numba(shape, A, b, c, out)

"""CPU oracle for the Gaussian->Fock hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline leg and its
``--impl reference`` arm) may import this package.  The product package
``mrmustard_gb300`` never does: it has no CPU path at all.

Contents:

* ``hermite_oracle.c`` -- a plain-C restatement of the reference's numba strategies
  (``mrmustard/math/lattice/strategies/vanilla/{core,batch,gradients}.py``), compiled with gcc
  (``-ffp-contract=off``, OpenMP over instances as numba's ``prange``).
* this module -- ctypes bindings with numpy in/out, plus the FP64 CPU oracle of the Fock
  contraction (numpy ``@``, i.e. BLAS zgemm, as ``ArrayAnsatz.contract`` reaches through
  ``math.einsum`` -> opt_einsum -> tensordot, mrmustard/physics/ansatz/array_ansatz.py:223 and
  mrmustard/math/backend_manager.py:526-548).

Parity of the C restatement is pinned against outputs of the reference source itself
(``tests/golden/hermite_golden.npz``, generated by ``tests/golden/make_golden.py``).
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "hermite_oracle.c"
SOURCES = (SRC, HERE / "autoshape_oracle.c", HERE / "binomial_oracle.c", HERE / "diagonal_oracle.c")
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "liboracle.so"
# the same recurrence and VJP source built for speed, used only as a timed CPU baseline:
# -O3 with contraction to FMA and unrolling (no -march flags: the box's baseline aarch64 ISA
# already has FMA and NEON), never as the parity checker
FAST_LIB_PATH = BUILD_DIR / "liboracle_fast.so"
FAST_FLAGS = ["-O3", "-ffp-contract=fast", "-funroll-loops"]

_lib = None
_fast = None


def build(force: bool = False) -> Path:
    """Compile the C restatement into ``oracle/_build/liboracle.so`` (OpenMP when available)."""
    BUILD_DIR.mkdir(exist_ok=True)
    if (LIB_PATH.exists() and not force
            and all(LIB_PATH.stat().st_mtime >= src.stat().st_mtime for src in SOURCES)):
        return LIB_PATH
    base = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
            *map(str, SOURCES)]
    tmp = BUILD_DIR / f"liboracle.{os.getpid()}.so"
    try:
        subprocess.run(base + ["-fopenmp", "-o", str(tmp), "-lm"], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base + ["-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, LIB_PATH)
    build_fast(force)
    return LIB_PATH


def build_fast(force: bool = False) -> Path:
    """Compile ``hermite_oracle.c`` with FAST_FLAGS into ``oracle/_build/liboracle_fast.so``."""
    BUILD_DIR.mkdir(exist_ok=True)
    if FAST_LIB_PATH.exists() and not force and FAST_LIB_PATH.stat().st_mtime >= SRC.stat().st_mtime:
        return FAST_LIB_PATH
    base = ["gcc", *FAST_FLAGS, "-std=c11", "-fPIC", "-shared", str(SRC)]
    tmp = BUILD_DIR / f"liboracle_fast.{os.getpid()}.so"
    try:
        subprocess.run(base + ["-fopenmp", "-o", str(tmp), "-lm"], check=True, capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base + ["-o", str(tmp), "-lm"], check=True)
    os.replace(tmp, FAST_LIB_PATH)
    return FAST_LIB_PATH


def fast_lib():
    """The speed build (timed baselines only)."""
    global _fast
    if _fast is None:
        build_fast()
        L = ctypes.CDLL(str(FAST_LIB_PATH))
        P, I64, I32 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
        for name, args in {
            "oracle_vanilla": [I32, P, P, P, P, P],
            "oracle_vjp": [I32, P, P, P, P, P, P, P],
            "oracle_fwd_ragged": [I64, P, P, P, P, P, P, P, P, I32, P, P, P],
            "oracle_vjp_ragged": [I64, P, P, P, P, P, P, P, P, P, P, P, P, P],
        }.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.oracle_num_threads.restype = ctypes.c_int
        _fast = L
    return _fast


def lib():
    global _lib
    if _lib is None:
        build()  # no-op unless a source is newer than the library
        L = ctypes.CDLL(str(LIB_PATH))
        P, I64, I32, D = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_double
        cplx = P
        for name, args in {
            "oracle_vanilla": [I32, P, P, P, cplx, P],
            "oracle_stable": [I32, P, P, P, cplx, P],
            "oracle_vjp": [I32, P, P, cplx, P, P, P, P],
            "oracle_fwd_batch": [I64, I32, P, P, P, P, I32, P],
            "oracle_vjp_batch": [I64, I32, P, P, P, P, P, P, P],
            "oracle_fwd_ragged": [I64, P, P, P, P, P, P, P, P, I32, P, P, P],
            "oracle_vjp_ragged": [I64, P, P, P, P, P, P, P, P, P, P, P, P, P],
            "oracle_autoshape": [I32, P, P, P, D, I64, I64, P],
            "oracle_autoshape_ragged": [I64, P, P, P, P, P, P, P, D, I64, I64, P],
        }.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.oracle_binomial.argtypes = [I32, P, P, P, P, D, I64, P, P]
        L.oracle_binomial.restype = D
        L.oracle_diagonal_amps.argtypes = [I32, P, I64, P, P, P, P]
        L.oracle_diagonal_amps.restype = ctypes.c_int
        L.oracle_diagonal_grad.argtypes = [I32, P, P, P, P, P]
        L.oracle_diagonal_grad.restype = ctypes.c_int
        L.oracle_diagonal_slots.argtypes = [I32]
        L.oracle_diagonal_slots.restype = I64
        L.oracle_fast_diagonal.argtypes = [I32, P, I64, P, P, P, I32, P]
        L.oracle_fast_diagonal.restype = ctypes.c_int
        L.oracle_leftover_amps.argtypes = [I32, P, P, P, P, P]
        L.oracle_leftover_amps.restype = ctypes.c_int
        L.oracle_leftover_grad.argtypes = [I32, P, P, P, P, P]
        L.oracle_leftover_grad.restype = ctypes.c_int
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_set_numpy_division.argtypes = [ctypes.c_int]
        L.oracle_set_numpy_division.restype = None
        _lib = L
    return _lib


def _c(x):
    x = complex(x)
    return ctypes.cast((ctypes.c_double * 2)(x.real, x.imag), ctypes.c_void_p)


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _cc(a):
    return np.ascontiguousarray(a, dtype=np.complex128)


def set_numpy_division(on: bool) -> None:
    """Select numpy's complex/real division (reference source under CPython) instead of numba's."""
    lib().oracle_set_numpy_division(int(bool(on)))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


def vanilla(shape, A, b, c, fast=False) -> np.ndarray:
    """``vanilla_numba(shape, A, b, c)`` (core.py:25-124); ``fast``: the speed build."""
    shape = tuple(int(s) for s in shape)
    A, b = _cc(A), _cc(b)
    sh = np.array(shape, np.int64)
    G = np.empty(shape, np.complex128)
    rc = (fast_lib() if fast else lib()).oracle_vanilla(len(shape), _ptr(sh), _ptr(A), _ptr(b), _c(c), _ptr(G))
    if rc:
        raise ValueError(f"oracle_vanilla failed ({rc})")
    return G


def stable(shape, A, b, c) -> np.ndarray:
    """``stable_numba(shape, A, b, c)`` (core.py:127-213)."""
    shape = tuple(int(s) for s in shape)
    A, b = _cc(A), _cc(b)
    sh = np.array(shape, np.int64)
    G = np.empty(shape, np.complex128)
    rc = lib().oracle_stable(len(shape), _ptr(sh), _ptr(A), _ptr(b), _c(c), _ptr(G))
    if rc:
        raise ValueError(f"oracle_stable failed ({rc})")
    return G


def vjp(G, c, dLdG, fast=False):
    """``vanilla_vjp_numba(G, c, dLdG)`` (gradients.py:25-82) -> (dA, db, dc); ``fast``: the speed build."""
    G, g = _cc(G), _cc(dLdG)
    D = G.ndim
    sh = np.array(G.shape, np.int64)
    dA = np.empty((D, D), np.complex128)
    db = np.empty(D, np.complex128)
    dc = np.empty(1, np.complex128)
    rc = (fast_lib() if fast else lib()).oracle_vjp(D, _ptr(sh), _ptr(G), _c(c), _ptr(g), _ptr(dA), _ptr(db), _ptr(dc))
    if rc:
        raise ValueError(f"oracle_vjp failed ({rc})")
    return dA, db, dc[0]


def fwd_batch(shape, A, b, c, stable=False) -> np.ndarray:
    """``vanilla_batch_numba(shape, A, b, c, stable)`` (batch.py:27-61)."""
    shape = tuple(int(s) for s in shape)
    A, b, c = _cc(A), _cc(b), _cc(c)
    B = A.shape[0]
    sh = np.array(shape, np.int64)
    G = np.empty((B, *shape), np.complex128)
    rc = lib().oracle_fwd_batch(B, len(shape), _ptr(sh), _ptr(A), _ptr(b), _ptr(c), int(bool(stable)), _ptr(G))
    if rc:
        raise ValueError(f"oracle_fwd_batch failed ({rc})")
    return G


def vjp_batch(G, c, dLdG):
    """``vanilla_batch_vjp_numba(G, c, dLdG)`` (gradients.py:85-116)."""
    G, c, g = _cc(G), _cc(c), _cc(dLdG)
    B, D = G.shape[0], G.ndim - 1
    sh = np.array(G.shape[1:], np.int64)
    dA = np.empty((B, D, D), np.complex128)
    db = np.empty((B, D), np.complex128)
    dc = np.empty(B, np.complex128)
    rc = lib().oracle_vjp_batch(B, D, _ptr(sh), _ptr(G), _ptr(c), _ptr(g), _ptr(dA), _ptr(db), _ptr(dc))
    if rc:
        raise ValueError(f"oracle_vjp_batch failed ({rc})")
    return dA, db, dc


class RaggedHost:
    """Packed host layout of a ragged batch (the same packing the GPU library uses)."""

    def __init__(self, shapes):
        self.shapes = [tuple(int(s) for s in sh) for sh in shapes]
        self.B = len(self.shapes)
        self.D = np.array([len(s) for s in self.shapes], np.int32)
        self.sizes = np.array([int(np.prod(s)) for s in self.shapes], np.int64)
        self.flat_shapes = np.array([x for s in self.shapes for x in s], np.int64)
        self.shape_off = np.concatenate([[0], np.cumsum(self.D)[:-1]]).astype(np.int64)
        self.a_off = np.concatenate([[0], np.cumsum(self.D.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
        self.b_off = self.shape_off.copy()
        self.g_off = np.concatenate([[0], np.cumsum(self.sizes)[:-1]]).astype(np.int64)
        self.total = int(self.sizes.sum())
        self.order = np.argsort(-self.sizes * (self.D + 1), kind="stable").astype(np.int64)


def fwd_ragged(rh: RaggedHost, A, b, c, stable=False, out=None, indices=None, fast=False):
    """Per-instance loop of ``vanilla_numba`` over a packed ragged batch (OpenMP over instances).
    ``fast``: run the speed build (timed baselines) instead of the checker build."""
    A, b, c = _cc(A), _cc(b), _cc(c)
    G = np.empty(rh.total, np.complex128) if out is None else out
    order = rh.order if indices is None else np.ascontiguousarray(indices, np.int64)
    rc = (fast_lib() if fast else lib()).oracle_fwd_ragged(len(order), _ptr(rh.D), _ptr(rh.flat_shapes), _ptr(rh.shape_off), _ptr(A),
                                 _ptr(rh.a_off), _ptr(b), _ptr(rh.b_off), _ptr(c), int(bool(stable)), _ptr(G),
                                 _ptr(rh.g_off), _ptr(order))
    if rc:
        raise ValueError(f"oracle_fwd_ragged failed ({rc})")
    return G


def vjp_ragged(rh: RaggedHost, G, c, dLdG, indices=None, fast=False):
    """Per-instance loop of ``vanilla_vjp_numba`` over a packed ragged batch (``fast``: speed build)."""
    G, c, g = _cc(G), _cc(c), _cc(dLdG)
    dA = np.zeros(int((rh.D.astype(np.int64) ** 2).sum()), np.complex128)
    db = np.zeros(int(rh.D.sum()), np.complex128)
    dc = np.zeros(rh.B, np.complex128)
    order = rh.order if indices is None else np.ascontiguousarray(indices, np.int64)
    rc = (fast_lib() if fast else lib()).oracle_vjp_ragged(len(order), _ptr(rh.D), _ptr(rh.flat_shapes), _ptr(rh.shape_off), _ptr(G),
                                 _ptr(rh.g_off), _ptr(c), _ptr(g), _ptr(dA), _ptr(rh.a_off), _ptr(db),
                                 _ptr(rh.b_off), _ptr(dc), _ptr(order))
    if rc:
        raise ValueError(f"oracle_vjp_ragged failed ({rc})")
    return dA, db, dc


def autoshape(A, b, c, max_prob, max_shape, min_shape) -> np.ndarray:
    """``autoshape_numba(A, b, c, max_prob, max_shape, min_shape)`` (autoshape.py:23-154) of one
    density-matrix triple (A 2M x 2M, b 2M, c scalar) -> int64 shape of M cutoffs."""
    A, b = _cc(A), _cc(b)
    M = b.shape[0] // 2
    if A.shape != (2 * M, 2 * M) or b.shape != (2 * M,):
        raise ValueError("autoshape needs A (2M, 2M) and b (2M,)")
    c = np.array([complex(np.asarray(c).reshape(-1)[0])], np.complex128)
    out = np.zeros(M, np.int64)
    rc = lib().oracle_autoshape(M, _ptr(A), _ptr(b), _ptr(c), float(max_prob), int(max_shape), int(min_shape),
                                _ptr(out))
    if rc:
        raise ValueError(f"oracle_autoshape failed ({rc})")
    return out


def autoshape_ragged(As, bs, cs, max_prob, max_shape, min_shape):
    """``autoshape`` of many triples with their own mode counts (OpenMP over states); returns the
    list of shapes."""
    Ms = np.array([len(b) // 2 for b in bs], np.int32)
    a_off = np.concatenate([[0], np.cumsum(4 * Ms.astype(np.int64) ** 2)[:-1]]).astype(np.int64)
    b_off = np.concatenate([[0], np.cumsum(2 * Ms.astype(np.int64))[:-1]]).astype(np.int64)
    s_off = np.concatenate([[0], np.cumsum(Ms.astype(np.int64))[:-1]]).astype(np.int64)
    A = _cc(np.concatenate([np.asarray(a).ravel() for a in As]))
    b = _cc(np.concatenate([np.asarray(x).ravel() for x in bs]))
    c = _cc(np.asarray(cs).ravel())
    out = np.zeros(int(Ms.sum()), np.int64)
    rc = lib().oracle_autoshape_ragged(len(Ms), _ptr(Ms), _ptr(a_off), _ptr(b_off), _ptr(s_off), _ptr(A), _ptr(b),
                                       _ptr(c), float(max_prob), int(max_shape), int(min_shape), _ptr(out))
    if rc:
        raise ValueError(f"oracle_autoshape_ragged failed ({rc})")
    return [out[o:o + m] for o, m in zip(s_off, Ms)]


def binomial(local_cutoffs, A, b, c, max_l2, global_cutoff):
    """``binomial(local_cutoffs, A, b, c, max_l2, global_cutoff)`` (strategies/binomial.py:30-70)
    -> (G, norm, last photon number filled).  ``max_l2=None`` never stops early."""
    shape = tuple(int(s) for s in local_cutoffs)
    A, b = _cc(A), _cc(b)
    cc = np.array([complex(np.asarray(c).reshape(-1)[0])], np.complex128)
    sh = np.array(shape, np.int64)
    G = np.empty(shape, np.complex128)
    stop = ctypes.c_int64(0)
    l2 = float("inf") if max_l2 is None else float(max_l2)
    norm = lib().oracle_binomial(len(shape), _ptr(sh), _ptr(A), _ptr(b), _ptr(cc), l2, int(global_cutoff), _ptr(G),
                                 ctypes.byref(stop))
    return G, float(norm), int(stop.value)


def _diag_split(W, M, cutoffs, nb_shape):
    """One slot buffer -> the reference's (arr0, arr2, arr1010, arr1001, arr1)."""
    cut = tuple(cutoffs)
    P = int(np.prod(cut))
    nb = int(np.prod(nb_shape)) if nb_shape else 1
    W = W.reshape(-1, P * nb)
    m1 = max(M - 1, 0)
    arr0 = W[0].reshape(cut + nb_shape)
    arr2 = W[1:1 + M].reshape((M,) + cut + nb_shape)
    o = 1 + M
    if M == 1:
        arr1010 = np.zeros((1, 1, 1) + nb_shape, np.complex128)
        arr1001 = np.zeros((1, 1, 1) + nb_shape, np.complex128)
    else:
        arr1010 = W[o:o + M * m1].reshape((M, m1) + cut + nb_shape)
        arr1001 = W[o + M * m1:o + 2 * M * m1].reshape((M, m1) + cut + nb_shape)
    o += 2 * M * m1
    arr1 = W[o:o + 2 * M].reshape((2 * M,) + cut + nb_shape)
    return arr0, arr2, arr1010, arr1001, arr1


def diagonal_amps(A, B, G0, cutoffs, slots=False):
    """``hermite_multidimensional_diagonal(A, B, G0, cutoffs)`` (compactFock/inputValidation.py:61-79,
    diagonal_amps.py:140-248) on A, B already in the interleaved (mode0, mode0', mode1, ...) order
    -> (arr0, arr2, arr1010, arr1001, arr1).  B may carry a batch axis last: (2M, nb).
    ``slots=True`` returns the raw slot buffer instead."""
    A, B = _cc(A), _cc(B)
    cut = tuple(int(x) for x in cutoffs)
    M = len(cut)
    nb_shape = B.shape[1:]
    nb = int(np.prod(nb_shape)) if nb_shape else 1
    g0 = np.broadcast_to(np.asarray(G0, np.complex128), (nb,)).copy() if nb_shape else \
        np.array([complex(np.asarray(G0).reshape(-1)[0])], np.complex128)
    W = np.empty(int(lib().oracle_diagonal_slots(M)) * int(np.prod(cut)) * nb, np.complex128)
    sh = np.array(cut, np.int64)
    if lib().oracle_diagonal_amps(M, _ptr(sh), nb, _ptr(A), _ptr(np.ascontiguousarray(B.reshape(2 * M, nb))),
                                  _ptr(g0), _ptr(W)):
        raise ValueError("bad arguments")
    return W if slots else _diag_split(W, M, cut, nb_shape)


def diagonal_grad(A, B, G0, cutoffs):
    """``grad_hermite_multidimensional_diagonal`` (compactFock/inputValidation.py:82-100,
    diagonal_grad.py:261-378) -> (arr0_dG0, arr0_dA, arr0_dB) with shapes cutoffs,
    cutoffs + (2M, 2M), cutoffs + (2M,).  Runs the forward pass itself."""
    A, B = _cc(A), _cc(B)
    cut = tuple(int(x) for x in cutoffs)
    M = len(cut)
    W = diagonal_amps(A, B, G0, cut, slots=True)
    n = 2 * M
    J = np.empty(W.size * (n * n + n), np.complex128)
    sh = np.array(cut, np.int64)
    if lib().oracle_diagonal_grad(M, _ptr(sh), _ptr(A), _ptr(B), _ptr(W), _ptr(J)):
        raise ValueError("bad arguments")
    P = int(np.prod(cut))
    J0 = J[:P * (n * n + n)].reshape(P, n * n + n)
    arr0 = W[:P].reshape(cut)
    dG0 = (arr0 / np.complex128(np.asarray(G0).reshape(-1)[0])).astype(np.complex128)
    return dG0, J0[:, :n * n].reshape(cut + (n, n)), J0[:, n * n:].reshape(cut + (n,))


def fast_diagonal(A, b, c, output_cutoff, pnr_cutoffs, stable=False):
    """``fast_diagonal(A, b, c, output_cutoff, pnr_cutoffs, stable)`` (strategies/fast_diagonal.py:32-77)
    -> (pnr_1+1, ..., oc+1, oc+1)."""
    A, b = _cc(A), _cc(b)
    pnr = tuple(int(p) for p in pnr_cutoffs)
    L = len(pnr) + 1
    oc = int(output_cutoff)
    out = np.empty(tuple(p + 1 for p in pnr) + (oc + 1, oc + 1), np.complex128)
    cc = np.array([complex(np.asarray(c).reshape(-1)[0])], np.complex128)
    sh = np.array(pnr if pnr else (0,), np.int64)
    if lib().oracle_fast_diagonal(L, _ptr(sh), oc, _ptr(A), _ptr(b), _ptr(cc), int(bool(stable)), _ptr(out)):
        raise ValueError("bad arguments")
    return out


def leftover_split(W, M, cutoffs):
    """Slot buffer [slot][m][n][P'] of the leftover strategy -> the reference's (arr0, arr2, arr1010,
    arr1001, arr1) with the block axes first (singleLeftoverMode_amps.py:385-408)."""
    q, tail = int(cutoffs[0]), tuple(int(c) for c in cutoffs[1:])
    Mt = M - 1
    W = np.asarray(W).reshape(-1, q, q, *tail)
    mv = lambda x: np.moveaxis(x, 0, 2)  # (k, q, q, *tail) -> (q, q, k, *tail)
    arr0 = W[0]
    arr2 = mv(W[1:1 + Mt])
    o = 1 + Mt
    if Mt == 1:
        arr1010 = np.zeros((1, 1, 1, 1, 1), np.complex128)
        arr1001 = np.zeros((1, 1, 1, 1, 1), np.complex128)
    else:
        k = Mt * (Mt - 1)
        arr1010 = mv(W[o:o + k]).reshape((q, q, Mt, Mt - 1) + tail)
        arr1001 = mv(W[o + k:o + 2 * k]).reshape((q, q, Mt, Mt - 1) + tail)
    o += 2 * Mt * (Mt - 1)
    arr1 = mv(W[o:o + 2 * Mt])
    return arr0, arr2, arr1010, arr1001, arr1


def leftover_amps(A, B, G0, cutoffs, slots=False):
    """``hermite_multidimensional_1leftoverMode(A, B, G0, cutoffs)`` (compactFock/inputValidation.py:103-119,
    singleLeftoverMode_amps.py:385-421) on A, B in the interleaved order; cutoffs[0] is the leftover
    mode's cutoff -> (arr0, arr2, arr1010, arr1001, arr1)."""
    A, B = _cc(A), _cc(B)
    cut = tuple(int(x) for x in cutoffs)
    M = len(cut)
    q = cut[0]
    P = int(np.prod(cut[1:]))
    W = np.empty(int(lib().oracle_diagonal_slots(M - 1)) * q * q * P, np.complex128)
    g0 = np.array([complex(np.asarray(G0).reshape(-1)[0])], np.complex128)
    sh = np.array(cut, np.int64)
    if lib().oracle_leftover_amps(M, _ptr(sh), _ptr(A), _ptr(B), _ptr(g0), _ptr(W)):
        raise ValueError("bad arguments")
    return W if slots else leftover_split(W, M, cut)


def leftover_grad(A, B, G0, cutoffs):
    """``grad_hermite_multidimensional_1leftoverMode`` (inputValidation.py:122-142,
    singleLeftoverMode_grad.py:571-724) -> (arr0_dG0, arr0_dA, arr0_dB) with shapes
    (q, q, *tail), (q, q, *tail, 2M, 2M), (q, q, *tail, 2M).  Runs the forward pass itself."""
    A, B = _cc(A), _cc(B)
    cut = tuple(int(x) for x in cutoffs)
    M = len(cut)
    q, tail = cut[0], cut[1:]
    W = leftover_amps(A, B, G0, cut, slots=True)
    n = 2 * M
    nc = n * n + n
    J = np.empty(W.size * nc, np.complex128)
    sh = np.array(cut, np.int64)
    if lib().oracle_leftover_grad(M, _ptr(sh), _ptr(A), _ptr(B), _ptr(W), _ptr(J)):
        raise ValueError("bad arguments")
    P = int(np.prod(tail))
    J0 = J[:q * q * P * nc].reshape((q, q) + tail + (nc,))
    arr0 = W[:q * q * P].reshape((q, q) + tail)
    dG0 = (arr0 / np.complex128(np.asarray(G0).reshape(-1)[0])).astype(np.complex128)
    return dG0, J0[..., :n * n].reshape((q, q) + tail + (n, n)), J0[..., n * n:]


def fock_gemm(U, B):
    """FP64 CPU oracle of the Fock contraction C = U @ B (numpy -> BLAS zgemm)."""
    return np.asarray(U, np.complex128) @ np.asarray(B, np.complex128)


def einsum(subscripts, *operands):
    """FP64 CPU oracle of the Fock einsum: numpy's einsum with a contraction path (BLAS underneath),
    as math.einsum reaches opt_einsum (mrmustard/math/backend_manager.py:526-548)."""
    return np.einsum(subscripts, *[np.asarray(x, np.complex128) for x in operands], optimize=True)


def rel_err(x, ref) -> float:
    """max|x - ref| / max|ref| (the per-instance error metric used throughout the tests)."""
    x, ref = np.asarray(x), np.asarray(ref)
    den = np.abs(ref).max() if ref.size else 0.0
    return float(np.abs(x - ref).max() / den) if den > 0 else float(np.abs(x - ref).max() if x.size else 0.0)

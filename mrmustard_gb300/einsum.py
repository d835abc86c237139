"""General Fock-space einsum on the GPU.

Mirrors ``math.einsum(string, *tensors)`` (mrmustard/math/backend_manager.py:526-548, evaluated by
opt_einsum with a greedy pairwise path) and ``ArrayAnsatz.contract(other, idx1, idx2, idx_out)``
(mrmustard/physics/ansatz/array_ansatz.py:159-226: labels are str (batch) or int (core), contracted
labels are sliced to the smaller of their two dimensions, then one einsum), which ``mm_einsum``
(mrmustard/physics/mm_einsum.py:51-170) chains pair by pair.

Every pairwise contraction is planned on the host and run by the library's kernels:
operands stay torch views (slices, permutations and repeated-label diagonals are strides only)
until ``mm_tensor_permute`` makes them contiguous in [batch, free, contracted] order, labels summed
inside one operand are reduced by ``mm_tensor_sum_inner``, and the product is
``mm_zgemm_batched`` (FP64) or, with ``mode="ozaki"`` for an unbatched product, the Ozaki-split
tcgen05 GEMM of ``fock_gemm``.  complex128 throughout; numpy in -> numpy out, CUDA tensors in ->
CUDA tensors out.
"""

from __future__ import annotations

import ctypes
from collections.abc import Sequence

import numpy as np
import torch

from . import _lib
from .hermite import _stream, require_cuda

__all__ = ["einsum", "contract", "parse_subscripts"]


def _is_dev(x) -> bool:
    return isinstance(x, torch.Tensor) and x.is_cuda


def _dev_tensor(x, dev) -> torch.Tensor:
    if isinstance(x, torch.Tensor):
        t = x.detach()
        if t.dtype != torch.complex128:
            t = t.to(torch.complex128)
        return t.resolve_conj().resolve_neg().to(dev)
    return torch.from_numpy(np.ascontiguousarray(np.asarray(x, dtype=np.complex128))).to(dev)


def _i64(seq):
    seq = [int(v) for v in seq]
    return (ctypes.c_int64 * max(1, len(seq)))(*seq)


def _materialize(t: torch.Tensor) -> torch.Tensor:
    """A contiguous copy of any strided view, made by the library's permutation kernel."""
    if t.is_contiguous():
        return t
    out = torch.empty(tuple(t.shape), dtype=torch.complex128, device=t.device)
    if out.numel() == 0:
        return out
    _lib.check(_lib.load().mm_tensor_permute(t.dim(), _i64(t.shape), _i64(t.stride()), 0, t.data_ptr(),
                                             out.data_ptr(), _stream()), "mm_tensor_permute")
    return out


def _arrange(t: torch.Tensor, labels: list, order: list) -> torch.Tensor:
    """The operand with its axes in `order` (a permutation of `labels`), contiguous."""
    return _materialize(t.permute([labels.index(lab) for lab in order]))


def _diagonals(t: torch.Tensor, labels: list):
    """Take the diagonal of every repeated label (a strided view, no copy)."""
    labels = list(labels)
    while True:
        rep = next((lab for lab in labels if labels.count(lab) > 1), None)
        if rep is None:
            return t, labels
        i = labels.index(rep)
        j = labels.index(rep, i + 1)
        t = torch.diagonal(t, dim1=i, dim2=j)  # the diagonal axis goes last
        labels = [lab for k, lab in enumerate(labels) if k not in (i, j)] + [rep]


def _sum_labels(t: torch.Tensor, labels: list, summed: list):
    """Sum over `summed` labels (present only in this operand and not needed afterwards)."""
    if not summed:
        return t, labels
    kept = [lab for lab in labels if lab not in summed]
    x = _arrange(t, labels, kept + summed)
    rows = int(np.prod([x.shape[i] for i in range(len(kept))])) if kept else 1
    inner = int(np.prod([x.shape[i] for i in range(len(kept), x.dim())]))
    out = torch.empty(tuple(x.shape[:len(kept)]), dtype=torch.complex128, device=t.device)
    if rows:
        _lib.check(_lib.load().mm_tensor_sum_inner(rows, inner, x.data_ptr(), out.data_ptr(), _stream()),
                   "mm_tensor_sum_inner")
    return out, kept


def _gemm(A: torch.Tensor, B: torch.Tensor, Bt: int, M: int, N: int, K: int, mode: str) -> torch.Tensor:
    C = torch.empty((Bt, M, N), dtype=torch.complex128, device=A.device)
    if C.numel() == 0:
        return C
    if mode == "ozaki" and Bt == 1 and min(M, N, K) > 1:
        from .fock import fock_gemm

        return fock_gemm(A.reshape(M, K), B.reshape(K, N), mode="ozaki").reshape(1, M, N)
    _lib.check(_lib.load().mm_zgemm_batched(Bt, M, N, K, A.data_ptr(), M * K, B.data_ptr(), K * N, C.data_ptr(), M * N,
                                            _stream()), "mm_zgemm_batched")
    return C


def _pair(A: torch.Tensor, la: list, B: torch.Tensor, lb: list, keep: set, mode: str):
    """Contract two operands; labels in `keep` (later operands or the output) survive."""
    A, la = _sum_labels(A, la, [lab for lab in la if lab not in lb and lab not in keep])
    B, lb = _sum_labels(B, lb, [lab for lab in lb if lab not in la and lab not in keep])
    dim = {}
    for t, labels in ((A, la), (B, lb)):
        for lab, n in zip(labels, t.shape):
            if lab in dim and dim[lab] != n:
                raise ValueError(f"einsum: label {lab!r} has dimensions {dim[lab]} and {n}")
            dim[lab] = int(n)
    batch = [lab for lab in la if lab in lb and lab in keep]
    contr = [lab for lab in la if lab in lb and lab not in keep]
    fa = [lab for lab in la if lab not in lb]
    fb = [lab for lab in lb if lab not in la]
    Bt = int(np.prod([dim[lab] for lab in batch])) if batch else 1
    M = int(np.prod([dim[lab] for lab in fa])) if fa else 1
    N = int(np.prod([dim[lab] for lab in fb])) if fb else 1
    K = int(np.prod([dim[lab] for lab in contr])) if contr else 1
    A2 = _arrange(A, la, batch + fa + contr)
    B2 = _arrange(B, lb, batch + contr + fb)
    C = _gemm(A2, B2, Bt, M, N, K, mode)
    out_labels = batch + fa + fb
    return C.reshape(tuple(dim[lab] for lab in out_labels)), out_labels


def _finish(t: torch.Tensor, labels: list, output: list):
    t, labels = _sum_labels(t, labels, [lab for lab in labels if lab not in output])
    return _arrange(t, labels, list(output)) if labels != list(output) else _materialize(t)


def _run(tensors: list, label_lists: list, output: list, mode: str) -> torch.Tensor:
    ops = []
    for t, labels in zip(tensors, label_lists):
        if t.dim() != len(labels):
            raise ValueError(f"einsum: operand of rank {t.dim()} has {len(labels)} labels")
        ops.append(_diagonals(t, labels))
    while len(ops) > 1:
        # greedy pair choice: the smallest intermediate (ties: first pair), as opt_einsum's greedy path
        best = None
        for i in range(len(ops)):
            for j in range(i + 1, len(ops)):
                keep = set(output)
                for k, (_, lk) in enumerate(ops):
                    if k not in (i, j):
                        keep |= set(lk)
                li, lj = ops[i][1], ops[j][1]
                dims = {lab: n for t, lb in (ops[i], ops[j]) for lab, n in zip(lb, t.shape)}
                size = int(np.prod([dims[lab] for lab in set(li) | set(lj) if lab in keep] or [1]))
                if best is None or size < best[0]:
                    best = (size, i, j, keep)
        _, i, j, keep = best
        C, lc = _pair(ops[i][0], ops[i][1], ops[j][0], ops[j][1], keep, mode)
        ops = [op for k, op in enumerate(ops) if k not in (i, j)] + [(C, lc)]
    return _finish(ops[0][0], ops[0][1], output)


def parse_subscripts(subscripts: str, n_operands: int):
    """'ab,bc->ac' -> ([['a','b'], ['b','c']], ['a','c']); implicit output as numpy (labels seen once, sorted)."""
    s = subscripts.replace(" ", "")
    if "." in s:
        raise ValueError("einsum: ellipsis ('...') is not supported")
    if "->" in s:
        lhs, rhs = s.split("->")
        output = list(rhs)
    else:
        lhs, output = s, None
    inputs = [list(term) for term in lhs.split(",")]
    if len(inputs) != n_operands:
        raise ValueError(f"einsum: {len(inputs)} operand subscripts for {n_operands} operands")
    if output is None:
        flat = [lab for term in inputs for lab in term]
        output = sorted(lab for lab in set(flat) if flat.count(lab) == 1)
    seen = set(lab for term in inputs for lab in term)
    for lab in output:
        if lab not in seen:
            raise ValueError(f"einsum: output label {lab!r} is not in the inputs")
    if len(set(output)) != len(output):
        raise ValueError("einsum: repeated output label")
    return inputs, output


def einsum(subscripts: str, *operands, mode: str = "fp64"):
    """``math.einsum(subscripts, *operands)`` on the GPU (complex128 result)."""
    if mode not in ("fp64", "ozaki"):
        raise ValueError(f"einsum: mode must be 'fp64' or 'ozaki', not {mode!r}")
    inputs, output = parse_subscripts(subscripts, len(operands))
    dev_mode = any(_is_dev(x) for x in operands)
    dev = next((x.device for x in operands if _is_dev(x)), None) or require_cuda()
    tensors = [_dev_tensor(x, dev) for x in operands]
    out = _run(tensors, inputs, output, mode)
    return out if dev_mode else out.cpu().numpy()


def contract(array1, idx1: Sequence, array2, idx2: Sequence, idx_out: Sequence, mode: str = "fp64"):
    """``ArrayAnsatz.contract`` on two arrays: labels (str batch / int core) per axis, contracted
    labels sliced to the smaller dimension (array_ansatz.py:198-217), then the einsum."""
    dev_mode = _is_dev(array1) or _is_dev(array2)
    dev = array1.device if _is_dev(array1) else array2.device if _is_dev(array2) else require_cuda()
    a1, a2 = _dev_tensor(array1, dev), _dev_tensor(array2, dev)
    idx1, idx2, idx_out = list(idx1), list(idx2), list(idx_out)
    if len(idx1) != a1.dim():
        raise ValueError(f"expected len(idx1)={a1.dim()} got {len(idx1)}")
    if len(idx2) != a2.dim():
        raise ValueError(f"expected len(idx2)={a2.dim()} got {len(idx2)}")
    if not set(idx_out).issubset(set(idx1) | set(idx2)):
        raise ValueError("Output labels must be present in input labels.")
    s1 = [slice(None)] * len(idx1)
    s2 = [slice(None)] * len(idx2)
    for label in set(idx1) & set(idx2):
        p1, p2 = idx1.index(label), idx2.index(label)
        d = min(a1.shape[p1], a2.shape[p2])
        s1[p1], s2[p2] = slice(0, d), slice(0, d)
    out = _run([a1[tuple(s1)], a2[tuple(s2)]], [idx1, idx2], idx_out, mode)
    return out if dev_mode else out.cpu().numpy()

"""Ragged batches: thousands of triples with their own mode count and cutoffs.

The reference batches only triples that share D and shape
(mrmustard/math/lattice/strategies/vanilla/batch.py:27-61,
mrmustard/math/backend_manager.py:683-720); a ragged set is a Python loop of
``vanilla_numba`` / ``vanilla_vjp_numba`` calls there.  ``RaggedBatch`` plans the set once on
the host (cost-sorted instance schedule, VJP work items), uploads the plan into a persistent
device workspace, and then runs the forward / VJP of every instance in a few launches that
can be captured in one CUDA graph.  Per instance, results equal ``vanilla_numba`` /
``vanilla_vjp_numba`` of that instance.

A ``RaggedBatch`` owns one workspace: use it from one stream at a time.
"""

from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from .hermite import Workspace, _stream, raw, require_cuda
from .settings import settings

__all__ = ["RaggedBatch", "plan_offsets"]


def plan_offsets(shapes):
    """Host-side plan of a ragged set (no device needed): (g_off, a_off, b_off, total) of the flat
    packing the library uses for these shapes, from mm_ragged_plan_offsets."""
    lib = _lib.load()
    shapes = [tuple(int(x) for x in s) for s in shapes]
    B = len(shapes)
    D = np.array([len(s) for s in shapes], np.int32)
    flat = np.array([x for s in shapes for x in s] or [0], np.int64)
    plan = ctypes.c_void_p()
    _lib.check(lib.mm_ragged_plan_create(B, D.ctypes.data, flat.ctypes.data, ctypes.byref(plan)),
               "mm_ragged_plan_create")
    try:
        offs = [np.zeros(B, np.int64) for _ in range(3)]
        _lib.check(lib.mm_ragged_plan_offsets(plan, *(o.ctypes.data for o in offs)), "mm_ragged_plan_offsets")
        total = int(lib.mm_ragged_plan_amplitudes(plan))
    finally:
        lib.mm_ragged_plan_destroy(plan)
    return offs[0], offs[1], offs[2], total


class RaggedBatch:
    def __init__(self, shapes, device=None, team_min_amps: int | None = None, vjp_item_amps: int | None = None):
        lib = _lib.load()
        self.device = torch.device(device) if device is not None else require_cuda()
        self.shapes = [tuple(int(x) for x in s) for s in shapes]
        self.B = len(self.shapes)
        self.D = np.array([len(s) for s in self.shapes], np.int32)
        flat = np.array([x for s in self.shapes for x in s] or [0], np.int64)
        plan = ctypes.c_void_p()
        _lib.check(lib.mm_ragged_plan_create(self.B, self.D.ctypes.data, flat.ctypes.data, ctypes.byref(plan)),
                   "mm_ragged_plan_create")
        self._plan = plan
        if team_min_amps is not None or vjp_item_amps is not None:
            _lib.check(lib.mm_ragged_plan_set_tuning(plan, int(team_min_amps or 0), int(vjp_item_amps or 65536)),
                       "mm_ragged_plan_set_tuning")
        self.g_off = np.zeros(self.B, np.int64)
        self.a_off = np.zeros(self.B, np.int64)
        self.b_off = np.zeros(self.B, np.int64)
        _lib.check(lib.mm_ragged_plan_offsets(plan, self.g_off.ctypes.data, self.a_off.ctypes.data,
                                              self.b_off.ctypes.data), "mm_ragged_plan_offsets")
        self.sizes = np.array([int(np.prod(s)) for s in self.shapes], np.int64)
        self.global_index = np.arange(self.B, dtype=np.int64)
        self.total = int(lib.mm_ragged_plan_amplitudes(plan))
        self.n_a = int((self.D.astype(np.int64) ** 2).sum())
        self.n_b = int(self.D.sum())
        self.tuning = {"team_min_amps": int(team_min_amps or 0), "vjp_item_amps": int(vjp_item_amps or 65536),
                       "team_cluster": 8}
        self._upload()

    @classmethod
    def shard(cls, shapes, rank: int, world: int, device=None, **tuning) -> "RaggedBatch":
        """The share of rank `rank` (of `world`) of one ragged batch of `shapes`.

        Instances are independent, so ranks split them with no collective: a greedy
        longest-processing-time split of the per-instance cost (``shard.shard_instances``).
        The returned batch holds this rank's instances in increasing global order;
        ``global_index[k]`` is the position in `shapes` of its instance k."""
        from .shard import instance_costs, shard_instances

        shapes = [tuple(int(x) for x in s) for s in shapes]
        if not 0 <= rank < max(world, 1):
            raise ValueError(f"rank {rank} outside world size {world}")
        local = shard_instances(instance_costs(shapes), world)[rank] if world > 1 else list(range(len(shapes)))
        rb = cls([shapes[k] for k in local], device=device, **tuning)
        rb.global_index = np.asarray(local, np.int64)
        return rb

    def _upload(self):
        lib = _lib.load()
        self.ws = Workspace(lib.mm_ragged_plan_workspace_bytes(self._plan), self.device)
        _lib.check(lib.mm_ragged_plan_upload(self._plan, self.ws.ptr, self.ws.nbytes, _stream()),
                   "mm_ragged_plan_upload")

    def retune(self, team_min_amps: int | None = None, vjp_item_amps: int | None = None,
               team_cluster: int | None = None):
        """Re-plan with new schedule settings (see mm_ragged_plan_set_tuning / _set_team_size)
        and upload the new plan; results are unchanged, only the work split differs."""
        lib = _lib.load()
        t = dict(self.tuning)
        if team_min_amps is not None:
            t["team_min_amps"] = int(team_min_amps)
        if vjp_item_amps is not None:
            t["vjp_item_amps"] = int(vjp_item_amps)
        if team_cluster is not None:
            t["team_cluster"] = int(team_cluster)
        _lib.check(lib.mm_ragged_plan_set_tuning(self._plan, t["team_min_amps"], t["vjp_item_amps"]),
                   "mm_ragged_plan_set_tuning")
        _lib.check(lib.mm_ragged_plan_set_team_size(self._plan, t["team_cluster"]), "mm_ragged_plan_set_team_size")
        self.tuning = t
        torch.cuda.synchronize(self.device)
        self._upload()
        return t

    def set_copy_split(self, eighths: int) -> None:
        """Instances k with k % 8 < eighths get their copy of G (``G_copy``) from the forward,
        the others from the VJP (mm_ragged_plan_set_copy_split; 0 = all from the VJP)."""
        _lib.check(_lib.load().mm_ragged_plan_set_copy_split(self._plan, int(eighths)), "mm_ragged_plan_set_copy_split")
        self.copy_split = int(eighths)

    def __del__(self):
        plan = getattr(self, "_plan", None)
        if plan is not None and plan.value:
            try:
                _lib.load().mm_ragged_plan_destroy(plan)
            except Exception:  # interpreter shutdown
                pass
            self._plan = None

    # ------------------------------------------------------------ packing
    def pack(self, As, bs, cs):
        """Pack per-instance (A_k, b_k, c_k) into the flat device layout of the plan."""
        A = np.concatenate([np.asarray(a, np.complex128).reshape(-1) for a in As]) if self.B else np.zeros(0, complex)
        b = np.concatenate([np.asarray(x, np.complex128).reshape(-1) for x in bs]) if self.B else np.zeros(0, complex)
        c = np.asarray(cs, np.complex128).reshape(-1)
        to = lambda x: torch.from_numpy(np.ascontiguousarray(x)).to(self.device)  # noqa: E731
        return to(A), to(b), to(c)

    def unpack(self, G_flat):
        """Per-instance views of a flat result (tensor or array)."""
        return [G_flat[o:o + n].reshape(s) for o, n, s in zip(self.g_off, self.sizes, self.shapes)]

    def unpack_grads(self, dA, db):
        dAs = [dA[o:o + d * d].reshape(d, d) for o, d in zip(self.a_off, self.D)]
        dbs = [db[o:o + d] for o, d in zip(self.b_off, self.D)]
        return dAs, dbs

    # ------------------------------------------------------------ compute
    def _check(self, where):
        if settings.CHECK_DEVICE_STATUS and not torch.cuda.is_current_stream_capturing():
            self.ws.check_status(where)

    def forward(self, A, b, c, stable: bool = False, out=None, G_copy=None):
        """Flat G of every instance (device tensor of ``self.total`` complex128).

        ``G_copy`` (optional, e.g. a pinned host tensor of ``self.total``) receives the forward's
        share of a copy of G (see ``set_copy_split``); ``vjp(..., G_copy=)`` writes the rest."""
        lib = _lib.load()
        A, b, c = raw(A), raw(b), raw(c)
        G = out if out is not None else torch.empty(self.total, dtype=torch.complex128, device=self.device)
        if G_copy is not None:
            if G_copy.dtype != torch.complex128 or not G_copy.is_contiguous() or G_copy.numel() != self.total:
                raise ValueError("G_copy must be a contiguous complex128 tensor of self.total elements")
        _lib.check(lib.mm_ragged_fwd_copy_g(self._plan, A.data_ptr(), b.data_ptr(), c.data_ptr(), int(bool(stable)),
                                            G.data_ptr(), G_copy.data_ptr() if G_copy is not None else None,
                                            self.ws.ptr, self.ws.nbytes, _stream()), "mm_ragged_fwd")
        self._check("ragged forward")
        return G

    def vjp(self, G, c, dLdG, out=None, G_copy=None):
        """(dA_flat, db_flat, dc) of every instance (holomorphic VJP, as vanilla_vjp_numba).

        ``dLdG`` may be a pinned host tensor: the kernels then read it through the host link.
        ``G_copy`` (optional, e.g. a pinned host tensor of ``self.total``) receives a copy of G
        written by the VJP kernels from the values they load: every instance outside the forward's
        share (``set_copy_split``; all of them by default)."""
        lib = _lib.load()
        G, c, dLdG = raw(G), raw(c), raw(dLdG)
        if G_copy is not None:
            if G_copy.dtype != torch.complex128 or not G_copy.is_contiguous() or G_copy.numel() != self.total:
                raise ValueError("G_copy must be a contiguous complex128 tensor of self.total elements")
        if out is None:
            dA = torch.empty(self.n_a, dtype=torch.complex128, device=self.device)
            db = torch.empty(self.n_b, dtype=torch.complex128, device=self.device)
            dc = torch.empty(self.B, dtype=torch.complex128, device=self.device)
        else:
            dA, db, dc = out
        _lib.check(lib.mm_ragged_vjp_copy_g(self._plan, G.data_ptr(), c.data_ptr(), dLdG.data_ptr(), dA.data_ptr(),
                                            db.data_ptr(), dc.data_ptr(), G_copy.data_ptr() if G_copy is not None else None,
                                            self.ws.ptr, self.ws.nbytes, _stream()), "mm_ragged_vjp")
        self._check("ragged vjp")
        return dA, db, dc

    def _chunks(self, n_chunks: int):
        """Contiguous instance ranges with about equal amplitude counts, each with its own plan
        (same schedule settings) whose packed buffers are slices of this batch's buffers."""
        key = int(n_chunks)
        cache = getattr(self, "_chunk_cache", {})
        if key in cache:
            return cache[key]
        g_pref = np.concatenate([[0], np.cumsum(self.sizes)])
        a_pref = np.concatenate([[0], np.cumsum(self.D.astype(np.int64) ** 2)])
        b_pref = np.concatenate([[0], np.cumsum(self.D.astype(np.int64))])
        if not (np.array_equal(self.g_off, g_pref[:-1]) and np.array_equal(self.a_off, a_pref[:-1])
                and np.array_equal(self.b_off, b_pref[:-1])):
            raise RuntimeError("ragged packing is not in instance order; chunked steps need it")
        cuts = [0]
        for k in range(1, key):
            cuts.append(int(np.searchsorted(g_pref, g_pref[-1] * k / key)))
        cuts.append(self.B)
        cuts = sorted(set(cuts))
        chunks = []
        for i0, i1 in zip(cuts[:-1], cuts[1:]):
            if i1 <= i0:
                continue
            sub = RaggedBatch(self.shapes[i0:i1], device=self.device, team_min_amps=self.tuning["team_min_amps"],
                              vjp_item_amps=self.tuning["vjp_item_amps"])
            if self.tuning["team_cluster"] != sub.tuning["team_cluster"]:
                sub.retune(team_cluster=self.tuning["team_cluster"])
            chunks.append((i0, i1, int(g_pref[i0]), int(g_pref[i1]), int(a_pref[i0]), int(a_pref[i1]),
                           int(b_pref[i0]), int(b_pref[i1]), sub))
        cache[key] = chunks
        self._chunk_cache = cache
        return chunks

    def step_host(self, A_h, b_h, c_h, dLdG_h, G_h, dA_h, db_h, dc_h, stable: bool = False,
                  cotangent: str = "fused", chunks: int = 2, copy_split: int = 2):
        """One forward + VJP step with every input and output in pinned host memory.

        A, b, c (small) are copied to the device and the forward writes G in device memory.  The
        two large tensors (dL/dG in, G out) move in one of four ways, all overlapped with compute
        (the default, ``"fused"`` with ``copy_split=2``, measured fastest); in the first three, G
        goes back by copy engine on a second stream while the VJP runs:

        * ``"prefetch"``: copied into device memory on the second stream while the forward runs;
        * ``"zero_copy"``: read by the VJP kernels straight from the pinned host buffer over the
          host link (the GPU addresses pinned host memory directly; no device copy is kept);
        * ``"pipelined"``: copied into device memory in ``chunks`` instance ranges on a third stream
          while the forward runs, the VJP of each range starting as soon as its part has arrived,
          so the cotangent upload, the G download and the kernels overlap;
        * ``"fused"``: read zero-copy as in ``"zero_copy"``, and G is written to ``G_h`` by the VJP
          kernels themselves (``mm_ragged_vjp_copy_g``) instead of a copy-engine transfer, so both
          directions of the host link are driven by the kernels; with ``copy_split`` = s > 0 the
          forward kernels write the G of the instances k with k % 8 < s (``mm_ragged_fwd_copy_g``),
          so the host link also carries G while the forward runs (s = 2 measured best on the
          4096-triple bench batch: 45.0 against 46.3 ms with s = 0).

        Enqueued asynchronously on the current stream; synchronise before reading the outputs.
        """
        if cotangent not in ("prefetch", "zero_copy", "pipelined", "fused"):
            raise ValueError("cotangent must be 'prefetch', 'zero_copy', 'pipelined' or 'fused'")
        if cotangent == "pipelined":
            return self._step_host_pipelined(A_h, b_h, c_h, dLdG_h, G_h, dA_h, db_h, dc_h, stable, chunks)
        if cotangent == "fused":
            # the split applies to this step's launches only (read when they are enqueued)
            prev = getattr(self, "copy_split", 0)
            if copy_split != prev:
                self.set_copy_split(copy_split)
            try:
                return self._step_host_fused(A_h, b_h, c_h, dLdG_h, G_h, dA_h, db_h, dc_h, stable)
            finally:
                if copy_split != prev:
                    self.set_copy_split(prev)
        cur = torch.cuda.current_stream(self.device)
        if getattr(self, "_dev_bufs", None) is None:
            mk = lambda n: torch.empty(n, dtype=torch.complex128, device=self.device)  # noqa: E731
            self._dev_bufs = (mk(self.n_a), mk(self.n_b), mk(self.B), mk(self.total),
                              (mk(self.n_a), mk(self.n_b), mk(self.B)))
            self._copy_stream = torch.cuda.Stream(device=self.device)
        if cotangent == "prefetch" and getattr(self, "_g_dev", None) is None:
            self._g_dev = torch.empty(self.total, dtype=torch.complex128, device=self.device)
        A, b, c, G, grads = self._dev_bufs
        for hbuf in (dLdG_h, G_h):
            if hbuf.is_cuda or not hbuf.is_pinned():
                raise ValueError("dLdG_h and G_h must be pinned host tensors")
        cs = self._copy_stream
        cs.wait_stream(cur)  # the previous step's readers of G and of the cotangent buffer are done
        if cotangent == "prefetch":
            with torch.cuda.stream(cs):
                self._g_dev.copy_(dLdG_h, non_blocking=True)
                g_ready = torch.cuda.Event()
                g_ready.record(cs)
        A.copy_(A_h, non_blocking=True)
        b.copy_(b_h, non_blocking=True)
        c.copy_(c_h, non_blocking=True)
        self.forward(A, b, c, stable, out=G)
        fwd_done = torch.cuda.Event()
        fwd_done.record(cur)
        with torch.cuda.stream(cs):
            cs.wait_event(fwd_done)
            G_h.copy_(G, non_blocking=True)
        if cotangent == "prefetch":
            cur.wait_event(g_ready)
            g = self._g_dev
        else:
            g = dLdG_h
        self.vjp(G, c, g, out=grads)
        dA_h.copy_(grads[0], non_blocking=True)
        db_h.copy_(grads[1], non_blocking=True)
        dc_h.copy_(grads[2], non_blocking=True)
        cur.wait_stream(cs)
        return G_h, (dA_h, db_h, dc_h)

    def _step_host_fused(self, A_h, b_h, c_h, dLdG_h, G_h, dA_h, db_h, dc_h, stable):
        if getattr(self, "_dev_bufs", None) is None:
            mk = lambda n: torch.empty(n, dtype=torch.complex128, device=self.device)  # noqa: E731
            self._dev_bufs = (mk(self.n_a), mk(self.n_b), mk(self.B), mk(self.total),
                              (mk(self.n_a), mk(self.n_b), mk(self.B)))
            self._copy_stream = torch.cuda.Stream(device=self.device)
        for hbuf in (dLdG_h, G_h):
            if hbuf.is_cuda or not hbuf.is_pinned():
                raise ValueError("dLdG_h and G_h must be pinned host tensors")
        A, b, c, G, grads = self._dev_bufs
        A.copy_(A_h, non_blocking=True)
        b.copy_(b_h, non_blocking=True)
        c.copy_(c_h, non_blocking=True)
        self.forward(A, b, c, stable, out=G, G_copy=G_h if getattr(self, "copy_split", 0) else None)
        self.vjp(G, c, dLdG_h, out=grads, G_copy=G_h)
        dA_h.copy_(grads[0], non_blocking=True)
        db_h.copy_(grads[1], non_blocking=True)
        dc_h.copy_(grads[2], non_blocking=True)
        return G_h, (dA_h, db_h, dc_h)

    def _step_host_pipelined(self, A_h, b_h, c_h, dLdG_h, G_h, dA_h, db_h, dc_h, stable, n_chunks):
        cur = torch.cuda.current_stream(self.device)
        if getattr(self, "_dev_bufs", None) is None:
            mk = lambda n: torch.empty(n, dtype=torch.complex128, device=self.device)  # noqa: E731
            self._dev_bufs = (mk(self.n_a), mk(self.n_b), mk(self.B), mk(self.total),
                              (mk(self.n_a), mk(self.n_b), mk(self.B)))
            self._copy_stream = torch.cuda.Stream(device=self.device)
        if getattr(self, "_g_dev", None) is None:
            self._g_dev = torch.empty(self.total, dtype=torch.complex128, device=self.device)
        if getattr(self, "_up_stream", None) is None:
            self._up_stream = torch.cuda.Stream(device=self.device)
        for hbuf in (dLdG_h, G_h):
            if hbuf.is_cuda or not hbuf.is_pinned():
                raise ValueError("dLdG_h and G_h must be pinned host tensors")
        A, b, c, G, (dA, db, dc) = self._dev_bufs
        parts = self._chunks(n_chunks)
        up, down = self._up_stream, self._copy_stream
        up.wait_stream(cur)    # the previous step's VJPs have read the device cotangent
        down.wait_stream(cur)  # and nothing still reads G
        ready = []
        with torch.cuda.stream(up):
            for (_, _, g0, g1, *_rest) in parts:
                self._g_dev[g0:g1].copy_(dLdG_h[g0:g1], non_blocking=True)
                ev = torch.cuda.Event()
                ev.record(up)
                ready.append(ev)
        A.copy_(A_h, non_blocking=True)
        b.copy_(b_h, non_blocking=True)
        c.copy_(c_h, non_blocking=True)
        self.forward(A, b, c, stable, out=G)
        fwd_done = torch.cuda.Event()
        fwd_done.record(cur)
        with torch.cuda.stream(down):
            down.wait_event(fwd_done)
            G_h.copy_(G, non_blocking=True)
        for ev, (i0, i1, g0, g1, a0, a1, b0, b1, sub) in zip(ready, parts):
            cur.wait_event(ev)
            sub.vjp(G[g0:g1], c[i0:i1], self._g_dev[g0:g1], out=(dA[a0:a1], db[b0:b1], dc[i0:i1]))
        dA_h.copy_(dA, non_blocking=True)
        db_h.copy_(db, non_blocking=True)
        dc_h.copy_(dc, non_blocking=True)
        cur.wait_stream(down)
        return G_h, (dA_h, db_h, dc_h)

    def capture(self, A, b, c, dLdG, stable: bool = False, warmup: int = 1):
        """Capture forward + VJP on static buffers into one CUDA graph.

        Returns (graph, G, (dA, db, dc)); ``graph.replay()`` recomputes them from the
        current contents of A, b, c and dLdG.
        """
        G = torch.empty(self.total, dtype=torch.complex128, device=self.device)
        grads = (torch.empty(self.n_a, dtype=torch.complex128, device=self.device),
                 torch.empty(self.n_b, dtype=torch.complex128, device=self.device),
                 torch.empty(self.B, dtype=torch.complex128, device=self.device))
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            with settings(CHECK_DEVICE_STATUS=False):
                for _ in range(warmup):
                    self.forward(A, b, c, stable, out=G)
                    self.vjp(G, c, dLdG, out=grads)
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with settings(CHECK_DEVICE_STATUS=False):
            with torch.cuda.graph(g):
                self.forward(A, b, c, stable, out=G)
                self.vjp(G, c, dLdG, out=grads)
        return g, G, grads

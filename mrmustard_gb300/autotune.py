"""Autotuner of the ragged-batch schedule.

A ragged plan has three schedule settings that change speed but never results:

* ``team_min_amps`` -- instances with at least this many amplitudes run their forward on a
  thread-block cluster instead of a single CTA (0 = the plan's automatic threshold);
* ``team_cluster`` -- CTAs per cluster team (1, 2, 4, 8, 16);
* ``vjp_item_amps`` -- target amplitudes per VJP work item.

``autotune(rb, A, b, c, dLdG)`` times candidate settings on the batch itself (CUDA events on the
current stream, forward and VJP separately, median of a few repeats), applies the fastest and
caches the choice in a JSON file keyed by the batch's shape multiset and the GPU name
(``MM_GB300_AUTOTUNE_CACHE`` or ``~/.cache/mrmustard_gb300/autotune.json``).
"""

from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

import torch

from . import _lib
from .settings import settings

TEAM_MIN = (0, 1 << 17, 1 << 18, 1 << 19, 1 << 20)
TEAM_CLUSTER = (4, 8, 16)
VJP_ITEMS = (1 << 14, 1 << 15, 1 << 16, 1 << 17, 1 << 18, 1 << 19)


def cache_path() -> Path:
    p = os.environ.get("MM_GB300_AUTOTUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "mrmustard_gb300" / "autotune.json"


def signature(rb) -> str:
    h = hashlib.sha1()
    for s in sorted(rb.shapes):
        h.update(repr(s).encode())
    h.update(torch.cuda.get_device_name(rb.device).encode())
    return h.hexdigest()[:16]


def _time(fn, reps: int) -> float:
    stream = torch.cuda.current_stream()
    fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def _load_cache(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def autotune(rb, A, b, c, dLdG, reps: int = 3, use_cache: bool = True) -> dict:
    """Pick and apply the fastest schedule for ``rb``; returns the chosen settings and timings."""
    path = cache_path()
    key = signature(rb)
    if use_cache:
        hit = _load_cache(path).get(key)
        if hit:
            rb.retune(hit["team_min_amps"], hit["vjp_item_amps"], hit["team_cluster"])
            return dict(hit, cached=True)
    G = torch.empty(rb.total, dtype=torch.complex128, device=rb.device)
    grads = (torch.empty(rb.n_a, dtype=torch.complex128, device=rb.device),
             torch.empty(rb.n_b, dtype=torch.complex128, device=rb.device),
             torch.empty(rb.B, dtype=torch.complex128, device=rb.device))
    best = None
    fwd_times = {}
    with settings(CHECK_DEVICE_STATUS=False):
        for cl in TEAM_CLUSTER:
            for tm in TEAM_MIN:
                try:
                    rb.retune(team_min_amps=tm, team_cluster=cl)
                    t = _time(lambda: rb.forward(A, b, c, out=G), reps)
                except _lib.MMError:  # e.g. a cluster size this GPU cannot schedule
                    continue
                fwd_times[f"{cl}/{tm}"] = t
                if best is None or t < best[0]:
                    best = (t, tm, cl)
        t_fwd, tm, cl = best
        rb.retune(team_min_amps=tm, team_cluster=cl)
        rb.forward(A, b, c, out=G)
        vjp_times = {}
        best_v = None
        for it in VJP_ITEMS:
            rb.retune(vjp_item_amps=it)
            t = _time(lambda: rb.vjp(G, c, dLdG, out=grads), reps)
            vjp_times[str(it)] = t
            if best_v is None or t < best_v[0]:
                best_v = (t, it)
        rb.retune(vjp_item_amps=best_v[1])
    rb.ws.check_status("autotune")
    choice = {"team_min_amps": tm, "team_cluster": cl, "vjp_item_amps": best_v[1],
              "forward_ms": t_fwd, "vjp_ms": best_v[0]}
    if use_cache:
        try:
            path.parent.mkdir(parents=True, exist_ok=True)
            data = _load_cache(path)
            data[key] = choice
            path.write_text(json.dumps(data, indent=1))
        except OSError:
            pass
    return dict(choice, cached=False, forward_candidates_ms=fwd_times, vjp_candidates_ms=vjp_times)

"""Benchmark of the Gaussian->Fock hot path on one GB300 (or N, one process per GPU).

Workload (the batched configuration the headline metric is quoted on): 4096 triples with
D ~ U{1..4} modes, per-mode cutoff ~ U{5..40}, A = Q diag(s) Q^T (Q Haar unitary,
s ~ U(0, 0.8)), b complex normal sigma = 0.3, c = 1, complex128, seeded per instance;
upstream dL/dG complex normal.  One step = forward + VJP of every instance (one CUDA-graph
replay of the ragged plan).  Synthetic data of exactly that shape; inputs (G, dL/dG: GBs)
are far larger than L2, so no flush is needed between steps.

Arms: ``--impl gb300`` (default) times the CUDA library; ``--impl reference`` times the CPU
oracle (C restatement of the reference's numba strategies, OpenMP over instances on every
host core) on the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Fock amplitudes/s fwd+VJP (c128, <=1e-12 rel) batched vs plain, 1 GB300"
UNIT = "amplitudes/s"
N_INST = 4096
VJP_DRAM_BYTES_PER_AMP = 52.1  # dram read + write per amplitude, ncu capture of the VJP items kernel
ERR_TOL = 1e-12                # max |x - oracle| / max |oracle| per instance, G and every gradient
MIN_BATCHED_OVER_PLAIN = 10.0  # one batched launch vs a loop of per-instance launches


# ------------------------------------------------------------------ workload
BASE_SEED = 20260000


def _instance(base_seed: int, k: int, with_triple: bool):
    rng = np.random.default_rng(base_seed + k)
    D = int(rng.integers(1, 5))
    shape = tuple(int(x) for x in rng.integers(5, 41, D))
    if not with_triple:
        return shape, None, None
    from scipy.stats import unitary_group

    if D == 1:
        Q = np.exp(1j * rng.uniform(0, 2 * np.pi, (1, 1)))
    else:
        Q = unitary_group.rvs(D, random_state=rng)
    s = rng.uniform(0.0, 0.8, D)
    A = (Q * s) @ Q.T
    b = 0.3 * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(2)
    return shape, A.astype(np.complex128), b.astype(np.complex128)


def workload_shapes(base_seed: int, n: int):
    """Shapes of instances 0..n-1 (the first draws of each instance's generator)."""
    return [_instance(base_seed, k, False)[0] for k in range(n)]


def make_workload(base_seed: int, n: int = N_INST, indices=None):
    """Per-instance seeded triples: (shapes, As, bs, cs) of instances `indices` (default 0..n-1)."""
    idx = range(n) if indices is None else indices
    shapes, As, bs = [], [], []
    for k in idx:
        shape, A, b = _instance(base_seed, int(k), True)
        shapes.append(shape)
        As.append(A)
        bs.append(b)
    cs = np.ones(len(shapes), np.complex128)
    return shapes, As, bs, cs


def workload_config(n_instances: int, amplitudes: int, world: int) -> dict:
    """The workload both arms run (identical dict in the GB300 and the reference line)."""
    return {"workload": f"ragged batch: {n_instances} triples, D~U{{1..4}}, cutoff~U{{5..40}}, Takagi A "
                        "s~U(0,0.8), b sigma 0.3, c=1, fwd+VJP per step",
            "instances": n_instances, "amplitudes": int(amplitudes),
            "l2": "inputs larger than L2 (G, dLdG ~4.4 GB per 4096 triples)",
            "parallelism": (f"instances sharded over {world} ranks (cost-balanced, no collective)" if world > 1
                            else "one GPU")}


def fp64_ops(shape):
    """FP64 pipe instructions (DFMA/DMUL each 1) of the forward and the VJP kernels for one shape."""
    C = np.array(shape, np.float64)
    n = float(np.prod(C))
    D = len(shape)
    fwd = 0.0
    for i in range(D):
        inner = float(np.prod(C[i + 1:]))
        lvl = (C[i] - 1) * inner
        fwd += 6 * lvl + 4 * max(C[i] - 2, 0) * inner
        for j in range(i + 1, D):
            fwd += 4 * (C[i] - 1) * (C[j] - 1) * inner / C[j]
    N1 = lambda i: n * (C[i] - 1) / C[i]  # noqa: E731
    N2 = lambda i: n * max(C[i] - 2, 0) / C[i]  # noqa: E731
    N11 = lambda i, j: n * (C[i] - 1) * (C[j] - 1) / (C[i] * C[j])  # noqa: E731
    vjp = 4 * n + 6 * N1(0) + 6 * N2(0) + sum(4 * N11(0, j) for j in range(1, D))
    for i in range(1, D):
        vjp += 4 * N1(i) + 4 * N2(i) + sum(4 * N11(i, j) for j in range(i + 1, D))
    return fwd, vjp


# ------------------------------------------------------------------ helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), ws


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        if self.proc is None or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        for r in rows:
            for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"),
                                 r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        loaded = sorted(sm)[len(sm) // 4:] if len(sm) > 4 else sm  # ignore the ramp at the start
        return {"sm_mhz": float(np.median(loaded)) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def measured_bf16_tflops():
    """Dense BF16 burst throughput of this part (cuBLAS, measured), else the earlier GB300 figure."""
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        if "bf16_tflops" in d:
            return float(d["bf16_tflops"]), "measured"
    return 1900.0, "fallback"


# ------------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return 0
    import oracle

    oracle.build()
    shapes, As, bs, cs = make_workload(BASE_SEED, args.instances * world)
    rh = oracle.RaggedHost(shapes)
    A = np.concatenate([a.ravel() for a in As])
    b = np.concatenate(bs)
    rng = np.random.default_rng(7)
    g = (rng.standard_normal(rh.total) + 1j * rng.standard_normal(rh.total)).astype(np.complex128)
    G = np.empty(rh.total, np.complex128)

    # bounded sample: a fixed subset of instances (cost-weighted stride) so a step takes a few seconds
    t0 = time.perf_counter()
    oracle.fwd_ragged(rh, A, b, cs, out=G, fast=True)
    oracle.vjp_ragged(rh, G, cs, g, fast=True)
    full_s = time.perf_counter() - t0
    frac = min(1.0, 4.0 / full_s) if full_s > 0 else 1.0
    idx = rh.order[:: max(1, int(round(1 / frac)))] if frac < 1 else rh.order
    amps = int(rh.sizes[idx].sum())
    for _ in range(args.warmup):
        oracle.fwd_ragged(rh, A, b, cs, out=G, indices=idx, fast=True)
        oracle.vjp_ragged(rh, G, cs, g, indices=idx, fast=True)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.fwd_ragged(rh, A, b, cs, out=G, indices=idx, fast=True)
        oracle.vjp_ragged(rh, G, cs, g, indices=idx, fast=True)
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    value = amps / t
    sample = (f"{len(idx)} of {len(shapes)} instances ({amps} of {rh.total} amplitudes), fwd+VJP per step"
              if len(idx) < len(shapes) else f"all {len(shapes)} instances ({amps} amplitudes), fwd+VJP per step")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic", "impl": "reference",
        "config": workload_config(len(shapes), int(rh.total), world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
                         "build": "gcc " + " ".join(oracle.FAST_FLAGS) + " -fopenmp (no -march flags)",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GB300 arm
def run_gb300(args, rank, local_rank, world):
    import torch

    import mrmustard_gb300 as mm
    from mrmustard_gb300 import _lib

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)

    # --- workload: one batch of 4096 x world triples, split over the ranks by cost (weak scaling:
    #     about 4096 triples' work per GPU; no collective on the data path)
    n_global = args.instances * world
    shapes_all = workload_shapes(BASE_SEED, n_global)
    total_all = int(sum(int(np.prod(s)) for s in shapes_all))
    rb = mm.RaggedBatch.shard(shapes_all, rank, world, device=dev)
    shapes, As, bs, cs = make_workload(BASE_SEED, indices=rb.global_index)
    A, b, c = rb.pack(As, bs, cs)
    gen = torch.Generator(device=dev)
    gen.manual_seed(7 + rank)
    g = torch.complex(torch.randn(rb.total, generator=gen, device=dev, dtype=torch.float64),
                      torch.randn(rb.total, generator=gen, device=dev, dtype=torch.float64))
    total = rb.total

    def barrier():
        if pg is not None:
            pg.barrier()

    # --- one status-checked forward + VJP before anything is timed (device status word read back);
    #     the results are compared with the oracle in the CPU-baseline leg
    with mm.settings(CHECK_DEVICE_STATUS=True):
        G_chk = rb.forward(A, b, c)
        rb.vjp(G_chk, c, g)
    del G_chk

    # --- schedule autotuning on this batch (outside the timed region)
    tuned = mm.autotune(rb, A, b, c, g, use_cache=False) if not args.no_autotune else None

    # --- one CUDA graph: forward + VJP of every instance
    n_before = int(lib.mm_launch_count())
    graph, G, grads = rb.capture(A, b, c, g, warmup=1)
    # rb.capture runs forward + VJP once eagerly (warm-up) and once under capture
    launches_per_step = (int(lib.mm_launch_count()) - n_before) // 2
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()

    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        barrier()
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            graph.replay()
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = ev0.elapsed_time(ev1) / args.steps
    if pg is not None:
        t = torch.tensor([ms], device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    value = total_all / (ms * 1e-3)
    clocks = clk.summary()

    # --- device status after the timed region
    rb.ws.check_status("timed region")

    # --- per-kernel timing (eager, same stream) for the roofline
    def time_eager(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    with mm.settings(CHECK_DEVICE_STATUS=False):
        t_fwd = time_eager(lambda: rb.forward(A, b, c, out=G))
        t_vjp = time_eager(lambda: rb.vjp(G, c, g, out=grads))
    fwd_ops = vjp_ops = 0.0
    for sh in shapes:
        f_, v_ = fp64_ops(sh)
        fwd_ops += f_
        vjp_ops += v_

    # FP64 pipe peak (DFMA instructions/s) from the probe
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = sms * 8, 4096
    probe_out = torch.empty(blocks * 256, dtype=torch.float64, device=dev)

    def probe():
        _lib.check(lib.mm_probe_dfma(probe_out.data_ptr(), blocks, iters, stream.cuda_stream), "mm_probe_dfma")

    t_probe = time_eager(probe, reps=5)
    dfma_peak = 8.0 * iters * blocks * 256 / (t_probe * 1e-3)

    hbm_peak, peak_kind = measured_peaks()
    if t_vjp >= t_fwd:
        dom, t_dom, bytes_dom, ops_dom = "vjp_items_kernel", t_vjp, 32.0 * total, vjp_ops
    else:
        dom, t_dom, bytes_dom, ops_dom = "fwd_cta_kernel", t_fwd, 16.0 * total, fwd_ops
    achieved_gbs = bytes_dom / (t_dom * 1e-3) / 1e9
    # DRAM bytes per launch from one ncu capture of the VJP on a 1024-triple batch
    # (52.1 B per amplitude: dram__bytes_read.sum + dram__bytes_write.sum), scaled by amplitudes
    traffic = VJP_DRAM_BYTES_PER_AMP * total if dom == "vjp_items_kernel" else None

    extras = {}
    if args.skip_extras:
        e2e_ms, h2d, d2h, plain_value, cpu = float("nan"), 0, 0, float("nan"), None
    else:
        e2e_ms, h2d, d2h, plain_value, cpu, extras = run_extras(args, rank, world, dev, rb, A, b, c, g, G, grads,
                                                                shapes, As, bs, cs, time_eager, dfma_peak)
    # self-certification: oracle error of every instance, batched over per-instance loop
    err = extras.pop("max_rel_err_vs_oracle", None)
    bop = value / world / plain_value if plain_value == plain_value else None
    single = extras.get("single_instance_forward") or {}
    gates = {"max_rel_err_vs_oracle": err, "err_tol": ERR_TOL,
             "err_checked": ("every instance's G, dA, db, dc of the host-buffer step vs the C oracle"
                             if err is not None else "not checked (--skip-cpu, or N > 1)"),
             "batched_over_plain": bop, "batched_over_plain_min": MIN_BATCHED_OVER_PLAIN,
             "single_instance_forward_ms": {k: v["ms"] for k, v in single.items()}}
    failed = []
    if err is not None and not err <= ERR_TOL:
        failed.append(f"oracle error {err:.3e} > {ERR_TOL:g}")
    if bop is not None and not bop >= MIN_BATCHED_OVER_PLAIN:
        failed.append(f"batched/plain {bop:.2f} < {MIN_BATCHED_OVER_PLAIN:g}")
    gates["pass"] = not failed
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "gates": gates,
            "config": workload_config(n_global, total_all, world),
            "e2e": {"value": total_all / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
            "gpu_launches": launches_per_step * args.steps,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s",
                         "frac": achieved_gbs / hbm_peak, "peak_kind": peak_kind, "traffic": traffic,
                         "algorithmic_bytes_per_launch": bytes_dom, "ms_per_launch": t_dom,
                         "fp64": {"achieved_dfma_per_s": ops_dom / (t_dom * 1e-3), "peak_dfma_per_s": dfma_peak,
                                  "frac": ops_dom / (t_dom * 1e-3) / dfma_peak,
                                  "peak_kind": "measured (mm_probe_dfma)"},
                         "binding_pipe": "fp64",
                         "note": "the recurrence and its VJP are FP64 arithmetic on a part with 1/64-rate FP64: "
                                 "the FP64 pipe (fp64.frac, of the measured DFMA peak) binds, not HBM"},
            "clocks": clocks,
            "step": "one CUDA graph replay (ragged forward + VJP of this rank's instances)",
            "kernels_ms": {"forward": t_fwd, "vjp": t_vjp},
            "plain_loop": {"value": plain_value, "unit": UNIT,
                           "sample": "256 instances drawn uniformly without replacement (numpy seed 11), "
                                     "device_fwd + device_vjp per instance", "batched_over_plain": bop},
            "schedule": ({k: tuned[k] for k in ("team_min_amps", "team_cluster", "vjp_item_amps")}
                         if tuned else "plan defaults"),
        }
        if cpu is not None:
            cpu["max_rel_err_vs_oracle"] = err
            line["cpu_baseline"] = cpu
        line.update(extras)
        print(json.dumps(line), flush=True)
        if failed:
            print("bench gates failed: " + "; ".join(failed), file=sys.stderr, flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 1 if failed else 0


def run_extras(args, rank, world, dev, rb, A, b, c, g, G, grads, shapes, As, bs, cs, time_eager, dfma_peak):
    """e2e with host copies, the per-instance loop, the CPU oracle, single-instance and contraction figures."""
    import torch

    import mrmustard_gb300 as mm

    stream = torch.cuda.current_stream(dev)
    total = rb.total
    barrier = (lambda: torch.distributed.barrier()) if world > 1 else (lambda: None)
    # --- e2e through the public API with pinned host buffers
    A_h = A.cpu().pin_memory()
    b_h = b.cpu().pin_memory()
    c_h = c.cpu().pin_memory()
    g_h = g.cpu().pin_memory()
    G_h = torch.empty(total, dtype=torch.complex128).pin_memory()
    dA_h = torch.empty(rb.n_a, dtype=torch.complex128).pin_memory()
    db_h = torch.empty(rb.n_b, dtype=torch.complex128).pin_memory()
    dc_h = torch.empty(rb.B, dtype=torch.complex128).pin_memory()
    h2d = sum(t.numel() * 16 for t in (A_h, b_h, c_h, g_h))
    d2h = sum(t.numel() * 16 for t in (G_h, dA_h, db_h, dc_h))

    e2e_steps = max(2, min(args.steps, 5))
    e2e_modes = {}
    # fused_sN: the forward writes the host copy of G for the instances k % 8 < N, the VJP the rest
    for name, mode, split in (("prefetch", "prefetch", 0), ("zero_copy", "zero_copy", 0),
                              ("pipelined", "pipelined", 0), ("fused", "fused", 0), ("fused_s2", "fused", 2),
                              ("fused_s3", "fused", 3), ("fused_s4", "fused", 4)):
        with mm.settings(CHECK_DEVICE_STATUS=False):
            rb.step_host(A_h, b_h, c_h, g_h, G_h, dA_h, db_h, dc_h, cotangent=mode, copy_split=split)
            torch.cuda.synchronize()
            barrier()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(e2e_steps):
                rb.step_host(A_h, b_h, c_h, g_h, G_h, dA_h, db_h, dc_h, cotangent=mode, copy_split=split)
            e1.record(stream)
            torch.cuda.synchronize()
            barrier()
        e2e_modes[name] = e0.elapsed_time(e1) / e2e_steps
    e2e_mode = min(e2e_modes, key=e2e_modes.get)
    e2e_ms = e2e_modes[e2e_mode]
    if world > 1:  # the slowest rank's step, as for the device-timed value
        t = torch.tensor([e2e_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    rb.ws.check_status("e2e")

    # --- plain per-instance GPU path on a sample of instances (scaled to amplitudes/s)
    rng = np.random.default_rng(11)
    sample = rng.choice(len(shapes), min(256, len(shapes)), replace=False)
    dev_inputs = [(torch.as_tensor(As[k], device=dev), torch.as_tensor(bs[k], device=dev),
                   torch.tensor(cs[k], device=dev), g[rb.g_off[k]:rb.g_off[k] + rb.sizes[k]].reshape(shapes[k]))
                  for k in sample]
    amps_sample = int(rb.sizes[sample].sum())

    def plain():
        for (Ak, bk, ck, gk), k in zip(dev_inputs, sample):
            Gk = mm.device_fwd(Ak, bk, ck, shapes[k])
            mm.device_vjp(Gk, ck, gk, batched=False)

    with mm.settings(CHECK_DEVICE_STATUS=False):
        t_plain = time_eager(plain, reps=2)
    plain_value = amps_sample / (t_plain * 1e-3)

    # --- CPU baseline: the oracle (C port) on the host cores, full workload, one pass
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        import oracle

        rh = oracle.RaggedHost(shapes)
        A_np = np.concatenate([a.ravel() for a in As])
        b_np = np.concatenate(bs)
        g_np = g_h.numpy()
        G_np = np.empty(total, np.complex128)
        # timed: the speed build of the C port (-O3, FMA contraction, OpenMP over instances)
        G_fast = np.empty(total, np.complex128)
        t0 = time.perf_counter()
        oracle.fwd_ragged(rh, A_np, b_np, cs, out=G_fast, fast=True)
        oracle.vjp_ragged(rh, G_fast, cs, g_np, fast=True)
        tc = time.perf_counter() - t0
        del G_fast
        # the checker build (-O2, no contraction: the parity oracle), also timed for reference
        t0 = time.perf_counter()
        oracle.fwd_ragged(rh, A_np, b_np, cs, out=G_np)
        dA_o, db_o, dc_o = oracle.vjp_ragged(rh, G_np, cs, g_np)
        tc_chk = time.perf_counter() - t0
        cpu = {"value": total / tc, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
               "build": "gcc " + " ".join(oracle.FAST_FLAGS) + " -fopenmp (no -march flags)",
               "sample": f"all {len(shapes)} instances ({total} amplitudes), one fwd+VJP pass, {tc:.2f} s",
               "checker_build_value": total / tc_chk}
        # the oracle as checker: every instance's G, dA, db, dc from the host-buffer step above
        # against the checker build's, max over instances of max|x - ref| / max|ref|
        assert all(np.array_equal(x, y) for x, y in ((rb.g_off, rh.g_off), (rb.a_off, rh.a_off), (rb.b_off, rh.b_off)))

        def inst_err(x, ref, off):
            num = np.maximum.reduceat(np.abs(x - ref), off)
            den = np.maximum.reduceat(np.abs(ref), off)
            return float(np.max(num / np.where(den > 0, den, 1.0)))

        extras_err = max(inst_err(G_h.numpy(), G_np, rh.g_off), inst_err(dA_h.numpy(), dA_o, rh.a_off),
                         inst_err(db_h.numpy(), db_o, rh.b_off), inst_err(dc_h.numpy(), dc_o, np.arange(len(shapes))))
        cpu["checked"] = "every instance's G, dA, db, dc of the host-buffer step against this run's outputs"

    extras = {"e2e_cotangent_ms": e2e_modes, "e2e_cotangent_path": e2e_mode}
    if cpu is not None:
        extras["max_rel_err_vs_oracle"] = extras_err
    extras["single_instance_forward"] = run_single(dev, time_eager, dfma_peak)
    extras["autoshape"] = run_autoshape(dev, time_eager, As, bs,
                                        with_cpu=(rank == 0 and world == 1 and not args.skip_cpu))
    extras["binomial"] = run_binomial(dev, time_eager, with_cpu=(rank == 0 and world == 1 and not args.skip_cpu))
    extras["diagonal"] = run_diagonal(dev, time_eager, with_cpu=(rank == 0 and world == 1 and not args.skip_cpu))
    extras["einsum"] = run_einsum(dev, time_eager, with_cpu=(rank == 0 and world == 1 and not args.skip_cpu))
    extras["plain_and_gradient"] = run_plain_and_gradient(dev, time_eager,
                                                          with_cpu=(rank == 0 and world == 1 and not args.skip_cpu))

    extras["fock_contraction"] = run_contraction(dev, time_eager)
    return e2e_ms, h2d, d2h, plain_value, cpu, extras


def run_autoshape(dev, time_eager, As, bs, with_cpu=True):
    """autoshape (per-mode cutoffs, the reference's defaults 0.99999 / 50 / 1) of every state of the
    workload as a normalised density-matrix triple, one launch per mode count; the C oracle with
    OpenMP is the CPU baseline and the exact-match check.  Normalisation: the trace of a
    density-matrix triple is |c exp(-b (A - X)^-1 b / 2) / sqrt(det(A - X))|, X = [[0, I], [I, 0]]."""
    import torch

    import mrmustard_gb300 as mm

    trip, groups = [], {}
    for k, (A, b) in enumerate(zip(As, bs)):
        Adm, bdm, _ = mm.ket_dm_triple(A, b, 1.0)
        M = len(b)
        K = Adm - np.block([[np.zeros((M, M)), np.eye(M)], [np.eye(M), np.zeros((M, M))]])
        tr = abs(np.exp(-0.5 * bdm @ np.linalg.solve(K, bdm)) / np.sqrt(np.linalg.det(K)))
        trip.append((Adm, bdm, np.complex128(1.0 / tr)))
        groups.setdefault(M, []).append(k)
    dev_groups = {M: tuple(torch.as_tensor(np.array([trip[k][i] for k in ks]), device=dev) for i in range(3))
                  for M, ks in groups.items()}

    streams = {M: torch.cuda.Stream(dev) for M in dev_groups}
    main = torch.cuda.current_stream(dev)

    def run():
        # one launch per mode count, each on its own stream (they are independent)
        res = {}
        for M in dev_groups:
            streams[M].wait_stream(main)
            with torch.cuda.stream(streams[M]):
                res[M] = mm.autoshape_batched(*dev_groups[M])
        for M in dev_groups:
            main.wait_stream(streams[M])
        return res

    t = time_eager(run, reps=20)
    got = {M: v.cpu().numpy() for M, v in run().items()}
    shapes = [None] * len(As)
    for M, ks in groups.items():
        for row, k in enumerate(ks):
            shapes[k] = got[M][row]
    flat = np.concatenate(shapes)
    out = {"states": len(As), "modes": int(flat.size), "ms": t, "states_per_s": len(As) / (t * 1e-3),
           "launches": len(groups), "mean_cutoff": float(flat.mean()),
           "clipped_at_max_fraction": float(np.mean(flat == 50)),
           "note": "time of the autoshape_batched calls (one per mode count, concurrent streams), Python included"}
    if with_cpu:
        import oracle

        t0 = time.perf_counter()
        ref = oracle.autoshape_ragged([x[0] for x in trip], [x[1] for x in trip], [x[2] for x in trip], 0.99999, 50, 1)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": len(As) / tc, "unit": "states/s", "cores": oracle.num_threads(),
                               "kind": "port", "sample": f"all {len(As)} states, one pass, {tc * 1e3:.1f} ms",
                               "mismatches_vs_gpu": int(sum(not np.array_equal(a, r) for a, r in zip(shapes, ref)))}
    return out


def run_binomial(dev, time_eager, with_cpu=True):
    """Binomial fill of one 4-mode pure state at local cutoff 30 (810 k amplitudes) with the
    reference's default max_l2 (0.99999) and global cutoff (sum(shape) - D + 1): GPU time of
    mm_binomial against the C oracle on one core (the reference's strategy is sequential over
    weights).  `ms` is the device time of the fill (mm_binomial on preallocated buffers, back to
    back); `api_ms` the same through mm.device_binomial (allocation, workspace, Python)."""
    import torch
    from scipy.stats import unitary_group

    import mrmustard_gb300 as mm

    rng = np.random.default_rng(4343)
    D, cut = 4, 30
    Q = unitary_group.rvs(D, random_state=rng)
    A = (Q * rng.uniform(0.0, 0.8, D)) @ Q.T
    b = 0.3 * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(2)
    # normalised ket: |c|^2 = 1 / trace of the density-matrix triple of c = 1
    Adm, bdm, _ = mm.ket_dm_triple(A, b, 1.0)
    K = Adm - np.block([[np.zeros((D, D)), np.eye(D)], [np.eye(D), np.zeros((D, D))]])
    c0 = 1.0 / np.sqrt(abs(np.exp(-0.5 * bdm @ np.linalg.solve(K, bdm)) / np.sqrt(np.linalg.det(K))))
    Ad, bd = torch.as_tensor(A, device=dev), torch.as_tensor(b, device=dev)
    cd = torch.tensor(complex(c0), dtype=torch.complex128, device=dev)
    shape = (cut,) * D
    gc = sum(shape) - D + 1
    from mrmustard_gb300 import _lib
    from mrmustard_gb300.hermite import Workspace, _shape_arr

    lib = _lib.load()
    _, sh = _shape_arr(shape)
    Gd = torch.empty(shape, dtype=torch.complex128, device=dev)
    nd = torch.empty((), dtype=torch.float64, device=dev)
    ws = Workspace(lib.mm_binomial_workspace_bytes(D, sh), dev)
    cd1 = cd.reshape(1)
    stream = torch.cuda.current_stream(dev).cuda_stream

    def fill():
        _lib.check(lib.mm_binomial(D, sh, Ad.data_ptr(), bd.data_ptr(), cd1.data_ptr(), 0.99999, gc, Gd.data_ptr(),
                                   nd.data_ptr(), ws.ptr, ws.nbytes, stream), "mm_binomial")

    t = time_eager(fill, reps=20)
    ws.check_status("binomial")
    with mm.settings(CHECK_DEVICE_STATUS=False):
        t_api = time_eager(lambda: mm.device_binomial(Ad, bd, cd, shape, 0.99999, gc), reps=10)
    G, norm = mm.device_binomial(Ad, bd, cd, shape, 0.99999, gc)
    Gh = G.cpu().numpy()
    if not np.array_equal(Gh, Gd.cpu().numpy()):
        raise RuntimeError("binomial: the buffered and the API fill differ")
    w = np.indices(shape).sum(axis=0)
    kept = int(w[Gh != 0].max()) if np.any(Gh != 0) else 0
    out = {"shape": list(shape), "amplitudes": cut ** D, "ms": t, "amplitudes_per_s": cut ** D / (t * 1e-3),
           "api_ms": t_api, "norm": float(norm), "stop_weight": kept}
    if with_cpu:
        import oracle

        t0 = time.perf_counter()
        ref, rnorm, stop = oracle.binomial(shape, A, b, complex(c0), 0.99999, gc)
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": cut ** D / tc, "unit": "amplitudes/s", "cores": 1, "kind": "port",
                               "sample": f"the same fill, one pass, {tc * 1e3:.1f} ms",
                               "stop_weight": stop, "max_rel_err_vs_gpu": float(np.abs(Gh - ref).max() / np.abs(ref).max())}
    return out


def _pnr_triple(M, seed, r_max=0.6, t_max=0.3, beta=0.4):
    """conj(-A), conj(b), c of a mixed M-mode Gaussian state in Bargmann order (bra modes, then ket
    modes): A = [[conj(K), C^T], [C, K]], K = U diag(tanh r) U^T, C = V diag(t) V^dagger."""
    from scipy.stats import unitary_group

    rng = np.random.default_rng(seed)
    U = unitary_group.rvs(M, random_state=rng)
    V = unitary_group.rvs(M, random_state=rng)
    K = (U * np.tanh(rng.uniform(0.05, r_max, M))) @ U.T
    Cm = (V * rng.uniform(0.0, t_max, M)) @ V.conj().T
    A = np.block([[K.conj(), Cm.T], [Cm, K]])
    bk = beta * (rng.standard_normal(M) + 1j * rng.standard_normal(M))
    return np.conj(-A), np.conj(np.concatenate([bk.conj(), bk])), np.complex128(0.7)


def run_diagonal(dev, time_eager, with_cpu=True):
    """Diagonal strategies on mixed Gaussian states: PNR amplitudes of 4 modes at cutoff 12 (20,736
    lattice points), of 3 modes at cutoff 10 with 64 B vectors, their Jacobians (3 modes at cutoff 8),
    compactFock's leftover-mode blocks of 3 modes (output cutoff 10, PNR cutoffs 10, 10) and their
    Jacobians (5; 4, 4), and fast_diagonal of 3 modes (output cutoff 20, PNR cutoffs 10, 10) and
    4 modes (10; 6, 6, 6).
    GPU time per call (device tensors in and out, Python included) against the C oracle on one core
    (the reference runs these single-threaded), with every output checked against the oracle."""
    import torch

    import mrmustard_gb300 as mm

    def ilv(A, b):
        o = np.arange(A.shape[0]).reshape(2, -1).T.flatten()
        return A[o][:, o], b[o]

    def td(x):
        return torch.as_tensor(x, device=dev)

    res = {}
    cases = (("pnr_4x12", 4, (12,) * 4, 1), ("pnr_3x10_b64", 3, (10,) * 3, 64))
    for name, M, cut, nb in cases:
        A, b, c = _pnr_triple(M, 600 + M)
        Ai, bi = ilv(A, b)
        B = bi if nb == 1 else bi[:, None] * np.linspace(0.5, 1.5, nb)[None, :]
        At, Bt, ct = td(Ai), td(B), td(c)
        with mm.settings(CHECK_DEVICE_STATUS=False):
            t = time_eager(lambda: mm.hermite_multidimensional_diagonal(At, Bt, ct, cut), reps=10)
        got = mm.hermite_multidimensional_diagonal(At, Bt, ct, cut)
        P = int(np.prod(cut))
        r = {"modes": M, "cutoffs": list(cut), "batch": nb, "points": P, "ms": t, "points_per_s": P * nb / (t * 1e-3)}
        if with_cpu:
            import oracle

            t0 = time.perf_counter()
            ref = oracle.diagonal_amps(Ai, B, c, cut)
            tc = time.perf_counter() - t0
            err = max(oracle.rel_err(x.cpu().numpy(), y) for x, y in zip(got, ref))
            r["cpu_baseline"] = {"value": P * nb / tc, "unit": "points/s", "cores": 1, "kind": "port",
                                 "sample": f"the same call, one pass, {tc * 1e3:.1f} ms", "max_rel_err_vs_gpu": err}
        res[name] = r
    # Jacobians
    M, cut = 3, (8, 8, 8)
    A, b, c = _pnr_triple(M, 700)
    Ai, bi = ilv(A, b)
    At, bt, ct = td(Ai), td(bi), td(c)
    arrs = mm.hermite_multidimensional_diagonal(At, bt, ct, cut)
    with mm.settings(CHECK_DEVICE_STATUS=False):
        t = time_eager(lambda: mm.grad_hermite_multidimensional_diagonal(At, bt, ct, *arrs), reps=10)
    got = mm.grad_hermite_multidimensional_diagonal(At, bt, ct, *arrs)
    P = int(np.prod(cut))
    r = {"modes": M, "cutoffs": list(cut), "points": P, "jacobian_entries": P * (4 * M * M + 2 * M), "ms": t}
    if with_cpu:
        import oracle

        t0 = time.perf_counter()
        ref = oracle.diagonal_grad(Ai, bi, c, cut)
        tc = time.perf_counter() - t0
        r["cpu_baseline"] = {"value": P / tc, "unit": "points/s", "cores": 1, "kind": "port",
                             "sample": f"amplitudes and Jacobians, one pass, {tc * 1e3:.1f} ms",
                             "max_rel_err_vs_gpu": max(oracle.rel_err(x.cpu().numpy(), y) for x, y in zip(got, ref))}
    res["jacobian_3x8"] = r
    # compactFock leftover mode (the JAX backend's path): amplitudes and Jacobians
    for name, M, cut, jac in (("leftover_compact_3_oc10_pnr10x10", 3, (11, 11, 11), False),
                              ("leftover_compact_jacobian_3_oc5_pnr4x4", 3, (6, 5, 5), True)):
        A, b, c = _pnr_triple(M, 900 + M)
        Ai, bi = ilv(A, b)
        At, bt, ct = td(Ai), td(bi), td(c)
        arrs = mm.hermite_multidimensional_1leftoverMode(At, bt, ct, cut)
        if jac:
            fn = lambda: mm.grad_hermite_multidimensional_1leftoverMode(At, bt, ct, *arrs)
        else:
            fn = lambda: mm.hermite_multidimensional_1leftoverMode(At, bt, ct, cut)
        with mm.settings(CHECK_DEVICE_STATUS=False):
            t = time_eager(fn, reps=10)
        got = fn()
        nout = int(np.prod(cut)) * cut[0]
        r = {"modes": M, "cutoffs": list(cut), "block_entries": nout, "ms": t}
        if with_cpu:
            import oracle

            t0 = time.perf_counter()
            ref = oracle.leftover_grad(Ai, bi, c, cut) if jac else oracle.leftover_amps(Ai, bi, c, cut)
            tc = time.perf_counter() - t0
            r["cpu_baseline"] = {"value": tc * 1e3, "unit": "ms", "cores": 1, "kind": "port",
                                 "sample": "the same call, one pass" + (" (amplitudes and Jacobians)" if jac else ""),
                                 "max_rel_err_vs_gpu": max(oracle.rel_err(x.cpu().numpy(), y) for x, y in zip(got, ref))}
        res[name] = r
    # fast_diagonal
    for name, L, oc, pnr in (("leftover_3_oc20_pnr10x10", 3, 20, (10, 10)), ("leftover_4_oc10_pnr6x6x6", 4, 10, (6, 6, 6))):
        A, b, c = _pnr_triple(L, 800 + L)
        At, bt, ct = td(A), td(b), td(c)
        with mm.settings(CHECK_DEVICE_STATUS=False):
            t = time_eager(lambda: mm.fast_diagonal(At, bt, ct, oc, pnr), reps=10)
        got = mm.fast_diagonal(At, bt, ct, oc, pnr)
        nout = int(np.prod([p + 1 for p in pnr])) * (oc + 1) ** 2
        r = {"modes": L, "output_cutoff": oc, "pnr_cutoffs": list(pnr), "output_amplitudes": nout, "ms": t}
        if with_cpu:
            import oracle

            t0 = time.perf_counter()
            ref = oracle.fast_diagonal(A, b, c, oc, pnr)
            tc = time.perf_counter() - t0
            r["cpu_baseline"] = {"value": nout / tc, "unit": "output amplitudes/s", "cores": 1, "kind": "port",
                                 "sample": f"the same call, one pass, {tc * 1e3:.1f} ms",
                                 "max_rel_err_vs_gpu": oracle.rel_err(got.cpu().numpy(), ref)}
        res[name] = r
    return res


def run_einsum(dev, time_eager, with_cpu=True):
    """Fock-space einsum: a 2-mode gate at cutoff 40 applied to 64 two-mode kets
    ('abcd,zcd->zab', a 1600 x 1600 x 64 complex GEMM plus the permutations of kets and result), and
    the ket0 / beamsplitter / ket1 network of mm_einsum's docstring at cutoff 60 ('a,cdab,b->cd', a
    207 MB gate read once: HBM-bound), GPU time per call (device tensors) against numpy einsum on the
    host cores (the reference's math.einsum is opt_einsum -> BLAS)."""
    import torch

    import mrmustard_gb300 as mm

    rng = np.random.default_rng(9090)

    def cn(*shape):
        return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)

    res = {}
    cases = (("gate40_on_64kets", "abcd,zcd->zab", (cn(40, 40, 40, 40) / 1600, cn(64, 40, 40)),
              8.0 * 1600 * 1600 * 64, None),
             ("bs60_network", "a,cdab,b->cd", (cn(60), cn(60, 60, 60, 60) / 3600, cn(60)), None, 16.0 * 60 ** 4))
    for name, sub, ops, flops, nbytes in cases:
        dops = [torch.as_tensor(x, device=dev) for x in ops]
        t = time_eager(lambda: mm.einsum(sub, *dops), reps=10)
        got = mm.einsum(sub, *dops).cpu().numpy()
        r = {"subscripts": sub, "shapes": [list(x.shape) for x in ops], "ms": t}
        if flops:
            r["fp64_tflops"] = flops / (t * 1e-3) / 1e12
        if nbytes:
            r["gate_read_gbs"] = nbytes / (t * 1e-3) / 1e9
        if name.startswith("gate"):
            tz = time_eager(lambda: mm.einsum(sub, *dops, mode="ozaki"), reps=10)
            r["ozaki_ms"] = tz
        if with_cpu:
            import oracle

            t0 = time.perf_counter()
            ref = oracle.einsum(sub, *ops)
            tc = time.perf_counter() - t0
            r["cpu_baseline"] = {"value": tc * 1e3, "unit": "ms", "cores": os.cpu_count(), "kind": "port",
                                 "sample": "numpy einsum (BLAS) of the same operands, one pass",
                                 "max_rel_err_vs_gpu": oracle.rel_err(got, ref)}
        res[name] = r
    return res


def run_plain_and_gradient(dev, time_eager, with_cpu=True):
    """The plain and the differentiation configurations: one 3-mode pure state at cutoff 20 (8,000
    amplitudes; latency of the public call with numpy in and out, and of the device call), one
    4-mode triple at cutoff 30 through the autograd function (forward + backward with a complex
    normal upstream gradient), and the 64-instance batched gradient step whose loss is the fidelity
    of each state to a fixed random normalised target Fock tensor (forward, loss, backward).  CPU
    oracle on one core for the single-instance ones (the reference's numba path is single-threaded
    per instance)."""
    import torch
    from scipy.stats import unitary_group

    import mrmustard_gb300 as mm

    def takagi(D, smax, seed):
        rng = np.random.default_rng(seed)
        Q = unitary_group.rvs(D, random_state=rng)
        A = (Q * rng.uniform(0.0, smax, D)) @ Q.T
        b = 0.3 * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(2)
        return A.astype(np.complex128), b.astype(np.complex128)

    res = {}
    # plain 3 x 20
    A, b = takagi(3, 0.8, 7070)
    shape = (20, 20, 20)
    with mm.settings(CHECK_DEVICE_STATUS=False):
        mm.hermite_renormalized(A, b, 1.0 + 0j, shape)
        t_api = time_eager(lambda: mm.hermite_renormalized(A, b, 1.0 + 0j, shape), reps=50)
        Ad, bd = torch.as_tensor(A, device=dev), torch.as_tensor(b, device=dev)
        cd = torch.tensor(1.0 + 0j, dtype=torch.complex128, device=dev)
        out = torch.empty(shape, dtype=torch.complex128, device=dev)
        t_dev = time_eager(lambda: mm.device_fwd(Ad, bd, cd, shape, out=out), reps=50)
    r = {"shape": list(shape), "amplitudes": 8000, "us_per_call_numpy_api": t_api * 1e3,
         "us_per_call_device": t_dev * 1e3, "amplitudes_per_s_device": 8000 / (t_dev * 1e-3)}
    if with_cpu:
        import oracle

        G = mm.hermite_renormalized(A, b, 1.0 + 0j, shape)
        tcs = {}
        for fast in (True, False):
            oracle.vanilla(shape, A, b, 1.0 + 0j, fast=fast)
            t0 = time.perf_counter()
            for _ in range(50):
                ref = oracle.vanilla(shape, A, b, 1.0 + 0j, fast=fast)
            tcs[fast] = (time.perf_counter() - t0) / 50
        r["cpu_baseline"] = {"value": tcs[True] * 1e6, "unit": "us per call", "cores": 1, "kind": "port",
                             "build": "gcc " + " ".join(oracle.FAST_FLAGS), "checker_build_us": tcs[False] * 1e6,
                             "sample": "the same call (numpy in, numpy out), 50 passes",
                             "max_rel_err_vs_gpu": oracle.rel_err(G, ref)}
    res["plain_3x20"] = r
    # autograd 4 x 30
    A, b = takagi(4, 0.8, 7171)
    shape = (30,) * 4
    At = torch.as_tensor(A, device=dev).requires_grad_(True)
    bt = torch.as_tensor(b, device=dev).requires_grad_(True)
    ct = torch.tensor(1.0 + 0j, dtype=torch.complex128, device=dev, requires_grad=True)
    gen = torch.Generator(device=dev)
    gen.manual_seed(71)
    gup = torch.complex(torch.randn(shape, generator=gen, device=dev, dtype=torch.float64),
                        torch.randn(shape, generator=gen, device=dev, dtype=torch.float64))

    def step():
        # gradients set to None every step (as a training loop's zero_grad does): accumulating into
        # .grad would make the first accumulating step launch torch's complex add kernel, whose
        # module CUDA loads lazily on first use (~0.75 s from a cold page cache on a fresh box)
        for x in (At, bt, ct):
            x.grad = None
        G = mm.hermite_renormalized_autograd(At, bt, ct, shape)
        G.backward(gup)

    def wall_ms(fn, reps):
        # autograd runs the backward on its own thread: time with a host clock between synchronisations
        for _ in range(3):
            fn()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize(dev)
        return (time.perf_counter() - t0) / reps * 1e3

    def per_rep(fn, reps):
        """Per-rep host time (synchronised each rep) and device time by CUDA events on the stream
        both the forward and autograd's backward run on (the current stream when the forward ran)."""
        stream = torch.cuda.current_stream(dev)
        host, devt = [], []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize(dev)
            host.append((time.perf_counter() - t0) * 1e3)
            devt.append(e0.elapsed_time(e1))

        def dist(a):
            a = np.asarray(a)
            return {"median": float(np.median(a)), "p10": float(np.percentile(a, 10)),
                    "p90": float(np.percentile(a, 90)), "max": float(a.max()), "mean": float(a.mean())}

        return {"reps": reps, "host_ms": dist(host), "device_ms": dist(devt)}

    with mm.settings(CHECK_DEVICE_STATUS=False):
        t = wall_ms(step, reps=50)
        reps = per_rep(step, 60)
    r = {"shape": list(shape), "amplitudes": 30 ** 4, "ms_fwd_bwd": t, "amplitudes_per_s": 30 ** 4 / (t * 1e-3),
         "timing": "host clock over 50 back-to-back steps after 3 warm-up steps; per_rep: 60 synchronised steps",
         "per_rep": reps}
    if with_cpu:
        import oracle

        gh = gup.cpu().numpy()
        t0 = time.perf_counter()
        for _ in range(3):
            G = oracle.vanilla(shape, A, b, 1.0 + 0j, fast=True)
            oracle.vjp(G, 1.0 + 0j, gh, fast=True)
        tc = (time.perf_counter() - t0) / 3
        r["cpu_baseline"] = {"value": tc * 1e3, "unit": "ms", "cores": 1, "kind": "port",
                             "build": "gcc " + " ".join(oracle.FAST_FLAGS),
                             "sample": "forward + VJP of the same triple, 3 passes"}
    res["autograd_4x30"] = r
    # the same step with a checkpointed backward (residual: checkpoint slabs instead of G)
    ck_rows = {}
    for K in (5, 10):
        def step_ck(K=K):
            for x in (At, bt, ct):
                x.grad = None
            G = mm.hermite_renormalized_autograd(At, bt, ct, shape, checkpoint=K)
            G.backward(gup)

        with mm.settings(CHECK_DEVICE_STATUS=False):
            t_ck = wall_ms(step_ck, reps=50)
        resid = mm.checkpoint_elems(shape, K) * 16
        ck_rows[f"K{K}"] = {"ms_fwd_bwd": t_ck, "residual_bytes": resid, "residual_frac_of_G": resid / (16 * 30 ** 4)}
    res["autograd_4x30_checkpointed"] = {"shape": list(shape), "full_G_residual_bytes": 16 * 30 ** 4,
                                         "segments": ck_rows,
                                         "timing": "host clock over 50 back-to-back steps after 3 warm-up steps"}
    # 64-instance batched fidelity gradient step
    B = 64
    trip = [takagi(4, 0.8, 7300 + k) for k in range(B)]
    Ab = torch.as_tensor(np.stack([t[0] for t in trip]), device=dev).requires_grad_(True)
    bb = torch.as_tensor(np.stack([t[1] for t in trip]), device=dev).requires_grad_(True)
    cb = torch.ones(B, dtype=torch.complex128, device=dev, requires_grad=True)
    T = torch.complex(torch.randn(shape, generator=gen, device=dev, dtype=torch.float64),
                      torch.randn(shape, generator=gen, device=dev, dtype=torch.float64))
    T = T / T.abs().pow(2).sum().sqrt()

    def fid_step():
        for x in (Ab, bb, cb):
            x.grad = None
        G = mm.hermite_renormalized_autograd(Ab, bb, cb, shape)
        ov = (T.conj() * G).sum(dim=(1, 2, 3, 4))
        loss = (1 - ov.abs() ** 2 / G.abs().pow(2).sum(dim=(1, 2, 3, 4))).sum()
        loss.backward()

    with mm.settings(CHECK_DEVICE_STATUS=False):
        t = wall_ms(fid_step, reps=10)
    res["fidelity_step_64x4x30"] = {"instances": B, "shape": list(shape), "amplitudes": B * 30 ** 4,
                                    "ms_per_step": t, "amplitudes_per_s": B * 30 ** 4 / (t * 1e-3),
                                    "note": "forward, fidelity loss (torch reductions), backward; host clock between "
                                            "device synchronisations"}
    return res


def run_single(dev, time_eager, dfma_peak=None):
    """Single large recurrences on the whole GPU (4 modes at cutoff 40, pure state; 4-index
    density-matrix triple at cutoff 50), timed with CUDA events; HBM and FP64-pipe fractions."""
    import torch

    import mrmustard_gb300 as mm

    single = {}
    for name, D, cut, kind in (("pure_4x40", 4, 40, "pure"), ("dm_4x50", 4, 50, "dm")):
        rng = np.random.default_rng(4242 + cut)
        if kind == "pure":
            from scipy.stats import unitary_group

            Q = unitary_group.rvs(D, random_state=rng)
            A1 = (Q * rng.uniform(0, 0.85, D)) @ Q.T
        else:
            X1 = rng.standard_normal((D, D)) + 1j * rng.standard_normal((D, D))
            A1 = X1 + X1.T
            A1 *= 0.89 / np.linalg.norm(A1, 2)
        b1 = 0.3 * (rng.standard_normal(D) + 1j * rng.standard_normal(D)) / np.sqrt(2)
        At, bt = torch.as_tensor(A1, device=dev), torch.as_tensor(b1, device=dev)
        ct = torch.tensor(1.0 + 0j, dtype=torch.complex128, device=dev)
        out = torch.empty((cut,) * D, dtype=torch.complex128, device=dev)
        with mm.settings(CHECK_DEVICE_STATUS=False):
            t1 = time_eager(lambda: mm.device_fwd(At, bt, ct, (cut,) * D, out=out), reps=10)
            t_st = time_eager(lambda: mm.device_fwd(At, bt, ct, (cut,) * D, stable=True, out=out), reps=5)
        n1 = cut ** D
        ops = fp64_ops((cut,) * D)[0]
        ops_st = fp64_ops_stable((cut,) * D)
        hbm_peak = measured_peaks()[0]
        r = {"amplitudes": n1, "ms": t1, "amplitudes_per_s": n1 / (t1 * 1e-3),
             "hbm_gbs": 16.0 * n1 / (t1 * 1e-3) / 1e9, "fp64_instructions": ops,
             "stable": {"ms": t_st, "amplitudes_per_s": n1 / (t_st * 1e-3), "fp64_instructions": ops_st,
                        "hbm_frac": 16.0 * n1 / (t_st * 1e-3) / 1e9 / hbm_peak}}
        if dfma_peak:
            r["fp64_frac"] = ops / (t1 * 1e-3) / dfma_peak
            r["stable"]["fp64_frac"] = ops_st / (t_st * 1e-3) / dfma_peak
        single[name] = r
    return single


def fp64_ops_stable(shape):
    """FP64 pipe instructions of the stable forward (stable_wave) for one shape: per amplitude and
    per pivot i (k_i > 0) b_i G (4), one complex FMA (4) per other non-zero axis and for k_i >= 2,
    the scaled add into the average (2); then the 1/#pivots scale (2)."""
    idx = np.indices(shape).reshape(len(shape), -1)
    nz = (idx > 0).sum(0)
    ops = 2.0 * (nz > 0).sum()
    for i in range(len(shape)):
        piv = idx[i] > 0
        ops += float((piv * (6 + 4 * (nz - 1) + 4 * (idx[i] >= 2))).sum())
    return ops


def fp64_probe(dev, time_eager):
    """Measured FP64 pipe rate (DFMA instructions/s) from mm_probe_dfma."""
    import torch

    from mrmustard_gb300 import _lib

    lib = _lib.load()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    blocks, iters = sms * 8, 4096
    probe_out = torch.empty(blocks * 256, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def probe():
        _lib.check(lib.mm_probe_dfma(probe_out.data_ptr(), blocks, iters, stream.cuda_stream), "mm_probe_dfma")

    t_probe = time_eager(probe, reps=5)
    return 8.0 * iters * blocks * 256 / (t_probe * 1e-3)


def run_contraction(dev, time_eager):
    """Gate tensor at cutoff 50 (2500 x 2500, built by the recurrence) applied to 256 kets: FP64 and
    Ozaki tensor-core paths, timed with CUDA events, error against numpy's zgemm on the host."""
    import torch

    import mrmustard_gb300 as mm

    rng = np.random.default_rng(55)
    X5 = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
    A5 = X5 + X5.T
    A5 *= 0.95 / np.linalg.norm(A5, 2)
    b5 = 0.3 * (rng.standard_normal(4) + 1j * rng.standard_normal(4)) / np.sqrt(2)
    U5 = mm.device_fwd(torch.as_tensor(A5, device=dev), torch.as_tensor(b5, device=dev),
                       torch.tensor(1.0 + 0j, dtype=torch.complex128, device=dev), (50, 50, 50, 50)).reshape(2500, 2500)
    kets = torch.complex(torch.randn(256, 2500, dtype=torch.float64, device=dev),
                         torch.randn(256, 2500, dtype=torch.float64, device=dev))
    kets = kets / kets.abs().pow(2).sum(1, keepdim=True).sqrt()
    Xk = kets.T.contiguous()
    U5h, Xkh = U5.cpu().numpy(), Xk.cpu().numpy()
    t0 = time.perf_counter()
    ref5 = U5h @ Xkh
    t_np = time.perf_counter() - t0
    flops = 8.0 * 2500 * 256 * 2500
    contraction = {"shape": "2500x2500 @ 2500x256 complex128", "flops": flops, "numpy_zgemm_ms": t_np * 1e3}
    for mode in ("fp64", "dmma", "ozaki"):
        with mm.settings(CHECK_DEVICE_STATUS=False):
            tm = time_eager(lambda: mm.fock_gemm(U5, Xk, mode), reps=5)
        Y = mm.fock_gemm(U5, Xk, mode).cpu().numpy()
        err = float(np.abs(Y - ref5).max() / np.abs(ref5).max())
        contraction[mode] = {"ms": tm, "tflops": flops / (tm * 1e-3) / 1e12, "max_rel_err_vs_fp64_cpu": err}
    # the Ozaki split issues one real BF16 GEMM quadruple (U_re/U_im x X_re/X_im) per kept slice pair:
    # 7 slices, pairs with p + q <= 8 -> 28 pairs
    pairs = 7 * 8 // 2
    peak, kind = measured_bf16_tflops()
    issued = pairs * flops
    contraction["ozaki"].update({"slice_pairs": pairs, "issued_bf16_flop": issued,
                                 "issued_bf16_tflops_whole_call": issued / (contraction["ozaki"]["ms"] * 1e-3) / 1e12,
                                 "bf16_peak_tflops": peak, "bf16_peak_kind": f"{kind} (burst)"})
    contraction["ozaki"]["frac_of_bf16_peak_whole_call"] = contraction["ozaki"]["issued_bf16_tflops_whole_call"] / peak
    return contraction


def rb_order_largest(rb, n):
    return list(np.argsort(-rb.sizes, kind="stable")[:n])


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--skip-cpu", action="store_true", help="skip the CPU-oracle baseline leg")
    ap.add_argument("--instances", type=int, default=N_INST, help="triples in the ragged batch (profiling runs)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the plan's default schedule")
    ap.add_argument("--only-contraction", action="store_true",
                    help="run only the Fock-contraction leg (gate tensor on 256 kets) and print its figures")
    ap.add_argument("--only-binomial", action="store_true",
                    help="run only the binomial fill of a 4-mode state at cutoff 30 (GPU and CPU oracle)")
    ap.add_argument("--only-plain-gradient", action="store_true",
                    help="run only the plain 3 x 20 call, the autograd 4 x 30 step and the 64-instance fidelity step")
    ap.add_argument("--only-einsum", action="store_true",
                    help="run only the Fock-space einsum cases (GPU and numpy on the host)")
    ap.add_argument("--only-diagonal", action="store_true",
                    help="run only the diagonal strategies (PNR amplitudes, Jacobians, fast_diagonal; GPU and CPU oracle)")
    ap.add_argument("--only-autoshape", action="store_true",
                    help="run only autoshape over the workload's states (GPU and CPU oracle)")
    ap.add_argument("--only-single", action="store_true",
                    help="run only the single large recurrences (4 x 40 pure, 4 x 50 density matrix)")
    ap.add_argument("--skip-extras", action="store_true",
                    help="time only the headline step (no e2e, per-instance loop, contraction, CPU legs)")
    args = ap.parse_args(argv)
    args.warmup = max(3, args.warmup)  # at least 3 untimed warm-up steps
    rank, local_rank, world = dist_env()
    if (args.only_contraction or args.only_single or args.only_autoshape or args.only_binomial or args.only_diagonal
            or args.only_einsum or args.only_plain_gradient):
        import torch

        dev = torch.device("cuda", local_rank)
        torch.cuda.set_device(dev)

        def time_eager(fn, reps=3):
            fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        if args.only_plain_gradient:
            print(json.dumps({"plain_and_gradient": run_plain_and_gradient(dev, time_eager, not args.skip_cpu)}),
                  flush=True)
        elif args.only_einsum:
            print(json.dumps({"einsum": run_einsum(dev, time_eager, not args.skip_cpu)}), flush=True)
        elif args.only_diagonal:
            print(json.dumps({"diagonal": run_diagonal(dev, time_eager, not args.skip_cpu)}), flush=True)
        elif args.only_binomial:
            print(json.dumps({"binomial": run_binomial(dev, time_eager, not args.skip_cpu)}), flush=True)
        elif args.only_autoshape:
            _, As, bs, _ = make_workload(20260000, args.instances)
            print(json.dumps({"autoshape": run_autoshape(dev, time_eager, As, bs, not args.skip_cpu)}), flush=True)
        elif args.only_single:
            print(json.dumps({"single_instance_forward": run_single(dev, time_eager, fp64_probe(dev, time_eager))}),
                  flush=True)
        else:
            print(json.dumps({"fock_contraction": run_contraction(dev, time_eager)}), flush=True)
        return 0
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_gb300(args, rank, local_rank, world)


if __name__ == "__main__":
    sys.exit(main())

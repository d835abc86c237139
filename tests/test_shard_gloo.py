"""Multi-rank path on the CPU: world_size 2 over gloo.

Instances of a ragged batch are independent, so ranks split one batch with
``mrmustard_gb300.shard.shard_instances`` (no data-path collective), as
``RaggedBatch.shard`` and bench.py under torchrun do.  Here each rank plans its share through
the library's host planner (``mm_ragged_plan_create`` / ``mm_ragged_plan_offsets``, no device
needed) and computes it with the CPU oracle in that packing (standing in for the rank's GPU).  The
shares are gathered only to check that every instance was computed exactly once, that the
per-rank plans put back together give the unsharded plan's offsets and packed result bit for bit,
and that the loads are balanced to within one instance.
"""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _case():
    rng = np.random.default_rng(3)
    shapes = [tuple(int(x) for x in rng.integers(1, 9, int(rng.integers(1, 5)))) for _ in range(40)]
    As, bs = [], []
    for k, sh in enumerate(shapes):
        r = np.random.default_rng(100 + k)
        D = len(sh)
        X = r.standard_normal((D, D)) + 1j * r.standard_normal((D, D))
        A = X + X.T
        A *= 0.7 / np.linalg.norm(A, 2)
        As.append(A)
        bs.append(0.3 * (r.standard_normal(D) + 1j * r.standard_normal(D)))
    return shapes, As, bs, np.ones(len(shapes), complex)


def _worker(rank, world, port, out_q):
    import oracle
    from mrmustard_gb300 import shard

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from mrmustard_gb300.ragged import plan_offsets

    shapes, As, bs, cs = _case()
    mine = shard.local_instances(shard.instance_costs(shapes), rank, world)
    results = {k: oracle.vanilla(shapes[k], As[k], bs[k], cs[k]) for k in mine}
    load = float(shard.instance_costs(shapes)[mine].sum())
    # this rank's plan (the packing RaggedBatch.shard uploads) and its packed result
    loc = [shapes[k] for k in mine]
    g_off, a_off, b_off, total = plan_offsets(loc)
    rh = oracle.RaggedHost(loc)
    assert np.array_equal(rh.g_off, g_off) and np.array_equal(rh.a_off, a_off) and np.array_equal(rh.b_off, b_off)
    packed = oracle.fwd_ragged(rh, np.concatenate([As[k].ravel() for k in mine]),
                               np.concatenate([bs[k] for k in mine]), cs[mine])
    plan = {"index": mine, "g_off": g_off, "a_off": a_off, "b_off": b_off, "total": total, "packed": packed}
    gathered = [None] * world
    dist.all_gather_object(gathered, (rank, results, load, plan))
    dist.barrier()
    dist.destroy_process_group()
    if rank == 0:
        out_q.put(gathered)


def test_two_ranks_shard_ragged_batch():
    import oracle

    oracle.build()
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shapes, As, bs, cs = _case()
    seen = {}
    for rank, results, _, _ in gathered:
        for k, G in results.items():
            assert k not in seen, "instance computed twice"
            seen[k] = G
    assert sorted(seen) == list(range(len(shapes)))
    for k, G in seen.items():
        assert np.array_equal(G, oracle.vanilla(shapes[k], As[k], bs[k], cs[k]))
    loads = [g[2] for g in gathered]
    from mrmustard_gb300 import shard
    from mrmustard_gb300.ragged import plan_offsets

    assert abs(loads[0] - loads[1]) <= shard.instance_costs(shapes).max()
    # the per-rank plans put back together give the unsharded plan's offsets and packed result
    g_all, a_all, b_all, total_all = plan_offsets(shapes)
    assert sum(g[3]["total"] for g in gathered) == total_all
    rh = oracle.RaggedHost(shapes)
    ref = oracle.fwd_ragged(rh, np.concatenate([a.ravel() for a in As]), np.concatenate(bs), cs)
    rebuilt = np.full(total_all, np.nan + 0j)
    sizes = np.array([int(np.prod(s)) for s in shapes])
    for _, _, _, plan in gathered:
        loc_sizes = sizes[plan["index"]]
        assert np.array_equal(plan["g_off"], np.concatenate([[0], np.cumsum(loc_sizes)[:-1]]))
        for j, k in enumerate(plan["index"]):
            D = len(shapes[k])
            assert a_all[k] == sum(len(shapes[i]) ** 2 for i in range(k)) and b_all[k] == sum(len(shapes[i])
                                                                                              for i in range(k))
            assert plan["a_off"][j] == sum(len(shapes[i]) ** 2 for i in plan["index"][:j])
            assert plan["b_off"][j] == sum(len(shapes[i]) for i in plan["index"][:j]) and D > 0
            rebuilt[g_all[k]:g_all[k] + sizes[k]] = plan["packed"][plan["g_off"][j]:plan["g_off"][j] + sizes[k]]
    assert np.array_equal(rebuilt, ref)

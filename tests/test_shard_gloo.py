"""Multi-rank path on the CPU: world_size 2 over gloo.

Instances of a ragged batch are independent, so ranks split them with
``mrmustard_gb300.shard.shard_instances`` (no data-path collective; bench.py gives every
rank its own batch).  Here each rank computes its share of a ragged batch with the CPU oracle
(standing in for that rank's GPU), and the shares are gathered only to check that every instance
was computed exactly once and that the union equals the unsharded result; the loads are balanced
to within one instance.
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
    shapes, As, bs, cs = _case()
    mine = shard.local_instances(shard.instance_costs(shapes), rank, world)
    results = {k: oracle.vanilla(shapes[k], As[k], bs[k], cs[k]) for k in mine}
    load = float(shard.instance_costs(shapes)[mine].sum())
    gathered = [None] * world
    dist.all_gather_object(gathered, (rank, results, load))
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
    for rank, results, _ in gathered:
        for k, G in results.items():
            assert k not in seen, "instance computed twice"
            seen[k] = G
    assert sorted(seen) == list(range(len(shapes)))
    for k, G in seen.items():
        assert np.array_equal(G, oracle.vanilla(shapes[k], As[k], bs[k], cs[k]))
    loads = [g[2] for g in gathered]
    from mrmustard_gb300 import shard

    assert abs(loads[0] - loads[1]) <= shard.instance_costs(shapes).max()

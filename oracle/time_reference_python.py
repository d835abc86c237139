"""Time the reference's own source of the path (pure CPython + numpy under a no-op numba module)
on a sample of the 4096-triple benchmark workload, one core.

numba is not installed in either container, so the reference's ``vanilla_numba`` /
``vanilla_vjp_numba`` (mrmustard/math/lattice/strategies/vanilla/core.py:25-124,
gradients.py:25-82) run as plain Python here; this is the "reference source under the shim"
baseline, labelled as such.  It runs only where the MrMustard source tree is available (not on
the GPU machine).  Sample: every `stride`-th instance of the workload in decreasing-cost order.

Usage (from the repository root)::

    python oracle/time_reference_python.py /path/to/mrmustard-source [stride]
"""

from __future__ import annotations

import importlib.util
import json
import os
import platform
import sys
import time
from pathlib import Path

import numpy as np

sys.dont_write_bytecode = True  # the reference tree must stay untouched
ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def main(ref_root: str, stride: int = 64) -> dict:
    spec = importlib.util.spec_from_file_location("_make_golden", ROOT / "tests" / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    mods = mg.load_reference(Path(ref_root))
    core, grads = mods["core"], mods["gradients"]
    import bench

    shapes, As, bs, cs = bench.make_workload(bench.BASE_SEED)
    sizes = np.array([int(np.prod(s)) for s in shapes])
    cost = sizes * (np.array([len(s) for s in shapes]) + 1)
    order = np.argsort(-cost, kind="stable")[::stride]
    rng = np.random.default_rng(7)
    amps = 0
    t_fwd = t_vjp = 0.0
    for k in order:
        t0 = time.perf_counter()
        G = core.vanilla_numba(shapes[k], As[k], bs[k], cs[k])
        t1 = time.perf_counter()
        g = rng.standard_normal(G.shape) + 1j * rng.standard_normal(G.shape)
        t2 = time.perf_counter()
        grads.vanilla_vjp_numba(G, cs[k], g)
        t3 = time.perf_counter()
        t_fwd += t1 - t0
        t_vjp += t3 - t2
        amps += int(sizes[k])
    return {"what": "reference source (vanilla_numba + vanilla_vjp_numba) as CPython under a no-op numba",
            "sample": f"{len(order)} of {len(shapes)} instances (every {stride}th by cost), {amps} amplitudes",
            "cores": 1, "cpu": platform.processor() or platform.machine(), "nproc": os.cpu_count(),
            "fwd_s": t_fwd, "vjp_s": t_vjp, "amplitudes_per_s_fwd_vjp": amps / (t_fwd + t_vjp)}


if __name__ == "__main__":
    print(json.dumps(main(sys.argv[1], int(sys.argv[2]) if len(sys.argv) > 2 else 64)))

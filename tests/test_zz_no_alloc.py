"""The workspace-free VJP entry point, for callers that cannot allocate device memory at call time.

``mm_hermite_vjp_noalloc`` keeps its scratch in a fixed array inside the library, so a caller
that runs inside another framework's allocator and stream (and may not call cudaMalloc) can
still get dL/dA, dL/db, dL/dc.  This test calls it through the C ABI and checks it against the
workspace-taking ``mm_hermite_vjp`` on two calls in a row with different inputs, queued back to
back on one stream with no synchronisation between them (the documented way to use the shared
array), so that state left in the array by the first call cannot leak into the second.  It lives
in its own file, collected last, and passes both alone and after the rest of the suite.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from mrmustard_gb300 import _lib
from mrmustard_gb300.hermite import device_vjp, ensure_device_ready

pytestmark = pytest.mark.gpu

VJP_TOL = 1e-12


def _case(seed, shape):
    rng = np.random.default_rng(seed)
    D = len(shape)
    X = rng.standard_normal((D, D)) + 1j * rng.standard_normal((D, D))
    A = X + X.T
    A *= 0.6 / np.linalg.norm(A, 2)
    G = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)  # any G: the VJP is linear in it
    g = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    c = complex(rng.uniform(0.5, 1.0), rng.uniform(-0.3, 0.3))
    return G, g, c


def _rel(x, ref):
    x, ref = x.cpu().numpy(), ref.cpu().numpy()
    return float(np.abs(x - ref).max() / np.abs(ref).max())


def test_noalloc_vjp_matches_workspace_vjp():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    dev = torch.device("cuda", 0)
    ensure_device_ready(dev)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    cases = []
    for seed, shape in ((1, (12, 9, 10, 7)), (2, (30, 25, 20))):
        G, g, c = _case(seed, shape)
        Gt = torch.as_tensor(G, device=dev)
        gt = torch.as_tensor(g, device=dev)
        ct = torch.tensor([c], dtype=torch.complex128, device=dev)
        ref = device_vjp(Gt, ct, gt, batched=False)
        D = len(shape)
        out = [torch.full(s, complex("nan"), dtype=torch.complex128, device=dev) for s in ((D, D), (D,), (1,))]
        cases.append((shape, Gt, gt, ct, ref, out))
    torch.cuda.synchronize()
    # both calls queued in order on one stream, no synchronisation in between
    for shape, Gt, gt, ct, _, (dA, db, dc) in cases:
        D = len(shape)
        sh = (ctypes.c_int64 * D)(*shape)
        rc = lib.mm_hermite_vjp_noalloc(D, sh, Gt.data_ptr(), ct.data_ptr(), gt.data_ptr(), dA.data_ptr(),
                                        db.data_ptr(), dc.data_ptr(), stream)
        assert rc == 0, lib.mm_status_string(rc)
    torch.cuda.synchronize()
    for _, _, _, _, ref, (dA, db, dc) in cases:
        assert _rel(dA, ref[0]) < VJP_TOL
        assert _rel(db, ref[1]) < VJP_TOL
        assert abs(dc[0].item() - ref[2].item()) <= VJP_TOL * abs(ref[2].item())


def test_noalloc_rejects_oversized_scratch():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = _lib.load()
    sh = (ctypes.c_int64 * 1)(1 << 20)  # sqrt tables alone need 24 MiB
    rc = lib.mm_hermite_vjp_noalloc(1, sh, None, None, None, None, None, None, None)
    assert rc == 3  # MM_ERR_TOO_LARGE
    sh = (ctypes.c_int64 * 2)(8, 8)  # fits, but a null pointer: rejected before the array is touched
    rc = lib.mm_hermite_vjp_noalloc(2, sh, None, None, None, None, None, None, None)
    assert rc == 1  # MM_ERR_INVALID_ARG

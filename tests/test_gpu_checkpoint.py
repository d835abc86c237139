"""Checkpointed VJP (``mm_hermite_vjp_checkpointed``, ``hermite_renormalized_autograd(checkpoint=K)``).

The reference's JAX VJP keeps the whole G as its residual (mrmustard/math/jax_vjps/hermite.py:80-81)
and ``vanilla_vjp_numba`` reads it (gradients.py:25-82).  The checkpointed path keeps slab 0 and the
two slabs before every K-th slab along axis 0, and recomputes G K slabs at a time in the backward.
Its gradients must agree with the full-G VJP and with the oracle to the VJP tolerance, for every
segment length (K = 2, K not dividing the cutoff, K >= the cutoff, one slab), and the residual must
stay below a stated memory cap on a shape whose G exceeds it.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

import mrmustard_gb300 as mm
from test_gpu_hermite import VJP_TOL, cn, dm_triple, rel, takagi

pytestmark = pytest.mark.gpu


def _vjp_pair(cuda, A, b, c, shape, K, seed):
    At, bt = torch.as_tensor(A, device=cuda), torch.as_tensor(b, device=cuda)
    ct = torch.tensor(c, dtype=torch.complex128, device=cuda)
    g = torch.as_tensor(cn(shape, seed), device=cuda)
    G = mm.device_fwd(At, bt, ct, shape)
    full = mm.device_vjp(G, ct, g, batched=False)
    ck = mm.device_checkpoint_save(G, shape, K, batched=False)
    assert ck.numel() == mm.checkpoint_elems(shape, K)
    part = mm.device_vjp_checkpointed(At, bt, ct, ck, g, shape, K, batched=False)
    return G, g, full, part


@pytest.mark.parametrize("shape,K", [((30, 30, 30, 30), 2), ((30, 30, 30, 30), 7), ((30, 30, 30, 30), 30),
                                     ((30, 30, 30, 30), 45), ((12, 9, 10, 7), 4), ((9,), 3), ((5, 6), 2),
                                     ((1, 7, 6), 2), ((40, 3), 6), ((6, 5, 4, 3, 3), 3)])
def test_checkpointed_vjp_matches_full_and_oracle(cuda, oracle_lib, shape, K):
    D = len(shape)
    A, b, _ = takagi(D, 0.8, 900 + D * 10 + K)
    c = 0.8 + 0.3j
    G, g, full, part = _vjp_pair(cuda, A, b, c, shape, K, 77 + K)
    rA, rb, rc = oracle_lib.vjp(G.cpu().numpy(), c, g.cpu().numpy())
    for x, y, r in zip(part[:2], full[:2], (rA, rb)):
        assert rel(x, y.cpu().numpy()) < VJP_TOL, (shape, K)
        assert rel(x, r) < VJP_TOL, (shape, K)
    assert abs(part[2].item() - full[2].item()) <= VJP_TOL * abs(rc)
    assert abs(part[2].item() - rc) <= VJP_TOL * abs(rc)


def test_checkpointed_vjp_dm_triple_cutoff50(cuda, oracle_lib):
    """The ill-conditioned density-matrix triple at cutoff 50 (the recurrence amplifies rounding):
    recomputed segments stay within the tolerance of the full-G VJP."""
    A, b, c = dm_triple(4, 0.89, 4292)
    shape = (50,) * 4
    G, g, full, part = _vjp_pair(cuda, A, b, c, shape, 8, 5)
    for x, y in zip(part, full):
        assert rel(x, y.cpu().numpy()) < VJP_TOL


def test_checkpoint_rejects_bad_segments(cuda):
    with pytest.raises(ValueError):
        mm.checkpoint_elems((10, 10), 1)
    At = torch.eye(2, dtype=torch.complex128, device=cuda) * 0.1
    bt = torch.zeros(2, dtype=torch.complex128, device=cuda)
    ct = torch.ones((), dtype=torch.complex128, device=cuda)
    with pytest.raises(ValueError):
        mm.hermite_renormalized_autograd(At, bt, ct, (4, 4), checkpoint=1)
    with pytest.raises(ValueError):
        mm.hermite_renormalized_autograd(At, bt, ct, (4, 4), stable=True, checkpoint=3)


def test_checkpointed_autograd_under_memory_cap(cuda, oracle_lib):
    """4 modes at cutoff 40: G is 41 MB; with checkpoint=8 the autograd residual (checkpoint slabs
    plus A, b, c) must stay under a 10 MB cap, and with G dropped by the caller after the loss the
    backward's peak device memory must be lower than the full-G backward's by more than 0.4 G (G
    minus the residual and the recompute window of K + 2 slabs).  The cotangent itself is as large
    as G in both.  Gradients equal the full-G autograd's and the oracle's to the VJP tolerance."""
    CAP = 10 * 2 ** 20
    shape = (40,) * 4
    A, b, _ = takagi(4, 0.8, 4343)
    c = 0.95 + 0.1j
    g = torch.as_tensor(cn(shape, 4344), device=cuda)
    G_bytes = 16 * 40 ** 4
    assert G_bytes > CAP

    def run(checkpoint):
        At = torch.as_tensor(A, device=cuda).requires_grad_(True)
        bt = torch.as_tensor(b, device=cuda).requires_grad_(True)
        ct = torch.tensor(c, dtype=torch.complex128, device=cuda, requires_grad=True)
        G = mm.hermite_renormalized_autograd(At, bt, ct, shape, checkpoint=checkpoint)
        loss = (G * g).sum().real  # grad_output of G: g (conjugated below: holomorphic VJP)
        saved = G.grad_fn.saved_tensors if checkpoint else None
        Gh = G.detach().cpu().numpy()
        del G
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        loss.backward()
        torch.cuda.synchronize()
        peak = torch.cuda.max_memory_allocated()
        return At.grad.cpu().numpy(), bt.grad.cpu().numpy(), ct.grad.item(), Gh, saved, peak

    dA0, db0, dc0, Gh, _, peak_full = run(None)
    dA1, db1, dc1, _, saved, peak_ck = run(8)
    residual = sum(t.numel() * t.element_size() for t in saved)
    assert residual <= CAP, residual
    assert peak_ck < peak_full - 0.4 * G_bytes, (peak_ck, peak_full, G_bytes)
    assert rel(dA1, dA0) < VJP_TOL and rel(db1, db0) < VJP_TOL and abs(dc1 - dc0) <= VJP_TOL * abs(dc0)
    # torch's gradient of Re(sum(G g)) w.r.t. A is conj(vanilla_vjp(G, c, g)) for the holomorphic map
    rA, rb, rc = oracle_lib.vjp(Gh, c, g.cpu().numpy())
    assert rel(dA1, np.conj(rA)) < VJP_TOL and rel(db1, np.conj(rb)) < VJP_TOL
    assert abs(dc1 - np.conj(rc)) <= VJP_TOL * abs(rc)


def test_checkpointed_batched_autograd(cuda):
    """Batched instances (B, D, D) with checkpoints: gradients equal the full-G batched autograd's."""
    B, shape = 3, (14, 11, 9)
    trip = [takagi(3, 0.8, 4500 + k) for k in range(B)]
    gt = torch.as_tensor(cn((B,) + shape, 4510), device=cuda)
    grads = []
    for ck in (None, 3):
        A = torch.as_tensor(np.stack([t[0] for t in trip]), device=cuda).requires_grad_(True)
        b = torch.as_tensor(np.stack([t[1] for t in trip]), device=cuda).requires_grad_(True)
        c = torch.full((B,), 0.9 + 0.1j, dtype=torch.complex128, device=cuda).requires_grad_(True)
        G = mm.hermite_renormalized_autograd(A, b, c, shape, checkpoint=ck)
        (G * gt).sum().real.backward()
        grads.append((A.grad.cpu().numpy(), b.grad.cpu().numpy(), c.grad.cpu().numpy()))
    for x, y in zip(*grads):
        assert rel(x, y) < VJP_TOL

"""``torch.autograd.Function`` around the GB300 forward and VJP.

Counterpart of the reference's JAX ``custom_vjp`` (mrmustard/math/jax_vjps/hermite.py:47-105
single, :113-175 batched), minus its host round-trips: G, the residual and the gradients
stay on the device.

Convention.  The reference VJP is holomorphic: it returns sum_u g_u dG_u/dtheta with the
cotangent g unconjugated (jax_vjps/hermite.py:91-101; gradients.py:25-82).  PyTorch passes
grad_output = dL/dRe(G) + i dL/dIm(G) and expects the same form for the inputs, which for a
holomorphic map is grad_in = conj(sum_u conj(grad_out_u) dG_u/dtheta).  So ``backward`` returns
conj(vjp(G, c, conj(grad_out))).  Like the reference, dL/dA is the symmetrised gradient
(dLdA + dLdA^T)/2 (gradients.py:82), i.e. A is treated as a symmetric matrix.
"""

from __future__ import annotations

import torch

from .hermite import device_checkpoint_save, device_fwd, device_vjp, device_vjp_checkpointed

__all__ = ["HermiteRenormalizedFn", "hermite_renormalized_autograd"]


class HermiteRenormalizedFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, b, c, shape, stable, checkpoint):
        batched = A.dim() == 3
        cc = c.detach().to(torch.complex128).contiguous()
        Ad = A.detach().to(torch.complex128).contiguous()
        bd = b.detach().to(torch.complex128).contiguous()
        G = device_fwd(Ad, bd, cc, tuple(shape), bool(stable))
        ctx.batched = batched
        ctx.c_shape = c.shape
        ctx.shape = tuple(shape)
        ctx.checkpoint = checkpoint
        if checkpoint:
            # residual: checkpoint slabs (about 2/K of G) plus the inputs that regenerate the rest
            ctx.save_for_backward(Ad, bd, cc, device_checkpoint_save(G, shape, checkpoint, batched))
        else:
            ctx.save_for_backward(G, cc)
        return G

    @staticmethod
    def backward(ctx, grad):
        if ctx.checkpoint:
            A, b, c, ck = ctx.saved_tensors
            dA, db, dc = device_vjp_checkpointed(A, b, c, ck, grad.conj(), ctx.shape, ctx.checkpoint, ctx.batched)
        else:
            G, c = ctx.saved_tensors
            dA, db, dc = device_vjp(G, c, grad.conj(), ctx.batched)  # device_vjp materialises the conj view
        return dA.conj(), db.conj(), dc.conj().reshape(ctx.c_shape), None, None, None


def hermite_renormalized_autograd(A, b, c, shape, stable: bool = False, checkpoint: int | None = None):
    """Differentiable G(A, b, c) for device tensors; A (D,D) or (B,D,D), b (D,) or (B,D), c () or (B,).

    ``checkpoint=K`` (K >= 2): keep only checkpoint slabs of G for the backward (slab 0 and the two
    slabs before every K-th slab along axis 0, about 2/K of G) and recompute the rest there, K slabs
    at a time (mm_hermite_vjp_checkpointed), instead of keeping the whole G as the reference's JAX
    VJP does (jax_vjps/hermite.py:80-81).  Vanilla recurrence only."""
    if checkpoint is not None:
        checkpoint = int(checkpoint)
        if checkpoint < 2:
            raise ValueError("checkpoint must be an int >= 2 (slabs per recomputed segment)")
        if stable:
            raise ValueError("the checkpointed backward recomputes the vanilla recurrence; stable=True is not "
                             "supported with checkpoint")
    return HermiteRenormalizedFn.apply(A, b, c, tuple(int(s) for s in shape), bool(stable), checkpoint)

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

from .hermite import device_fwd, device_vjp

__all__ = ["HermiteRenormalizedFn", "hermite_renormalized_autograd"]


class HermiteRenormalizedFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, A, b, c, shape, stable):
        batched = A.dim() == 3
        cc = c.detach().to(torch.complex128).contiguous()
        G = device_fwd(A.detach().to(torch.complex128).contiguous(), b.detach().to(torch.complex128).contiguous(),
                       cc, tuple(shape), bool(stable))
        ctx.save_for_backward(G, cc)
        ctx.batched = batched
        ctx.c_shape = c.shape
        return G

    @staticmethod
    def backward(ctx, grad):
        G, c = ctx.saved_tensors
        dA, db, dc = device_vjp(G, c, grad.conj(), ctx.batched)  # device_vjp materialises the conj view
        return dA.conj(), db.conj(), dc.conj().reshape(ctx.c_shape), None, None


def hermite_renormalized_autograd(A, b, c, shape, stable: bool = False):
    """Differentiable G(A, b, c) for device tensors; A (D,D) or (B,D,D), b (D,) or (B,D), c () or (B,)."""
    return HermiteRenormalizedFn.apply(A, b, c, tuple(int(s) for s in shape), bool(stable))

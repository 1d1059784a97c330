"""``torch.autograd.Function`` over the engine's energy + adjoint-force ABI.

``PesFunction.apply(xp, pes)`` returns F + Vpp (Rydberg) for a pes made with
``make_pes(..., forces=True)``: a scalar for xp (n, 3), a (B,) vector for a
batch (B, n, 3).  F = E - sigma S is the free energy of ``pes.value_and_grad``
(E itself without smearing), so that backward is the derivative of forward
under smearing too.  Its backward multiplies the incoming gradient (per
configuration) by dF/dxp from ``hqcgb_forces`` + the Ewald gradient, so
``torch.autograd.grad`` works through the SCF like ``jax.grad(make_pes(...))``
does for the reference's differentiable parts.  For a pes made with
``gamma=False``, ``PesFunction.apply(xp, pes, kpt)`` (kpt (3,) or (B, 3) in
1/Bohr) differentiates the single-k free energy with respect to xp.
"""
import torch


class PesFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xp, pes, kpt=None):
        E, g = pes.value_and_grad(xp) if kpt is None else pes.value_and_grad(xp, kpt)
        ctx.save_for_backward(g.to(device=xp.device, dtype=xp.dtype))
        if E.dim() > 0 and xp.dim() == 2:  # one configuration over several k-points
            ctx.kmesh = True
        return E.to(device=xp.device, dtype=xp.dtype)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        grad = gout[..., None, None] * g
        if getattr(ctx, "kmesh", False):
            grad = grad.sum(dim=0)  # the shared positions collect every k-point's gradient
        return grad, None, None


def pes_energy(xp, pes, kpt=None):
    return PesFunction.apply(xp, pes, kpt)

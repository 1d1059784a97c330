"""``torch.autograd.Function`` over the engine's energy + adjoint-force ABI.

``PesFunction.apply(xp, pes)`` returns F + Vpp (Rydberg) for a pes made with
``make_pes(..., forces=True)``: a scalar for xp (n, 3), a (B,) vector for a
batch (B, n, 3).  F = E - sigma S is the free energy of ``pes.value_and_grad``
(E itself without smearing), so that backward is the derivative of forward
under smearing too.  Its backward multiplies the incoming gradient (per
configuration) by dF/dxp from ``hqcgb_forces`` + the Ewald gradient, so
``torch.autograd.grad`` works through the SCF like ``jax.grad(make_pes(...))``
does for the reference's differentiable parts.
"""
import torch


class PesFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xp, pes):
        E, g = pes.value_and_grad(xp)
        ctx.save_for_backward(g.to(device=xp.device, dtype=xp.dtype))
        return E.to(device=xp.device, dtype=xp.dtype)

    @staticmethod
    def backward(ctx, gout):
        (g,) = ctx.saved_tensors
        return gout[..., None, None] * g, None


def pes_energy(xp, pes):
    return PesFunction.apply(xp, pes)

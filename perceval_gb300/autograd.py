"""SLOS output probabilities as a differentiable torch function of the unitary.

``slos_probabilities(U, input_state)`` returns every output probability of ``input_state``
through the unitaries U (batch x m x m complex128, or one m x m unitary) as a float64
tensor (outputs x batch, descending-lexicographic output order).  Its backward pass is
the hand-written SLOS adjoint (``pcvl_slos_backward``): for the upstream gradient w of the
probabilities it returns dL/dU for L = sum w p in torch's convention for complex inputs
(dL/dRe U + i dL/dIm U), so ``U`` may come from any differentiable torch expression (for
example ``components.mesh.clements_mesh_unitary`` of MZI phases) and the chain rule
reaches its parameters.  The forward keeps every photon layer resident for the adjoint.
"""
from __future__ import annotations

import torch

from . import _native


class SlosProbabilities(torch.autograd.Function):
    """Forward: SLOS probabilities of one input state (a plan with every layer kept);
    backward: the SLOS adjoint of that plan."""

    @staticmethod
    def forward(ctx, U: torch.Tensor, input_state, precision):
        batched = U.dim() == 3
        Ub = U.detach().contiguous() if batched else U.detach().contiguous()[None]
        B, m = Ub.shape[0], Ub.shape[-1]
        plan = _native.SlosPlan(m, list(input_state), batch=B, keep_layers=True, precision=precision)
        plan.forward(Ub)
        probs = plan.probabilities().view(plan.count, B)
        ctx.plan, ctx.batched = plan, batched
        return probs if batched else probs[:, 0]

    @staticmethod
    def backward(ctx, grad_p: torch.Tensor):
        plan = ctx.plan
        w = grad_p.contiguous().to(torch.float64)
        if not ctx.batched:
            w = w[:, None].contiguous()
        g = plan.backward(w.reshape(-1)).view(plan.batch, plan.m, plan.m)
        plan.close()
        ctx.plan = None
        return (g if ctx.batched else g[0]), None, None


def slos_probabilities(U: torch.Tensor, input_state, precision="fp64") -> torch.Tensor:
    """Differentiable SLOS probabilities of ``input_state`` through U (see module doc)."""
    if not (U.is_cuda and U.dtype == torch.complex128):
        raise TypeError("U must be a complex128 CUDA tensor")
    return SlosProbabilities.apply(U, tuple(int(v) for v in input_state), precision)

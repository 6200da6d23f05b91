"""The log-likelihood as a differentiable torch function.

``log_likelihood(engine, params)`` evaluates log L for a batch of parameter sets
(float64 CUDA tensor, one row per set, the reference's physical parameter
vector) on the engine's batched kernels. When ``params`` requires a gradient,
the forward call runs the adjoint kernel chain instead (it returns log L and
d log L / d params in one pass, recomputing level opacities rather than storing
them) and keeps the Jacobian rows for ``backward``; otherwise it runs the plain
batched forward. Neglected models (log L = -1e30) get a zero gradient.
"""

from __future__ import annotations

import torch


class LogLikelihood(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params: torch.Tensor, engine) -> torch.Tensor:
        if ctx.needs_input_grad[0]:
            ll, grad, _ = engine.grad_batch(params)
            ctx.save_for_backward(grad)
        else:
            ll, _ = engine.loglike_batch(params.detach())
        return ll

    @staticmethod
    def backward(ctx, grad_ll: torch.Tensor):
        (grad,) = ctx.saved_tensors
        return grad_ll.unsqueeze(1) * grad, None


def log_likelihood(engine, params: torch.Tensor) -> torch.Tensor:
    """log L of every row of ``params`` (B, P); differentiable with respect to ``params``."""
    return LogLikelihood.apply(params, engine)

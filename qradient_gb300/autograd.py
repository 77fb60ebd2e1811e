"""grad_run as a ``torch.autograd.Function``.

When the input needs a gradient, the forward pass runs the adjoint kernel
sequence (``qg_grad``), which produces the expectation value and the full
gradient in one sweep pair, and the backward pass scales that gradient by
the incoming gradient.  When it does not (grad mode off, or an input that
does not require grad), the forward pass runs the forward kernels alone
(``qg_run``), about a third of the adjoint's work.  Angles can be any
float64 CUDA tensor (or a CPU tensor, copied over).

    E = mcclean_expectation(angles, circuit)      # angles [L, n], requires_grad
    E.backward()                                  # angles.grad = dE/dangles

Batched form: ``batched_mcclean_expectation(angles[B, L, n], batch)`` with a
``qradient_gb300.batched.Batch`` of B jobs of one circuit structure.
"""
import torch


class McCleanFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, angles, circuit):
        a = angles.detach().to(torch.float64).reshape(-1)
        if not ctx.needs_input_grad[0]:
            nat = circuit.native()
            e, _ = nat.run(a, circuit._dtype_code, circuit._device())
            return e.reshape(()).to(angles.dtype)
        e, g = circuit.grad_run_tensors(angles=a)
        ctx.save_for_backward(g.reshape(angles.shape).to(angles.dtype))
        return e.reshape(()).to(angles.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g, None


class QaoaFunction(torch.autograd.Function):
    """params [p, 2] (beta, gamma) -> E."""

    @staticmethod
    def forward(ctx, params, circuit):
        import numpy as np

        p = params.detach().to(torch.float64).reshape(-1)
        nat = circuit.native()
        if not ctx.needs_input_grad[0]:
            e, _ = nat.run(p, circuit._dtype_code, circuit._device())
            return e.reshape(()).to(params.dtype)
        op = circuit._grad_op(nat)
        e, g = nat.grad(p, circuit._dtype_code, circuit._device(), op)
        ctx.save_for_backward(g.reshape(params.shape).to(params.dtype))
        return e.reshape(()).to(params.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g, None


class BatchedFunction(torch.autograd.Function):
    """params [B, P] for a Batch of B jobs with P parameters each -> E [B]."""

    @staticmethod
    def forward(ctx, params, batch):
        B = params.shape[0]
        flat = params.detach().to(torch.float64).reshape(-1)
        batch.params_flat[: flat.numel()].copy_(flat)
        e, _ = batch.grad()
        g = batch.grads_flat[: flat.numel()].reshape(params.shape).clone()
        ctx.save_for_backward(g.to(params.dtype))
        return e[:B].clone().to(params.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        shape = [grad_out.shape[0]] + [1] * (g.dim() - 1)
        return grad_out.reshape(shape) * g, None


def _wants_grad(x):
    return torch.is_grad_enabled() and isinstance(x, torch.Tensor) and x.requires_grad


def mcclean_expectation(angles, circuit):
    """E(angles) as a differentiable tensor; a forward run alone when no
    gradient can flow back to ``angles``."""
    if not _wants_grad(angles):
        a = torch.as_tensor(angles).detach().to(torch.float64).reshape(-1)
        e, _ = circuit.native().run(a, circuit._dtype_code, circuit._device())
        return e.reshape(()).to(angles.dtype if isinstance(angles, torch.Tensor) else torch.float64)
    return McCleanFunction.apply(angles, circuit)


def qaoa_expectation(params, circuit):
    """E(params [p, 2]) as a differentiable tensor; a forward run alone when
    no gradient can flow back to ``params``."""
    if not _wants_grad(params):
        p = torch.as_tensor(params).detach().to(torch.float64).reshape(-1)
        e, _ = circuit.native().run(p, circuit._dtype_code, circuit._device())
        return e.reshape(()).to(params.dtype if isinstance(params, torch.Tensor) else torch.float64)
    return QaoaFunction.apply(params, circuit)


def batched_expectation(params, batch):
    return BatchedFunction.apply(params, batch)

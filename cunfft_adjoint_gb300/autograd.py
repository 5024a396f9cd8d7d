"""Differentiable adjoint NFFT: gradients with respect to the sample values y
and the sample times t through a torch.autograd.Function.

    F = adjoint_nfft(t, y, plan, t0, T)      # t: float64, y: plan dtype
    loss = (w * F.abs() ** 2).sum()
    loss.backward()                            # t.grad, y.grad

The backward is the library's hand-written vector-Jacobian product
(cuna2_adjoint_backward): one FFT of the deconvolved upstream gradient to a
real field on the oversampled grid, interpolated at every sample with the
Gaussian kernel (dL/dy) and its derivative (dL/dt).  The forward grid is not
stored; the backward needs only t and y.
"""
import torch


class AdjointNFFTFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, t, y, plan, t0, T):
        F = plan.adjoint(t.detach(), y.detach(), t0, T)
        ctx.save_for_backward(t, y)
        ctx.plan, ctx.t0, ctx.T = plan, t0, T
        return F

    @staticmethod
    def backward(ctx, grad_F):
        t, y = ctx.saved_tensors
        need_t, need_y = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        gy, gt = ctx.plan.backward(t.detach(), y.detach(), grad_F, ctx.t0, ctx.T, need_y, need_t)
        return gt, gy, None, None, None


def adjoint_nfft(t, y, plan, t0, T):
    """F[k + nf/2] = sum_j y_j exp(2 pi i k ((t_j - t0)/T - 1/2)), differentiable in t and y."""
    return AdjointNFFTFunction.apply(t, y, plan, float(t0), float(T))

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


class _BatchFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, t, y, op):
        F = op.bplan(t.detach().reshape(-1), y.detach().reshape(-1)).view(op.B, op.nf)
        ctx.save_for_backward(t, y)
        ctx.op = op
        return F

    @staticmethod
    def backward(ctx, grad_F):
        t, y = ctx.saved_tensors
        op = ctx.op
        need_t, need_y = ctx.needs_input_grad[0], ctx.needs_input_grad[1]
        # all series' vector-Jacobian products in one batched execution
        gy, gt = op.plan.backward_batch(t.detach(), y.detach(), grad_F, op.t0, op.T, need_y, need_t)
        return gt, gy, None


class BatchedAdjointNFFT:
    """Differentiable adjoint NFFTs of B series of N samples each (the
    training form: a batch of light curves per step).

        op = BatchedAdjointNFFT(B, N, nf, R, m, t0, T)   # t0, T: B values
        F = op(t, y)                                      # t (B, N) float64, y (B, N); F (B, nf)

    The forward runs all series in one batched execution (one launch per
    stage for the whole batch); so does the backward (the hand-written VJP,
    cuna2_adjoint_backward_batch).
    """

    def __init__(self, B, N, nf, R=2, m=8, t0=None, T=None, dtype=torch.float32, device=None, graph=False):
        import numpy as np
        from .nfft import AdjointNFFT, BatchAdjointNFFT
        self.B, self.N, self.nf = int(B), int(N), int(nf)
        self.t0 = [0.0] * self.B if t0 is None else [float(v) for v in t0]
        self.T = [1.0] * self.B if T is None else [float(v) for v in T]
        self.bplan = BatchAdjointNFFT(np.full(self.B, self.N), np.full(self.B, self.nf), R, m, self.t0, self.T,
                                      dtype, device, graph)
        self.plan = AdjointNFFT(self.nf, R, m, dtype, device)

    def __call__(self, t, y):
        if t.shape != (self.B, self.N) or y.shape != (self.B, self.N):
            raise ValueError("t and y must be (B, N) = (%d, %d)" % (self.B, self.N))
        return _BatchFunction.apply(t.contiguous(), y.contiguous(), self)

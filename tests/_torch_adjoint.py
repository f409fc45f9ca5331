"""torch.autograd.Function wrappers of the GPU adjoint entry points.  Test
harness only: they let a test write the final-state misfit as an ordinary torch
expression and differentiate it with loss.backward(); the shipped library
exposes the VJPs through the C ABI (wv_rk4_adjoint_device, wv_inverse_vjp_device)
and never depends on torch autograd.

Complex gradients follow torch's convention, dL/dRe + i dL/dIm for a real loss,
which is the cotangent convention of the C entry points."""
import torch


class RK4Steps(torch.autograd.Function):
    """(Ap, Am, A0) at t -> (Ap, Am, A0) after `steps` fixed RK4 steps of dt;
    backward is the checkpointed adjoint (checkpoints every `checkpoint_every`
    steps, recomputation in between)."""

    @staticmethod
    def forward(ctx, Ap, Am, A0, kernel, t, t0, dt, steps, checkpoint_every):
        ctx.kernel = kernel
        ctx.args = (t, t0, dt, steps, checkpoint_every)
        ctx.save_for_backward(Ap, Am, A0)
        y = [x.detach().clone().contiguous() for x in (Ap, Am, A0)]
        kernel.rk4(*y, t, t0, dt, steps)
        return tuple(y)

    @staticmethod
    def backward(ctx, gAp, gAm, gA0):
        Ap, Am, A0 = ctx.saved_tensors
        t, t0, dt, steps, K = ctx.args
        g = [torch.zeros_like(Ap) if x is None else x.contiguous() for x in (gAp, gAm, gA0)]
        out = ctx.kernel.rk4_adjoint(Ap.detach(), Am.detach(), A0.detach(), t, t0, dt, steps, K, *g)
        return (*out, None, None, None, None, None, None)


class WaveVortexToUVWEta(torch.autograd.Function):
    """(Ap, Am, A0) at time t -> fields (u, v, w, eta) [4, Nz, Ny, Nx]; backward
    is the transposed transform (wv_inverse_vjp_device)."""

    @staticmethod
    def forward(ctx, Ap, Am, A0, kernel, t, t0):
        ctx.kernel = kernel
        ctx.args = (t, t0)
        return kernel.transformWaveVortexToUVWEta(t, t0, Ap.detach().contiguous(), Am.detach().contiguous(),
                                                  A0.detach().contiguous())

    @staticmethod
    def backward(ctx, gf):
        t, t0 = ctx.args
        out = ctx.kernel.inverse_vjp(t, t0, gf.contiguous())
        return (*out, None, None, None)

"""Differentiable forward transform.

``radon(f, lp, gpu)`` applies the log-polar Radon transform to a CUDA tensor
f[S, N0, N0] and returns R[S, Nproj, N0].  Its backward is the hand-written
exact discrete transpose of the forward (``lp_fwd_transpose``): transposed
interpolations (the forward's cubic weights, summed in a fixed order without
atomics, so a backward gives the same bits on every call), the conjugate kernel
multiply and the transposed prefilter recursions -- not lprec's approximate
adjoint.  Nothing from the forward is saved (the operator is linear).
"""
import torch


class LpRadon(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f, lp, gpu):
        h = lp._handle(gpu)
        f = f.contiguous()
        R = torch.empty((f.shape[0], h.Nproj, h.N0), dtype=torch.float32, device=f.device)
        lp.fwdp(R, f, gpu)
        ctx.lp = lp
        ctx.gpu = gpu
        return R

    @staticmethod
    def backward(ctx, gR):
        lp, gpu = ctx.lp, ctx.gpu
        h = lp._handle(gpu)
        gR = gR.contiguous().float()
        gf = torch.empty((gR.shape[0], h.N0, h.N0), dtype=torch.float32, device=gR.device)
        lp.fwdp_T(gf, gR, gpu)
        return gf, None, None


def radon(f, lp, gpu=0):
    """Forward transform with autograd support (backward = exact transpose)."""
    return LpRadon.apply(f, lp, gpu)

"""torch.autograd bindings of the residual and of the boundary-pressure
functional, for verifying the discrete adjoint against finite differences and
forward mode (torch.autograd.gradcheck, dot-product tests).

The compute runs on the GPU through the C ABI (rflu_gpu_residual,
rflu_gpu_vjp, rflu_gpu_jvp, rflu_gpu_patch_pressure); tensors crossing this
layer are CPU float64 arrays in the reference layout, cv[nCells, 5].
"""
import numpy as np
import torch


def _np(t):
    return np.ascontiguousarray(t.detach().cpu().numpy(), dtype=np.float64)


class Residual(torch.autograd.Function):
    """rhs = R(cv) of Region.residual; backward = (dR/dcv)^T g by the adjoint
    kernels, forward mode = (dR/dcv) v by the tangent kernels."""

    @staticmethod
    def forward(cv, region):
        rhs, _ = region.residual(_np(cv), with_grad=False)
        return torch.from_numpy(rhs)

    @staticmethod
    def setup_context(ctx, inputs, output):
        cv, region = inputs
        ctx.region = region
        ctx.save_for_backward(cv)
        ctx.save_for_forward(cv)

    @staticmethod
    def backward(ctx, g):
        (cv,) = ctx.saved_tensors
        return torch.from_numpy(ctx.region.vjp(_np(cv), _np(g))), None

    @staticmethod
    def jvp(ctx, cv_dot, _):
        (cv,) = ctx.saved_tensors
        return torch.from_numpy(ctx.region.jvp(_np(cv), _np(cv_dot)))


class PatchPressure(torch.autograd.Function):
    """J = sum over the faces of one boundary patch of p_f |A_f|
    (Region.patch_pressure) with its adjoint gradient."""

    @staticmethod
    def forward(cv, region, ipatch):
        J, _ = region.patch_pressure(_np(cv), ipatch, with_grad=False)
        return torch.tensor(J, dtype=torch.float64)

    @staticmethod
    def setup_context(ctx, inputs, output):
        cv, region, ipatch = inputs
        ctx.region, ctx.ipatch = region, ipatch
        ctx.save_for_backward(cv)

    @staticmethod
    def backward(ctx, g):
        (cv,) = ctx.saved_tensors
        _, grad = ctx.region.patch_pressure(_np(cv), ctx.ipatch, with_grad=True)
        return g * torch.from_numpy(grad), None, None


def residual(cv, region):
    return Residual.apply(cv, region)


def patch_pressure(cv, region, ipatch):
    return PatchPressure.apply(cv, region, ipatch)

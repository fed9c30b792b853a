"""Voxel dose as a differentiable function of the voxel densities.

    dose = voxel_dose(rhor, engine, geometry, n, seed)      # torch tensor, Gy
    loss = ((dose - target) ** 2).sum()
    loss.backward()                                         # rhor.grad = dL/d(rhor)

The forward pass runs n histories through the CUDA engine with the given
relative densities; the backward pass calls the engine's seed-replay adjoint
(egsgpu_adjoint), which replays the same histories instead of storing their
paths.  The engine must not run other histories between the two passes.
"""
import numpy as np
import torch

from . import XYZGeometry


class VoxelDose(torch.autograd.Function):
    @staticmethod
    def forward(ctx, rhor, engine, geometry, n, seed, nbatch):
        r = rhor.detach().to("cpu", torch.float64).numpy().ravel()
        g = XYZGeometry(geometry.xb, geometry.yb, geometry.zb, geometry.med, r)
        engine.set_geometry(g)
        engine.reset()
        engine.run(int(n), nbatch=int(nbatch), seed=int(seed))
        dose, _ = engine.dose()
        ctx.engine, ctx.n, ctx.seed = engine, int(n), int(seed)
        ctx.shape = rhor.shape
        return torch.from_numpy(dose.reshape(tuple(rhor.shape))).to(rhor.device, rhor.dtype)

    @staticmethod
    def backward(ctx, grad_dose):
        gD = grad_dose.detach().to("cpu", torch.float64).numpy().ravel()
        g = ctx.engine.adjoint(gD, ctx.n, seed=ctx.seed)
        grad = torch.from_numpy(np.asarray(g).reshape(tuple(ctx.shape))).to(grad_dose.device, grad_dose.dtype)
        return grad, None, None, None, None, None


def voxel_dose(rhor, engine, geometry, n, seed=1, nbatch=10):
    """Dose per voxel (Gy per source particle) of n histories with relative
    densities `rhor` (a tensor of nvox values); differentiable in rhor."""
    return VoxelDose.apply(rhor, engine, geometry, n, seed, nbatch)

"""A thin torch.autograd.Function over the library's recorded forward run and
hand-written adjoint kernels (pbf_forward_record / pbf_backward).

    x, v = PBFRun.apply(x0, v0, theta, sim, substeps, checkpoint_every)

x0, v0: (n, 4) float32 CUDA tensors (id order); theta: (num_scenes, 4)
float64 tensor of (epsilon, s_corr k, XSPH c, vorticity epsilon) per scene.
The outputs are the state after `substeps` substeps; backward() returns the
gradients with respect to x0, v0 and theta.  Torch is plumbing here: every
substep and every adjoint kernel runs in libpbf_gb300.so.
"""
from __future__ import annotations

import numpy as np
import torch

from .sph import SPH, SPHBatch

PARAMS = SPH.PARAM_NAMES


def _apply_theta(sim: SPH, theta: torch.Tensor) -> None:
    th = theta.detach().double().cpu().numpy().reshape(-1, 4)
    if isinstance(sim, SPHBatch):
        for k in range(sim.num_scenes):
            p = sim.scene_params(k)
            for j, nm in enumerate(PARAMS):
                setattr(p, nm, float(np.float32(th[k, j])))
            sim.set_scene_params(k, p)
    else:
        p = sim.params
        for j, nm in enumerate(PARAMS):
            setattr(p, nm, float(np.float32(th[0, j])))
        sim.set_params(p)


class PBFRun(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x0, v0, theta, sim, substeps: int, checkpoint_every: int = 8):
        assert x0.is_cuda and v0.is_cuda and x0.dtype == torch.float32
        x0c = x0.detach().contiguous()
        v0c = v0.detach().contiguous()
        _apply_theta(sim, theta)
        torch.cuda.synchronize()
        sim.set_state_device(x0c.data_ptr(), v0c.data_ptr())
        sim.forward_record(substeps, checkpoint_every)
        x = torch.empty_like(x0c)
        v = torch.empty_like(v0c)
        sim.get_state_into(x.data_ptr(), v.data_ptr(), 1)
        ctx.sim = sim
        ctx.theta_shape = theta.shape
        ctx.theta_dtype = theta.dtype
        return x, v

    @staticmethod
    def backward(ctx, gx, gv):
        sim = ctx.sim
        gx = torch.zeros_like(gx) if gx is None else gx.contiguous()
        gv = torch.zeros_like(gv) if gv is None else gv.contiguous()
        dx0 = torch.empty_like(gx)
        dv0 = torch.empty_like(gv)
        torch.cuda.synchronize()
        g = sim.backward_device(gx.data_ptr(), gv.data_ptr(), dx0.data_ptr(), dv0.data_ptr())
        gtheta = torch.as_tensor(g, dtype=ctx.theta_dtype).reshape(ctx.theta_shape)
        return dx0, dv0, gtheta, None, None, None


def run(sim: SPH, x0: torch.Tensor, v0: torch.Tensor, theta: torch.Tensor, substeps: int,
        checkpoint_every: int = 8):
    return PBFRun.apply(x0, v0, theta, sim, substeps, checkpoint_every)


def theta_of(sim: SPH) -> torch.Tensor:
    """The current (num_scenes, 4) parameter tensor of a handle."""
    if isinstance(sim, SPHBatch):
        rows = [[getattr(sim.scene_params(k), nm) for nm in PARAMS] for k in range(sim.num_scenes)]
    else:
        rows = [[getattr(sim.params, nm) for nm in PARAMS]]
    return torch.tensor(rows, dtype=torch.float64)

"""The differentiable 32,768-particle scene (32^3 lattice at 0.5h, jittered,
in a 64^3 box, velocities N(0, 0.25^2) from seed A, 4 iterations, dt 0.008)
and its loss, L = mean over particles of |x_N - target|^2, the target being
the final positions of the same run started from seed-B velocities.

Three gradients of L with respect to 64 random components of the initial
velocities and the scalars (CFM epsilon, s_corr k, XSPH c, vorticity
epsilon):
  fd_grads    central differences of the FP64 oracle twin (step 1e-3 on the
              FP32 inputs, relative for the scalars), one pair of full runs
              per coordinate;
  dual_grads  forward-mode dual numbers of the FP64 twin (exact derivatives
              of that floating-point program, 16 directions per run), or
              of the FP32 oracle's own trajectory (fp32=True);
and the GPU's FP32 adjoint (pbf_forward_record + pbf_backward, checkpoints
every 8 substeps) in the tests that import this module.
"""
from __future__ import annotations

import numpy as np

from oracle import scenes as osc

PARAMS = ("epsilon", "tensile_instability_k", "xsph_viscosity_c", "vorticity_epsilon")
N_COORDS = 64


def scene(epsilon: float):
    a, b = osc.diff_32k()
    for s in (a, b):
        s.params.epsilon = epsilon
    return a, b


def coords(n: int, count: int = N_COORDS, seed: int = 5):
    rng = np.random.default_rng(seed)
    flat = rng.choice(3 * n, size=count, replace=False)
    return [(int(f // 3), int(f % 3)) for f in flat]


def target(oracle_mod, b, substeps: int) -> np.ndarray:
    """Final positions of the seed-B run (FP32 oracle: the GPU's own bits)."""
    o = oracle_mod.Oracle(b.params, b.n)
    o.set_state(b.x4, b.v4)
    o.step(substeps)
    return o.get_state()[0][:, :3].astype(np.float64)


def fp64_loss(oracle_mod, params, x4, v4, substeps: int, tgt: np.ndarray) -> float:
    o = oracle_mod.Oracle(params, x4.shape[0], fp64=True)
    o.set_state(x4, v4)
    o.step(substeps)
    x = o.get_state()[0][:, :3]
    return float(np.mean(np.sum((x - tgt) ** 2, axis=1)))


def fd_grads(oracle_mod, a, substeps: int, tgt, cs, params=PARAMS, step: float = 1e-3):
    """Central differences of the FP64 twin; the denominator is the FP32
    perturbation actually applied."""
    out = []
    for what in [("v",) + c for c in cs] + [(p,) for p in params]:
        vals, at = [], []
        for sg in (1, -1):
            pp, vv = a.params.copy(), a.v4.copy()
            if what[0] == "v":
                vv[what[1], what[2]] = np.float32(a.v4[what[1], what[2]] + sg * step)
                at.append(float(vv[what[1], what[2]]))
            else:
                base = getattr(a.params, what[0])
                setattr(pp, what[0], float(np.float32(base * (1 + sg * step))))
                at.append(float(getattr(pp, what[0])))
            vals.append(fp64_loss(oracle_mod, pp, a.x4, vv, substeps, tgt))
        out.append((vals[0] - vals[1]) / (at[0] - at[1]))
    return np.array(out)


def dual_grads(oracle_mod, a, substeps: int, tgt, cs, params=PARAMS, fp32: bool = False):
    """Forward-mode gradients of the loss; fp32=True differentiates the FP32
    oracle's trajectory (the GPU's own, bit for bit) instead of the FP64
    twin's."""
    dirs = [("v",) + c for c in cs] + [(p,) for p in params]
    x, _, xd, _ = oracle_mod.dual_tangents(a.params, a.x4, a.v4, substeps, dirs, fp32=fp32)
    w = (2.0 / a.n) * (x - tgt)
    return np.einsum("nc,knc->k", w, xd)


def rel_err(g, ref, floor: float = 1e-3):
    g = np.asarray(g, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.abs(g - ref) / (np.abs(ref) + floor * np.max(np.abs(ref)))

"""The GPU adjoint on the differentiable 32,768-particle scene as specified:
32^3 lattice in a 64^3 box, velocities N(0, 0.25^2) from seed A, 4 solver
iterations, checkpoints every 8 substeps, loss = mean squared distance of the
final positions to those of the seed-B run; gradients with respect to 64
random initial-velocity components and the four scalars (CFM epsilon,
s_corr k, XSPH c, vorticity epsilon).

Two FP64 references (tests/adjoint_32k.py): central differences of the FP64
oracle twin (step 1e-3) and forward-mode dual numbers of the same twin
(exact derivatives of that program).  The FP32 adjoint must agree with the
dual-number gradients within 1e-3 relative (with a floor of 1e-3 of the
largest component), at a horizon where the two FP64 references agree with
each other:
  - epsilon = 5 (the reference's default CFM epsilon, a stable run): all 64
    substeps;
  - epsilon = 0.01 (the workload's own, unstable: the gradient grows
    ~100-300x per substep): 2 substeps.  Central differences at step 1e-3
    agree with the dual numbers to 1e-6 on the velocity components over 2
    substeps, to 3e-2 over 3 and not at all over 4 (the step leaves the
    linear range); the s_corr k component already needs a step of 1e-5 at 2
    substeps (measured: 1e-3 gives 12% truncation error, 1e-5 gives 1e-6).
"""
import numpy as np
import pytest

import pbf_gb300 as pg
from pbf_gb300 import _capi
from tests import adjoint_32k as A

pytestmark = pytest.mark.gpu

# central differences on a subset at the full horizon (each coordinate is
# two full 64-substep FP64 runs); the dual numbers cover all 64 coordinates
N_FD_LONG = 8


def gpu_grads(a, substeps, tgt, cs, every=8):
    p = _capi.Params.from_buffer_copy(bytes(a.params))
    sim = pg.SPH(a.n, tuple(p.grid), p)
    sim.set_state(a.x4, a.v4)
    sim.forward_record(substeps, every)
    x = sim.positions()[:, :3].astype(np.float64)
    w = np.zeros((a.n, 4), np.float32)
    w[:, :3] = (2.0 / a.n) * (x - tgt)
    _, dv0, g = sim.backward(w, None)
    sim.close()
    return np.array([dv0[i, c] for i, c in cs] + list(np.asarray(g[0], np.float64)))


def test_adjoint_32k_epsilon_5_all_64_substeps(gpu, oracle_mod):
    a, b = A.scene(5.0)
    S = 64
    cs = A.coords(a.n)
    tgt = A.target(oracle_mod, b, S)
    g = gpu_grads(a, S, tgt, cs)
    assert np.all(np.isfinite(g))
    dual = A.dual_grads(oracle_mod, a, S, tgt, cs)
    err = A.rel_err(g, dual)
    assert err.max() < 1e-3, (err.max(), int(err.argmax()))
    sub = cs[:N_FD_LONG]
    fd = A.fd_grads(oracle_mod, a, S, tgt, sub)
    ref = np.concatenate([dual[:N_FD_LONG], dual[-4:]])
    # the two FP64 references agree, and the GPU agrees with the differences
    assert A.rel_err(fd, ref).max() < 1e-3
    assert A.rel_err(np.concatenate([g[:N_FD_LONG], g[-4:]]), fd).max() < 1e-3


def test_adjoint_32k_epsilon_001_two_substeps(gpu, oracle_mod):
    a, b = A.scene(0.01)
    S = 2
    cs = A.coords(a.n)
    tgt = A.target(oracle_mod, b, S)
    g = gpu_grads(a, S, tgt, cs, every=1)
    dual = A.dual_grads(oracle_mod, a, S, tgt, cs)
    fd = A.fd_grads(oracle_mod, a, S, tgt, cs, params=("epsilon", "xsph_viscosity_c",
                                                        "vorticity_epsilon"))
    fd_k = A.fd_grads(oracle_mod, a, S, tgt, [], params=("tensile_instability_k",), step=1e-5)
    fd = np.concatenate([fd[:-3], fd[-3:-2], fd_k, fd[-2:]])
    assert A.rel_err(fd, dual).max() < 1e-3
    err = A.rel_err(g, dual)
    assert err.max() < 1e-3, (err.max(), int(err.argmax()))

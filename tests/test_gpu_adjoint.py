"""GPU adjoint (pbf_forward_record / pbf_backward) against central finite
differences of the FP64 oracle twin.

Loss: a random linear functional of the final state, L = sum w.x_N + sum u.v_N,
so dL/dx_N = w and dL/dv_N = u.  Coordinates: random components of the
initial velocities and positions, and the four scalars (epsilon, s_corr k,
XSPH c, vorticity epsilon).  The FP32 adjoint must match the FP64 central
differences within 1e-3 relative (with an absolute floor of 1e-3 of the
largest gradient, for components that are nearly zero).
"""
import numpy as np
import pytest
import torch

import pbf_gb300 as pg
from pbf_gb300 import scenes

pytestmark = pytest.mark.gpu

PARAMS = pg.SPH.PARAM_NAMES


def scene(eps, substeps=4, iterations=3, vort=True, seed=4):
    x4, v4 = scenes.block((8, 8, 8), origin=(8.0, 8.0, 8.0), seed=seed, vel_uniform=0.5)
    p = scenes.dam_params((24, 24, 24), iterations, epsilon=eps, vorticity=vort)
    p.vorticity_epsilon = 0.05  # large enough that its gradient is well above round-off
    return p, x4, v4, substeps


def loss_fp64(oracle_mod, p, x4, v4, substeps, w, u):
    o = oracle_mod.Oracle(p, x4.shape[0], fp64=True)
    o.set_state(x4, v4)
    o.step(substeps)
    x, v = o.get_state()
    return float(np.sum(w[:, :3] * x[:, :3]) + np.sum(u[:, :3] * v[:, :3]))


def fd(oracle_mod, p, x4, v4, substeps, w, u, what, idx, comp, delta):
    """Central difference; the denominator is the float32 perturbation actually applied."""
    vals = []
    steps = []
    for sgn in (+1, -1):
        pp, xx, vv = p.copy(), x4.copy(), v4.copy()
        if what == "v":
            vv[idx, comp] = np.float32(v4[idx, comp] + sgn * delta)
            steps.append(float(vv[idx, comp]))
        elif what == "x":
            xx[idx, comp] = np.float32(x4[idx, comp] + sgn * delta)
            steps.append(float(xx[idx, comp]))
        else:
            base = getattr(p, what)
            setattr(pp, what, float(np.float32(base * (1 + sgn * delta))))
            steps.append(float(getattr(pp, what)))
        vals.append(loss_fp64(oracle_mod, pp, xx, vv, substeps, w, u))
    return (vals[0] - vals[1]) / (steps[0] - steps[1])


def gpu_grads(p, x4, v4, substeps, w, u, every=2):
    sim = pg.SPH(x4.shape[0], tuple(p.grid), p)
    sim.set_state(x4, v4)
    sim.forward_record(substeps, every)
    dx0, dv0, g = sim.backward(w, u)
    return dx0, dv0, g[0], sim


def check(g, ref, what, rel=1e-3):
    g = np.asarray(g, np.float64)
    ref = np.asarray(ref, np.float64)
    floor = rel * np.max(np.abs(ref))
    err = np.abs(g - ref)
    bad = err > rel * np.abs(ref) + floor
    assert not np.any(bad), f"{what}: gpu {g[bad]} vs fd {ref[bad]} (rel err {err[bad] / np.abs(ref[bad])})"


# With the workload's epsilon = 0.01 the map is violently unstable: the
# gradient grows ~50-100x per substep, the FP32 trajectory leaves the FP64 one,
# and the FP32 adjoint matches FP64 finite differences to ~1e-4 of the gradient
# norm over 2 substeps, ~2% over 3 and O(1) over 4 (measured; conditioning,
# not the adjoint: over 1 substep it agrees to 1e-5).  Each case runs at a
# horizon where FP32 is meaningful; over 2 violent substeps the scalar
# parameters' gradients are held to 1e-2 (measured 5e-3).
@pytest.mark.parametrize("eps,substeps,ptol", [(0.01, 1, 1e-3), (0.01, 2, 1e-2), (5.0, 4, 1e-3)])
def test_adjoint_matches_fp64_finite_differences(gpu, oracle_mod, eps, substeps, ptol):
    p, x4, v4, S = scene(eps, substeps=substeps)
    n = x4.shape[0]
    rng = np.random.default_rng(7)
    w = rng.normal(size=(n, 4)).astype(np.float32)
    u = rng.normal(size=(n, 4)).astype(np.float32) * 0.01
    w[:, 3] = 0
    u[:, 3] = 0
    dx0, dv0, gp, _ = gpu_grads(p, x4, v4, S, w, u)
    coords = [(int(rng.integers(n)), int(rng.integers(3))) for _ in range(10)]
    gv = [dv0[i, c] for i, c in coords]
    fv = [fd(oracle_mod, p, x4, v4, S, w, u, "v", i, c, 1e-3) for i, c in coords]
    check(gv, fv, f"dL/dv0 (eps={eps})")
    coords = [(int(rng.integers(n)), int(rng.integers(3))) for _ in range(6)]
    gx = [dx0[i, c] for i, c in coords]
    fx = [fd(oracle_mod, p, x4, v4, S, w, u, "x", i, c, 1e-4) for i, c in coords]
    check(gx, fx, f"dL/dx0 (eps={eps})")
    fp = [fd(oracle_mod, p, x4, v4, S, w, u, nm, 0, 0, 1e-3) for nm in PARAMS]
    for k, nm in enumerate(PARAMS):
        check([gp[k]], [fp[k]], f"dL/d{nm} (eps={eps})", rel=ptol)


def test_adjoint_without_vorticity_and_checkpoint_spacing(gpu, oracle_mod):
    p, x4, v4, S = scene(5.0, substeps=5, vort=False)
    n = x4.shape[0]
    rng = np.random.default_rng(3)
    w = rng.normal(size=(n, 4)).astype(np.float32)
    w[:, 3] = 0
    u = np.zeros_like(w)
    a = gpu_grads(p, x4, v4, S, w, u, every=1)
    b = gpu_grads(p, x4, v4, S, w, u, every=3)
    c = gpu_grads(p, x4, v4, S, w, u, every=8)
    # the checkpoint spacing only changes what is recomputed, never the result
    for k in range(3):
        assert np.array_equal(a[k], b[k]) and np.array_equal(a[k], c[k])
    coords = [(int(rng.integers(n)), int(rng.integers(3))) for _ in range(8)]
    fv = [fd(oracle_mod, p, x4, v4, S, w, u, "v", i, cc, 1e-3) for i, cc in coords]
    check([a[1][i, cc] for i, cc in coords], fv, "dL/dv0 without vorticity")
    # the backward pass leaves the state at the end of the run
    o = oracle_mod.Oracle(p, n)
    o.set_state(x4, v4)
    o.step(S)
    assert np.array_equal(a[3].positions(), o.get_state()[0])


@pytest.mark.parametrize("tuning", [dict(pair_list_capacity=0), dict(pair_list_capacity=3),
                                    dict(sweep_mode="direct", pair_list_capacity=0),
                                    dict(use_neighbour_lists=True, skin_h=0.2),
                                    dict(sweep_mode="coop"), dict(coop_candidates=100)])
def test_adjoint_independent_of_tuning(gpu, tuning):
    """The reverse sweeps scan once per position set into the pair-list
    buffer and replay it; without pair lists, or with lists that overflow
    (capacity 3), they visit the stencil directly.  The gradients are the same
    bits under every tuning (the forward is bit-identical, and the reverse
    pair terms run in the same order)."""
    p, x4, v4, S = scene(0.01, substeps=3)
    n = x4.shape[0]
    rng = np.random.default_rng(11)
    w = rng.normal(size=(n, 4)).astype(np.float32)
    u = rng.normal(size=(n, 4)).astype(np.float32) * 0.01
    w[:, 3] = 0
    u[:, 3] = 0
    ref = gpu_grads(p, x4, v4, S, w, u)
    sim = pg.SPH(n, tuple(p.grid), p)
    sim.set_tuning(**{"sweep_mode": "masked", **tuning})
    sim.set_state(x4, v4)
    sim.forward_record(S, 2)
    dx0, dv0, g = sim.backward(w, u)
    assert np.array_equal(dx0.view(np.uint32), ref[0].view(np.uint32))
    assert np.array_equal(dv0.view(np.uint32), ref[1].view(np.uint32))
    assert np.array_equal(np.asarray(g[0]), np.asarray(ref[2]))


def test_autograd_function(gpu):
    from pbf_gb300 import autograd
    p, x4, v4, S = scene(5.0, substeps=3)
    sim = pg.SPH(x4.shape[0], tuple(p.grid), p)
    x0 = torch.from_numpy(x4).cuda().requires_grad_(True)
    v0 = torch.from_numpy(v4).cuda().requires_grad_(True)
    theta = autograd.theta_of(sim).requires_grad_(True)
    x, v = autograd.run(sim, x0, v0, theta, S, 2)
    target = x.detach() + 0.1
    loss = ((x - target) ** 2)[:, :3].sum(1).mean()
    loss.backward()
    n = x4.shape[0]
    w = (2.0 / n) * (x - target).detach().cpu().numpy()
    w[:, 3] = 0
    sim2 = pg.SPH(n, tuple(p.grid), p)
    sim2.set_state(x4, v4)
    sim2.forward_record(S, 2)
    dx0, dv0, g = sim2.backward(w, None)
    assert np.allclose(v0.grad.cpu().numpy(), dv0, rtol=1e-5, atol=1e-9)
    assert np.allclose(x0.grad.cpu().numpy(), dx0, rtol=1e-5, atol=1e-9)
    assert np.allclose(theta.grad.numpy(), g, rtol=1e-5, atol=1e-12)


def test_batched_adjoint_matches_single_scenes(gpu):
    sc = scenes.batch_scenes(3, seed=9, iterations=2, nmin=300, nmax=900, box_min=14, box_max=20)
    for k, s in enumerate(sc):
        s.params.xsph_viscosity_c = 0.01 + 0.005 * k
    b = pg.SPHBatch([s.params for s in sc], [s.n for s in sc])
    x4, v4 = scenes.concat_state(sc)
    rng = np.random.default_rng(1)
    w = rng.normal(size=x4.shape).astype(np.float32)
    w[:, 3] = 0
    b.set_state(x4, v4)
    b.forward_record(4, 2)
    bdx, bdv, bg = b.backward(w, None)
    for k, s in enumerate(sc):
        sl = b.scene_slice(k)
        dx0, dv0, g, _ = gpu_grads(s.params, s.x4, s.v4, 4, w[sl], np.zeros_like(w[sl]))
        assert np.allclose(bdv[sl], dv0, rtol=1e-6, atol=1e-9)
        assert np.allclose(bdx[sl], dx0, rtol=1e-6, atol=1e-9)
        assert np.allclose(bg[k], g, rtol=1e-6, atol=1e-12)


def test_adjoint_with_stencils_outside_the_grid(gpu, oracle_mod):
    """Particles predicted below the floor centre their stencil outside the
    grid (neighbourcells.glsl:57), so they may be candidates of a neighbour
    that is not one of theirs.  The reverse sweeps weigh each pair's two
    directions separately; the adjoint must match the exact derivative of the
    same FP32 trajectory (dual numbers on the FP32 oracle) within 1e-3."""
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
    import pin_scenes
    p, x4, v4 = pin_scenes.make("h1_eps5_below_floor")
    n = x4.shape[0]
    S = 2
    rng = np.random.default_rng(5)
    w = rng.normal(size=(n, 4)).astype(np.float32)
    w[:, 3] = 0
    dx0, dv0, gp, _ = gpu_grads(p, x4, v4, S, w, np.zeros_like(w), every=1)
    low = np.flatnonzero(v4[:, 1] < -150)[:6]  # predicted below y = -1 in the first substep
    coords = [(int(i), 1) for i in low] + [(int(rng.integers(n)), int(rng.integers(3))) for _ in range(6)]
    dirs = [("v", i, c) for i, c in coords] + [("x", i, c) for i, c in coords[:4]]
    dirs += [(nm,) for nm in PARAMS]
    x, _, xd, _ = oracle_mod.dual_tangents(p, x4, v4, S, dirs, fp32=True)
    ref = np.einsum("nc,knc->k", w[:, :3].astype(np.float64), xd)
    g = [dv0[i, c] for i, c in coords] + [dx0[i, c] for i, c in coords[:4]] + list(gp)
    check(g, ref, "gradients with stencils outside the grid")


def test_warp_sweeps_match_thread_sweeps(gpu):
    """Collapsed state: the 32,768-particle epsilon = 0.01 run after 40
    substeps holds most particles in coincident piles of 32 or more.  From
    those positions at rest, with epsilon = 5, the reverse sweeps that give
    each particle with a dense stencil a warp (its pair terms summed across
    the lanes) agree with the thread-per-particle sweeps.  The sums run in
    another order (thousands of terms in float), so the two agree to 1e-3 of
    the largest component, not bitwise; each is deterministic."""
    a, _ = scenes.diff_32k()
    n = a.n
    sim = pg.SPH(n, tuple(a.params.grid), a.params)
    sim.set_state(a.x4, a.v4)
    sim.step(40)
    x0, _ = sim.get_state()
    _, cnt = np.unique(x0[:, :3], axis=0, return_counts=True)
    assert cnt[cnt >= 32].sum() > n // 2 and cnt.max() >= 1000  # the piles exist
    v0 = np.zeros_like(x0)
    p = a.params.copy()
    p.epsilon = 5.0
    sim.set_params(p)
    rng = np.random.default_rng(3)
    w = rng.normal(size=(n, 4)).astype(np.float32)
    u = rng.normal(size=(n, 4)).astype(np.float32)
    w[:, 3] = 0
    u[:, 3] = 0
    out = []
    for warp_above in (0xFFFFFFFF, 0, 0):
        sim.set_tuning(adjoint_warp_candidates=warp_above)
        sim.set_state(x0, v0)
        sim.forward_record(4, 2)
        out.append(sim.backward(w, u))
    (dx_t, dv_t, g_t), (dx_w, dv_w, g_w), (dx_w2, dv_w2, g_w2) = out
    assert np.array_equal(dx_w, dx_w2) and np.array_equal(dv_w, dv_w2)  # deterministic
    assert np.array_equal(g_w, g_w2)
    for name, got, want in (("dL/dx0", dx_w, dx_t), ("dL/dv0", dv_w, dv_t)):
        assert np.all(np.isfinite(want[:, :3])), name
        scale = float(np.abs(want[:, :3]).max())
        err = float(np.abs(got[:, :3] - want[:, :3]).max())
        assert err <= 1e-3 * scale, (name, err, scale)
    np.testing.assert_allclose(g_w, g_t, rtol=1e-3, atol=1e-6 * float(np.abs(g_t).max()))

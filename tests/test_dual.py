"""CPU tests of the dual-number (forward-mode) FP64 twin, oracle/pbf_dual.cpp.

The dual simulation runs the oracle's own template on a number type that
carries tangents, so its value part must equal the FP64 twin bit for bit, and
its tangents must agree with central finite differences of the FP64 twin
wherever the map is smooth at the step size.  The GPU adjoint is then checked
against both (tests/test_gpu_adjoint_32k.py).
"""
import numpy as np
import pytest

from oracle import scenes as osc

PARAMS = ("epsilon", "tensile_instability_k", "xsph_viscosity_c", "vorticity_epsilon")


def small(eps, iterations=3):
    x4, v4 = osc.block((8, 8, 8), origin=(8.0, 8.0, 8.0), seed=4, vel_uniform=0.5)
    p = osc.dam_params((24, 24, 24), iterations, epsilon=eps)
    p.vorticity_epsilon = 0.05
    return p, x4, v4


def fp64_loss(oracle_mod, p, x4, v4, S, w, u):
    o = oracle_mod.Oracle(p, x4.shape[0], fp64=True)
    o.set_state(x4, v4)
    o.step(S)
    x, v = o.get_state()
    return float(np.sum(w * x[:, :3]) + np.sum(u * v[:, :3]))


def central(oracle_mod, p, x4, v4, S, w, u, d, step):
    vals, at = [], []
    for sg in (1, -1):
        pp, xx, vv = p.copy(), x4.copy(), v4.copy()
        if d[0] in ("v", "x"):
            arr, src = (vv, v4) if d[0] == "v" else (xx, x4)
            arr[d[1], d[2]] = np.float32(src[d[1], d[2]] + sg * step)
            at.append(float(arr[d[1], d[2]]))
        else:
            base = getattr(p, d[0])
            setattr(pp, d[0], float(np.float32(base * (1 + sg * step))))
            at.append(float(getattr(pp, d[0])))
        vals.append(fp64_loss(oracle_mod, pp, xx, vv, S, w, u))
    return (vals[0] - vals[1]) / (at[0] - at[1])


@pytest.mark.parametrize("eps,S", [(5.0, 4), (0.01, 1)])
def test_dual_twin_matches_fp64_central_differences(oracle_mod, eps, S):
    p, x4, v4 = small(eps)
    n = x4.shape[0]
    rng = np.random.default_rng(7)
    w = rng.normal(size=(n, 3))
    u = rng.normal(size=(n, 3)) * 0.01
    dirs = [("v", int(rng.integers(n)), int(rng.integers(3))) for _ in range(6)]
    dirs += [("x", int(rng.integers(n)), int(rng.integers(3))) for _ in range(4)]
    dirs += [(nm,) for nm in PARAMS]
    xo, vo, xd, vd = oracle_mod.dual_tangents(p, x4, v4, S, dirs)
    # the value part is the FP64 twin, bit for bit
    o = oracle_mod.Oracle(p, n, fp64=True)
    o.set_state(x4, v4)
    o.step(S)
    xf, vf = o.get_state()
    assert np.array_equal(xo, xf[:, :3]) and np.array_equal(vo, vf[:, :3])
    dual = np.array([np.sum(w * xd[k]) + np.sum(u * vd[k]) for k in range(len(dirs))])
    fd = np.array([central(oracle_mod, p, x4, v4, S, w, u, d, 1e-4 if d[0] == "x" else 1e-3)
                   for d in dirs])
    # measured agreement 1e-5 or better; 1e-4 leaves room for the FD truncation
    err = np.abs(dual - fd) / (np.abs(fd) + 1e-3 * np.abs(fd).max())
    assert np.all(err < 1e-4), (dirs, err)


def test_dual_lanes_are_independent(oracle_mod):
    """More directions than one pass holds (16 lanes): each tangent is the
    same whether it shares its pass with others or runs alone."""
    p, x4, v4 = small(5.0, iterations=2)
    n = x4.shape[0]
    dirs = [("v", i * 7 % n, i % 3) for i in range(18)] + [("epsilon",)]
    _, _, xd, vd = oracle_mod.dual_tangents(p, x4, v4, 2, dirs)
    for k in (0, 15, 16, 18):
        _, _, xk, vk = oracle_mod.dual_tangents(p, x4, v4, 2, [dirs[k]])
        assert np.array_equal(xk[0], xd[k]) and np.array_equal(vk[0], vd[k])
    with pytest.raises(ValueError):
        oracle_mod.dual_tangents(p, x4, v4, 1, [("v", n, 0)])

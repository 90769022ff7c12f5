"""CPU tests of the oracle: known-answer tests derived from the reference's
shader source, sort / cell-range unit cases and determinism.

The reference ships no tests or golden vectors, so these KATs are what pins
the oracle: the kernel constants (calclambda.glsl:46,54), the poly6 density
of the rest lattice, the stable (key, id) order of RadixSort, GetHash at and
beyond the grid edges, and the findcells / neighbourcells ranges of
hand-built cell layouts.
"""
import ctypes as C
import math

import numpy as np
import pytest

from pbf_gb300 import scenes
from pbf_gb300._capi import Params


def small_params(grid=(8, 8, 8), iterations=2, **kw):
    p = scenes.dam_params(tuple(g - 1 for g in grid), iterations, **kw)
    return p


def test_params_layout_matches(oracle_mod):
    assert oracle_mod.params_size() == C.sizeof(Params) == 84


def test_kernel_constants(oracle_mod):
    # Wpoly6 normalisation 315/(64 pi), spiky 15/pi, as the shaders write them
    assert abs(1.56668147106 - 315.0 / (64.0 * math.pi)) < 1e-10
    assert abs(4.774648292756860 - 15.0 / math.pi) < 1e-14
    p = small_params()
    o = oracle_mod.Oracle(p, 8)
    c = o.consts()
    assert c["k6"] == np.float32(1.56668147106)
    assert c["kg"] == np.float32(-3.0 * 4.774648292756860)
    assert c["kg_lambda"] == np.float32(-3.0 * 4.774648292756860 * p.one_over_rho_0)
    assert c["h2"] == 1.0
    # h = 2 folds h^9 and h^6 into the constants
    p2 = small_params()
    p2.h = 2.0
    c2 = oracle_mod.Oracle(p2, 8).consts()
    assert c2["k6"] == np.float32(1.56668147106 / 512.0)
    assert c2["kg"] == np.float32(-3.0 * 4.774648292756860 / 64.0)


def test_wpoly6_and_rest_density():
    # W(0; h) = 1.56668147106 / h^3
    assert scenes.wpoly6(0.0, 1.0) == pytest.approx(1.56668147106, rel=1e-15)
    assert scenes.wpoly6(0.0, 2.0) == pytest.approx(1.56668147106 / 8.0, rel=1e-15)
    assert scenes.wpoly6(1.0, 1.0) == 0.0
    assert scenes.wpoly6(1.5, 1.0) == 0.0
    # lattice spacing 0.5, h = 1: 6 at 0.5, 12 at sqrt(.5), 8 at sqrt(.75), 6 at 1 (W = 0)
    expect = 1.56668147106 * (6 * 0.75 ** 3 + 12 * 0.5 ** 3 + 8 * 0.25 ** 3)
    assert scenes.rest_density(1.0, 0.5) == pytest.approx(expect, rel=1e-14)
    # s_corr scale 1 / W(0.2h)
    assert scenes.wpoly6(0.2, 1.0) == pytest.approx(1.56668147106 * 0.96 ** 3, rel=1e-14)


def test_rest_lattice_has_zero_constraint(oracle_mod):
    """An unjittered interior lattice point has rho = rho0, so C = 0 and lambda = 0."""
    lat = (12, 12, 12)
    x4, v4 = scenes.block(lat, jitter=0.0, origin=(10.25, 10.25, 10.25))
    p = scenes.dam_params((40, 40, 40), 1, vorticity=False)
    p.gravity = 0.0
    o = oracle_mod.Oracle(p, x4.shape[0], fp64=True)
    o.set_state(x4, v4)
    o.step(1)
    lam, xp = o.get_solver()
    # interior: at least 2 lattice spacings from every face
    lo, hi = 10.25 + 2 * 0.5, 10.25 + (lat[0] - 3) * 0.5
    inner = np.all((xp[:, :3] >= lo - 1e-9) & (xp[:, :3] <= hi + 1e-9), axis=1)
    assert inner.sum() > 100
    # C = rho * fl32(1/rho0) - 1 is the float32 rounding error of 1/rho0 only
    oorho = float(np.float32(p.one_over_rho_0))
    c_round = abs(scenes.rest_density(1.0, 0.5) * oorho - 1.0)
    assert c_round < 2.0 ** -23
    assert np.max(np.abs(lam[inner])) <= c_round  # denominator > 1
    assert np.ptp(lam[inner]) < 1e-15


def test_keys_at_and_beyond_grid_edges(oracle_mod):
    """GetHash: key = cx + cy*Gx*Gz + cz*Gx with cell = min(int(clamp(x,0,G)), G-1)."""
    G = (5, 4, 3)
    p = small_params(grid=G)
    pos = np.array([
        [0.0, 0.0, 0.0], [0.999, 0.0, 0.0], [1.0, 0.0, 0.0], [-3.0, -0.5, -7.0],
        [4.5, 0.0, 0.0], [5.0, 0.0, 0.0], [9.0, 0.0, 0.0], [0.0, 3.99, 0.0],
        [0.0, 4.0, 0.0], [0.0, 0.0, 2.5], [0.0, 0.0, 3.0], [np.nan, 1.5, np.inf],
    ], np.float32)
    n = pos.shape[0]
    x4 = np.zeros((n, 4), np.float32)
    x4[:, :3] = pos
    p.gravity = 0.0
    p.num_solver_iterations = 0
    p.vorticity_confinement = 0
    for a in range(3):
        p.wall_lo[a] = -100.0
        p.wall_hi[a] = 100.0
    o = oracle_mod.Oracle(p, n)
    o.set_state(x4, np.zeros_like(x4))
    o.step(1)
    kb, _, _ = o.get_sort()

    def key(c):
        return c[0] + c[1] * G[0] * G[2] + c[2] * G[0]

    expect = [key(c) for c in [
        (0, 0, 0), (0, 0, 0), (1, 0, 0), (0, 0, 0), (4, 0, 0), (4, 0, 0), (4, 0, 0), (0, 3, 0),
        (0, 3, 0), (0, 0, 2), (0, 0, 2), (0, 1, 2)]]
    assert list(kb) == expect


@pytest.mark.parametrize("numbits", [1, 7, 8, 9, 17, 24, 32])
def test_oracle_sort_is_stable_key_then_id(oracle_mod, numbits):
    rng = np.random.default_rng(numbits)
    n = 5000
    keys = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    keys[::7] = keys[3]  # many ties
    ko, po = oracle_mod.radix_sort(keys, numbits)
    mask = np.uint32(0xFFFFFFFF if numbits == 32 else (1 << numbits) - 1)
    ref = np.argsort(keys & mask, kind="stable")
    assert np.array_equal(po, ref.astype(np.uint32))
    assert np.array_equal(ko, keys[ref])


def test_substep_sort_matches_numpy_stable_argsort(oracle_mod):
    sc = scenes.plain_16k()
    o = oracle_mod.Oracle(sc.params, sc.n)
    o.set_state(sc.x4, sc.v4)
    o.step(1)
    kb, sk, pm = o.get_sort()
    ref = np.argsort(kb, kind="stable")
    assert np.array_equal(pm, ref.astype(np.uint32))
    assert np.array_equal(sk, kb[ref])


def test_cell_ranges_hand_built(oracle_mod):
    """findcells with Q3 fixed: start of the first cell is 0, end of the last is n."""
    G = (4, 3, 2)
    p = small_params(grid=G)
    p.gravity = 0.0
    p.num_solver_iterations = 0
    p.vorticity_confinement = 0
    # cells (x, y, z): two particles in (0,0,0), one in (3,0,0), three in (1,2,1), one in (3,2,1)
    cells = [(0, 0, 0), (1, 2, 1), (0, 0, 0), (3, 0, 0), (1, 2, 1), (3, 2, 1), (1, 2, 1)]
    x4 = np.zeros((len(cells), 4), np.float32)
    for i, c in enumerate(cells):
        x4[i, :3] = np.array(c, np.float32) + 0.5
    o = oracle_mod.Oracle(p, len(cells))
    o.set_state(x4, np.zeros_like(x4))
    o.step(1)
    st, en = o.get_cells()

    def key(c):
        return c[0] + c[1] * G[0] * G[2] + c[2] * G[0]

    expect_st = np.full(G[0] * G[1] * G[2], -1, np.int32)
    expect_en = np.full(G[0] * G[1] * G[2], -1, np.int32)
    # sorted order by key then id: (0,0,0) ids 0,2 | (3,0,0) id 3 | (1,2,1) ids 1,4,6 | (3,2,1) id 5
    for c, s, e in [((0, 0, 0), 0, 2), ((3, 0, 0), 2, 3), ((1, 2, 1), 3, 6), ((3, 2, 1), 6, 7)]:
        expect_st[key(c)] = s
        expect_en[key(c)] = e
    assert np.array_equal(st, expect_st)
    assert np.array_equal(en, expect_en)
    _, _, pm = o.get_sort()
    assert list(pm) == [0, 2, 3, 1, 4, 6, 5]
    # neighbour runs of sorted particle 3 (cell (1,2,1)): rows in (dy, dz) order
    runs = o.get_runs(3)
    # row (dy,dz)=(0,0) -> y=2,z=1, x in 0..2 -> only cell (1,2,1): [3, 6)
    assert tuple(runs[4]) == (3, 6)
    # rows with y=3 are outside the grid (Q4): empty
    for o_ in (6, 7, 8):
        assert runs[o_][0] == runs[o_][1]
    # row (-1,-1) -> y=1, z=0: empty
    assert runs[0][0] == runs[0][1]
    # sorted particle 2 is in cell (3,0,0): row (0,0) covers x in 2..3 of (y=0,z=0) -> [2,3)
    runs2 = o.get_runs(2)
    assert tuple(runs2[4]) == (2, 3)
    # row (0,-1) for particle 0 in cell (0,0,0) is z=-1: empty; row (0,0) covers x 0..1 -> [0,2)
    r0 = o.get_runs(0)
    assert tuple(r0[4]) == (0, 2)
    assert r0[3][0] == r0[3][1]


def test_oracle_deterministic_across_thread_counts(oracle_mod):
    sc = scenes.plain_16k()
    outs = []
    for t in (1, 3, 0):
        o = oracle_mod.Oracle(sc.params, sc.n, threads=t)
        o.set_state(sc.x4, sc.v4)
        o.step(3)
        outs.append(o.get_state())
    for x, v in outs[1:]:
        assert np.array_equal(x, outs[0][0])
        assert np.array_equal(v, outs[0][1])


def test_fp32_against_fp64_twin_one_substep(oracle_mod):
    sc = scenes.plain_16k()
    o32 = oracle_mod.Oracle(sc.params, sc.n)
    o64 = oracle_mod.Oracle(sc.params, sc.n, fp64=True)
    for o in (o32, o64):
        o.set_state(sc.x4, sc.v4)
        o.step(1)
    x32, v32 = o32.get_state()
    x64, v64 = o64.get_state()
    err = np.max(np.abs(x32[:, :3].astype(np.float64) - x64[:, :3]))
    # FP32 rounding of positions near 16h, amplified through 3 Jacobi iterations
    assert err < 1e-3, err


def test_zero_iterations_and_no_vorticity(oracle_mod):
    """With 0 iterations the substep is free fall: x = x*, v = (x* - x)/dt."""
    sc = scenes.plain_16k()
    p = sc.params.copy()
    p.num_solver_iterations = 0
    p.vorticity_confinement = 0
    o = oracle_mod.Oracle(p, sc.n)
    o.set_state(sc.x4, sc.v4)
    o.step(1)
    x, v = o.get_state()
    dt = np.float32(p.timestep)
    vy = sc.v4[:, 1] - np.float32(p.gravity) * dt
    xs = sc.x4[:, 1] + dt * vy
    assert np.array_equal(x[:, 1], xs.astype(np.float32))
    assert np.array_equal(v[:, 1], ((xs - sc.x4[:, 1]) / dt).astype(np.float32))


def test_oracle_scenes_equal_the_product_generator(oracle_mod, product_lib):
    """bench.py's CPU reference arm builds its scenes with the oracle's own
    generator (so it never loads the product library); the scenes and the
    folded constants must be the same bytes as the product's."""
    from oracle import scenes as oscenes
    assert C.sizeof(oscenes.Params) == C.sizeof(Params)
    assert [f for f, _ in oscenes.Params._fields_] == [f for f, _ in Params._fields_]
    for name in ("plain_16k", "plain_262k", "plain_2m"):
        a, b = getattr(oscenes, name)(), getattr(scenes, name)()
        assert a.name == b.name and a.substeps == b.substeps and a.meta == b.meta
        assert bytes(a.params) == bytes(b.params), name
        assert np.array_equal(a.x4.view(np.uint32), b.x4.view(np.uint32)), name
        assert np.array_equal(a.v4.view(np.uint32), b.v4.view(np.uint32)), name
    (oa, ob), (pa, pb) = oscenes.diff_32k(), scenes.diff_32k()
    for u, w in ((oa, pa), (ob, pb)):
        assert bytes(u.params) == bytes(w.params)
        assert np.array_equal(u.x4.view(np.uint32), w.x4.view(np.uint32))
        assert np.array_equal(u.v4.view(np.uint32), w.v4.view(np.uint32))
    # uniform and normal velocity draws, other origins and spacings
    for kw in ({"vel_uniform": 0.5, "seed": 3}, {"vel_sigma": 0.25, "seed": 9, "spacing": 0.37},
               {"vel_uniform": 0.2, "vel_sigma": 0.1, "origin": (1.5, 0.25, 7.0), "seed": 2**63 + 5}):
        xa, va = oscenes.block((5, 7, 3), **kw)
        xb, vb = scenes.block((5, 7, 3), **kw)
        assert np.array_equal(xa.view(np.uint32), xb.view(np.uint32))
        assert np.array_equal(va.view(np.uint32), vb.view(np.uint32))
    for h, s in ((1.0, 0.5), (2.0, 0.94), (0.7, 0.33)):
        assert oscenes.rest_density(h, s) == scenes.rest_density(h, s)
        assert oscenes.wpoly6(0.3 * h, h) == scenes.wpoly6(0.3 * h, h)
    for grid in ((128, 64, 128), (20, 8, 40)):
        po, pp = oscenes.Params(), Params()
        assert oracle_mod.load().pbfo_params_default((C.c_uint32 * 3)(*grid), C.addressof(po)) == 0
        assert product_lib.pbf_params_default((C.c_uint32 * 3)(*grid), C.byref(pp)) == 0
        assert bytes(po) == bytes(pp)

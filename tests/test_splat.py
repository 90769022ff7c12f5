"""Headless splatting: SurfaceReconstruction's particle depth and thickness
passes (pbf_splat) against the reference's own particledepth / thickness
shaders compiled as C++ (oracle/ref_build.py, fixtures in
tests/golden/ref_splat.npz) and against the CPU oracle (oracle/
pbf_splat_oracle.cpp).

Bar: bit-exact.  Both passes reduce to an order-independent result per pixel
(the smallest clamped depth; an exact count), and every per-fragment value is
one fixed sequence of IEEE binary32 operations, so the GPU, the oracle and the
compiled reference shaders agree bit for bit.
"""
import hashlib
import json
import math
import os
import sys

import numpy as np
import pytest

import oracle
from pbf_gb300 import scenes, splat

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import splat_cases  # noqa: E402


def golden():
    return np.load(os.path.join(HERE, "ref_splat.npz"))


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def test_splat_golden_digest():
    m = json.load(open(os.path.join(HERE, "manifest.json")))
    raw = open(os.path.join(HERE, "ref_splat.npz"), "rb").read()
    assert hashlib.sha256(raw).hexdigest() == m["splat"]["ref_splat.npz"]


@pytest.mark.parametrize("name", splat_cases.CASES)
def test_oracle_matches_reference_golden(oracle_mod, name):
    x4, V, P, dsz, tsz = splat_cases.make(name)
    Vc, Pc = splat_cases.columns(V), splat_cases.columns(P)
    g = golden()
    d = oracle_mod.splat(0, x4, Vc, Pc, *dsz)
    t = oracle_mod.splat(1, x4, Vc, Pc, *tsz)
    assert np.array_equal(bits(d), bits(g[f"{name}_depth"]))
    assert np.array_equal(bits(t), bits(g[f"{name}_thickness"]))
    assert (t > 0).any()  # every case draws something


@pytest.mark.skipif(not oracle.ref_available(), reason="the reference checkout is not on this machine")
def test_oracle_matches_live_reference_shaders(oracle_mod):
    rng = np.random.default_rng(3)
    x4 = np.zeros((2000, 4), np.float32)
    x4[:, :3] = rng.uniform((20, 0, 20), (110, 60, 110), (2000, 3)).astype(np.float32)
    for eye in [(20.0, 10.0, 10.0), (-5.0, 14.0, 22.0)]:
        V = splat.look_at(eye, (0.0, 3.0, 0.0), (0.0, 1.0, 0.0))
        P = splat.perspective(math.radians(45.0), 1.5, 1.0, 200.0)
        Vc, Pc = splat_cases.columns(V), splat_cases.columns(P)
        for p, (w, h) in ((0, (150, 100)), (1, (64, 64))):
            a = oracle_mod.splat(p, x4, Vc, Pc, w, h)
            b = oracle_mod.ref_splat(p, x4, Vc, Pc, w, h)
            assert np.array_equal(bits(a), bits(b)), (eye, p)


DIST = 6.0  # past the distance where clip z / clip w turns negative and clamps to 0


def one_particle_view():
    # a particle at grid (64, 19, 64) sits at world (0, 4, 0); the eye looks
    # at it from DIST units along +z
    x4 = np.array([[64.0, 19.0, 64.0, 0.0]], np.float32)
    V = splat.look_at((0.0, 4.0, DIST), (0.0, 4.0, 0.0), (0.0, 1.0, 0.0))
    P = splat.perspective(math.radians(45.0), 1.0, 1.0, 200.0)
    return x4, V, P


def test_known_answers_one_particle(oracle_mod):
    x4, V, P = one_particle_view()
    Vc, Pc = splat_cases.columns(V), splat_cases.columns(P)
    W = H = 201  # odd: the screen centre is the centre of pixel (100, 100)
    d = oracle_mod.splat(0, x4, Vc, Pc, W, H)
    t = oracle_mod.splat(1, x4, Vc, Pc, W, H)
    # the sprite is a disc of radius 0.1 at distance DIST: on screen
    # 0.1 / DIST * f * W / 2 pixels, f = 1 / tan(22.5 deg)
    rad = 0.1 / DIST / math.tan(math.radians(22.5)) * W / 2
    covered = t > 0
    assert abs(covered.sum() - math.pi * rad * rad) < 2 * math.pi * rad + 4
    assert np.array_equal(covered, d < 1)
    assert set(np.unique(t)) == {0.0, 1.0}
    # the centre fragment is the sphere's front point, DIST - 0.1 from the eye:
    # depth = clip z / clip w of view z = -(DIST - 0.1)
    z = -(DIST - 0.1)
    want = ((-(201.0) / 199.0) * z - 2 * 200.0 / 199.0) / (-z)
    assert abs(d[100, 100] - want) < 2e-6
    assert d[covered].min() == d[100, 100]  # the nearest point of the sphere
    # a second particle at the same place doubles the thickness, not the depth
    x2 = np.concatenate([x4, x4])
    assert np.array_equal(oracle_mod.splat(1, x2, Vc, Pc, W, H), 2 * t)
    assert np.array_equal(bits(oracle_mod.splat(0, x2, Vc, Pc, W, H)), bits(d))


def test_order_independence(oracle_mod):
    x4, V, P, dsz, tsz = splat_cases.make("inside")
    Vc, Pc = splat_cases.columns(V), splat_cases.columns(P)
    perm = np.random.default_rng(0).permutation(x4.shape[0])
    for p, sz in ((0, dsz), (1, tsz)):
        assert np.array_equal(bits(oracle_mod.splat(p, x4, Vc, Pc, *sz)),
                              bits(oracle_mod.splat(p, x4[perm], Vc, Pc, *sz)))


def test_reference_view_matches_the_reference_camera():
    """Camera::Rotate(30, 240) after SetPosition(20, 10, 10): the view
    direction rot * (0, 0, 1) with rot = R_y(240) R_x(30)."""
    V, P = splat.reference_view(1280, 720).matrices()
    fwd = -V[2, :3]  # the camera looks along -z of view space
    assert np.allclose(fwd, [-0.75, -0.5, -0.4330127], atol=1e-6)
    assert np.allclose(V[:3, :3] @ V[:3, :3].T, np.eye(3), atol=1e-6)
    assert np.allclose(V[:3, :3] @ np.array([20, 10, 10]) + V[:3, 3], 0, atol=1e-5)
    assert abs(P[1, 1] - 1 / math.tan(math.radians(22.5))) < 1e-6
    assert abs(P[0, 0] - P[1, 1] * 720 / 1280) < 1e-6


# ---- on the GPU ---------------------------------------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("name", splat_cases.CASES)
def test_gpu_matches_reference_golden(gpu, name):
    x4, V, P, dsz, tsz = splat_cases.make(name)
    view = splat.View.of(V, P)
    g = golden()
    d = splat.splat(splat.DEPTH, x4, view, *dsz).cpu().numpy()
    t = splat.splat(splat.THICKNESS, x4, view, *tsz).cpu().numpy()
    assert np.array_equal(bits(d), bits(g[f"{name}_depth"]))
    assert np.array_equal(bits(t), bits(g[f"{name}_thickness"]))


@pytest.mark.gpu
def test_gpu_reference_scene_full_size(gpu, oracle_mod):
    """The reference's own scene and camera at its framebuffer sizes (depth
    1280 x 720, thickness 512 x 512), straight from the simulation's device
    position buffer after a few substeps."""
    import pbf_gb300 as pg
    import torch
    s = scenes.reference_two_blocks(seed=1)
    sim = pg.SPH(s.n, tuple(s.params.grid), s.params)
    sim.set_state(s.x4, s.v4)
    sim.step(4)
    x, _ = sim.get_state()
    view = splat.reference_view(1280, 720)
    Vc, Pc = view.columns()
    for p, (w, h) in ((splat.DEPTH, (1280, 720)), (splat.THICKNESS, (512, 512))):
        out = torch.empty((h, w), dtype=torch.float32, device="cuda")
        splat.splat_device(p, sim.GetPositionBuffer(), s.n, view, w, h, out.data_ptr())
        want = oracle_mod.splat(p, x, Vc, Pc, w, h)
        assert np.array_equal(bits(out.cpu().numpy()), bits(want)), p


@pytest.mark.gpu
def test_gpu_degenerate_inputs(gpu):
    import pbf_gb300 as pg
    x4, V, P = one_particle_view()
    view = splat.View.of(V, P)
    empty = np.zeros((0, 4), np.float32)
    assert np.all(splat.splat(splat.DEPTH, empty, view, 17, 9).cpu().numpy() == 1.0)
    assert np.all(splat.splat(splat.THICKNESS, empty, view, 17, 9).cpu().numpy() == 0.0)
    # a particle behind the eye and one past the far plane draw nothing
    far = np.array([[64.0, 19.0, 64.0 + 5.0 * 300, 0.0], [64.0, 19.0, 64.0 - 5.0 * 400, 0.0]],
                   np.float32)
    assert np.all(splat.splat(splat.THICKNESS, far, view, 64, 64).cpu().numpy() == 0.0)
    with pytest.raises(pg.PbfError):
        splat.splat(7, x4, view, 8, 8)
    with pytest.raises(pg.PbfError):
        splat.splat(splat.DEPTH, x4, view, 0, 8)

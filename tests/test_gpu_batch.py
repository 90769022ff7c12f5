"""GPU tests of batched scenes (pbf_create_batch): each scene of a batch steps
bit-identically to the same scene in its own handle and to the FP32 oracle."""
import numpy as np
import pytest

import pbf_gb300 as pg
from pbf_gb300 import scenes
from tests.test_gpu_parity import assert_bits

pytestmark = pytest.mark.gpu


def small_batch(num=6, seed=3):
    return scenes.batch_scenes(num, seed=seed, iterations=3, nmin=300, nmax=3000, box_min=12,
                               box_max=30)


def test_batch_matches_single_handles_and_oracle(gpu, oracle_mod):
    sc = small_batch()
    # per-scene constants differ too (XSPH c and vorticity epsilon)
    for k, s in enumerate(sc):
        s.params.xsph_viscosity_c = 0.005 + 0.002 * k
        s.params.vorticity_epsilon = 0.0002 * k
    b = pg.SPHBatch([s.params for s in sc], [s.n for s in sc])
    x4, v4 = scenes.concat_state(sc)
    b.set_state(x4, v4)
    b.step(12)
    bx, bv = b.get_state()
    for k, s in enumerate(sc):
        one = pg.SPH(s.n, tuple(s.params.grid), s.params)
        one.set_state(s.x4, s.v4)
        one.step(12)
        ox, ov = one.get_state()
        sl = b.scene_slice(k)
        assert_bits(bx[sl], ox, f"scene {k} positions vs its own handle")
        assert_bits(bv[sl], ov, f"scene {k} velocities vs its own handle")
        o = oracle_mod.Oracle(s.params, s.n)
        o.set_state(s.x4, s.v4)
        o.step(12)
        rx, rv = o.get_state()
        assert_bits(bx[sl], rx, f"scene {k} positions vs oracle")
        assert_bits(bv[sl], rv, f"scene {k} velocities vs oracle")


@pytest.mark.parametrize("threshold", [1, 40, 120])
def test_batch_mixed_sweeps(gpu, threshold):
    """Mixed sweeps over a batch: the heavy list spans scenes (each particle
    keeps its own scene's constants in the cooperative kernels), and the
    result is the same bits as the one-thread sweeps."""
    sc = small_batch(5, seed=21)
    x4, v4 = scenes.concat_state(sc)
    runs = []
    for thr in (0, threshold):
        b = pg.SPHBatch([s.params for s in sc], [s.n for s in sc])
        b.set_tuning(sweep_mode="masked", coop_candidates=thr)
        b.set_state(x4, v4)
        b.step(10)
        runs.append(b.get_state())
    assert_bits(runs[1][0], runs[0][0], f"positions, mixed threshold {threshold}")
    assert_bits(runs[1][1], runs[0][1], f"velocities, mixed threshold {threshold}")


def test_batch_scene_params_and_tuning(gpu):
    sc = small_batch(4, seed=11)
    b = pg.SPHBatch([s.params for s in sc], [s.n for s in sc])
    x4, v4 = scenes.concat_state(sc)
    b.set_state(x4, v4)
    b.step(3)
    p = b.scene_params(2)
    p.xsph_viscosity_c = 0.03
    b.set_scene_params(2, p)
    b.set_tuning(use_neighbour_lists=False, sweep_mode="coop")
    b.step(4)
    bx, bv = b.get_state()
    # the same sequence on scene 2 alone
    s = sc[2]
    one = pg.SPH(s.n, tuple(s.params.grid), s.params)
    one.set_state(s.x4, s.v4)
    one.step(3)
    one.SetXSPHViscosity(0.03)
    one.step(4)
    ox, ov = one.get_state()
    assert_bits(bx[b.scene_slice(2)], ox, "scene 2 after a parameter change")
    assert_bits(bv[b.scene_slice(2)], ov, "scene 2 velocities after a parameter change")
    # the other scenes are untouched by scene 2's parameters
    s0 = sc[0]
    z = pg.SPH(s0.n, tuple(s0.params.grid), s0.params)
    z.set_state(s0.x4, s0.v4)
    z.step(7)
    assert_bits(bx[b.scene_slice(0)], z.get_state()[0], "scene 0 unaffected")


def test_batch_rejects_mixed_iterations(gpu):
    sc = small_batch(2)
    sc[1].params.num_solver_iterations = 2
    with pytest.raises(pg.PbfError):
        pg.SPHBatch([s.params for s in sc], [s.n for s in sc])


def test_batch_cells_and_sort_are_scene_major(gpu):
    sc = small_batch(3, seed=5)
    b = pg.SPHBatch([s.params for s in sc], [s.n for s in sc])
    x4, v4 = scenes.concat_state(sc)
    b.set_state(x4, v4)
    b.step(1)
    kb, sk, pm = b.get_sort()
    assert np.all(np.diff(sk.astype(np.int64)) >= 0)
    # every scene's particles stay inside its own key range and id range
    base = 0
    for k, s in enumerate(sc):
        nc = int(np.prod(list(s.params.grid)))
        sl = b.scene_slice(k)
        assert np.all((kb[sl] >= base) & (kb[sl] < base + nc))
        base += nc
    assert np.array_equal(pm, np.argsort(kb, kind="stable").astype(np.uint32))

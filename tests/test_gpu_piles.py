"""GPU tests of the direct sweeps' coincident blocks.  The epsilon = 0.01 dam
break drives particles into the box corners, where the clamp stacks them on
single points: by substep 200 of the 16,384-particle configuration about
12,000 particles sit in piles of 32 to ~2,700 at one position.  A cell whose
particles all share one position is swept as a block (density: W(0) added m
times by the exact jump over repeated additions; delta-p and the second
vorticity pass: no term), and the result must still be the oracle's bits."""
import numpy as np
import pytest

import pbf_gb300 as pg
from pbf_gb300 import scenes
from tests.test_gpu_batch import small_batch
from tests.test_gpu_parity import assert_bits

pytestmark = pytest.mark.gpu

SUBSTEPS = 200


@pytest.fixture(scope="module")
def piled(oracle_mod):
    sc = scenes.plain_16k()
    o = oracle_mod.Oracle(sc.params, sc.n)
    o.set_state(sc.x4, sc.v4)
    o.step(SUBSTEPS)
    return sc, o.get_state()


@pytest.mark.parametrize("tuning", [dict(sweep_mode="direct"),
                                    dict(sweep_mode="auto", auto_period=8),
                                    dict(sweep_mode="direct", coop_candidates=300)])
def test_corner_piles_bit_exact(gpu, piled, tuning):
    sc, (ox, ov) = piled
    _, counts = np.unique(ox[:, :3], axis=0, return_counts=True)
    assert counts.max() >= 1000 and counts[counts >= 32].sum() >= 8000  # the piles exist
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    g.set_tuning(**tuning)
    g.set_state(sc.x4, sc.v4)
    for _ in range(SUBSTEPS // 25):
        g.step(25)
    x, v = g.get_state()
    assert_bits(x, ox, f"positions after {SUBSTEPS} substeps with {tuning}")
    assert_bits(v, ov, f"velocities after {SUBSTEPS} substeps with {tuning}")
    # the reference's packed 8-bit run count (foreachneighbour.glsl:5) would
    # have dropped these runs: the informational status bit says so
    assert g.device_status() & pg.PBF_DEV_RUN_OVER_127


def test_run_flag_clear_while_calm(gpu):
    """Near rest density (8 particles per cell) no 3-cell run reaches 128:
    the informational bit stays clear, so the packed form would agree.  In
    the oracle's sort the first window of 128 particles within three cells
    appears at substep 8 of the 16,384-particle dam break, and the bit sets
    there."""
    sc = scenes.plain_16k()
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    g.set_state(sc.x4, sc.v4)
    g.step(7)
    assert g.device_status() & pg.PBF_DEV_RUN_OVER_127 == 0
    g.step(1)
    assert g.device_status() & pg.PBF_DEV_RUN_OVER_127


def test_corner_piles_in_a_batch(gpu, oracle_mod):
    """Small scenes in one batch (per-scene cell ranges and constants) pile up
    too; each scene keeps the oracle's bits under the direct sweeps."""
    sc = small_batch(4, seed=5)
    b = pg.SPHBatch([s.params for s in sc], [s.n for s in sc])
    b.set_tuning(sweep_mode="direct")
    x4, v4 = scenes.concat_state(sc)
    b.set_state(x4, v4)
    b.step(150)
    bx, bv = b.get_state()
    piles = 0
    for k, s in enumerate(sc):
        o = oracle_mod.Oracle(s.params, s.n)
        o.set_state(s.x4, s.v4)
        o.step(150)
        rx, rv = o.get_state()
        sl = b.scene_slice(k)
        assert_bits(bx[sl], rx, f"scene {k} positions")
        assert_bits(bv[sl], rv, f"scene {k} velocities")
        _, counts = np.unique(rx[:, :3], axis=0, return_counts=True)
        piles += int(counts[counts >= 32].sum())
    assert piles > 0

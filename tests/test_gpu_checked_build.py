"""The bounds-checked build (-DPBF_CHECK, pbf_gb300/_build_check/): every
neighbour-run bound, list index and permutation entry a kernel reads is
checked, and a failed check latches PBF_DEV_INDEX and skips the access
instead of faulting.  On valid inputs it must give the normal build's bits
with the bit clear, across the sweep configurations, a batch and the adjoint."""
import numpy as np
import pytest

import pbf_gb300 as pg
from pbf_gb300 import _capi, build, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def checked(gpu):
    build.build(check=True)
    return _capi.load_checked()


def status_bits(sim):
    return sim.device_status()


@pytest.mark.parametrize("mode", ["auto", "masked", "direct", "coop"])
def test_checked_build_equals_normal_build(checked, mode):
    sc = scenes.plain_16k()
    out = []
    for lib in (None, checked):
        sim = pg.SPH(sc.n, tuple(sc.params.grid), sc.params, lib=lib)
        sim.set_tuning(sweep_mode=mode)
        sim.set_state(sc.x4, sc.v4)
        sim.step(60)  # through the collapse into clumps and corner piles
        x, v = sim.get_state()
        assert not (status_bits(sim) & _capi.PBF_DEV_INDEX)
        out.append((x, v))
        sim.close()
    assert np.array_equal(out[0][0].view(np.uint32), out[1][0].view(np.uint32))
    assert np.array_equal(out[0][1].view(np.uint32), out[1][1].view(np.uint32))


def test_checked_build_batch_and_adjoint(checked):
    sc = scenes.batch_scenes(3, seed=9, iterations=2, nmin=300, nmax=900, box_min=14, box_max=20)
    x4, v4 = scenes.concat_state(sc)
    rng = np.random.default_rng(1)
    w = rng.normal(size=x4.shape).astype(np.float32)
    w[:, 3] = 0
    res = []
    for lib in (None, checked):
        b = pg.SPHBatch([s.params for s in sc], [s.n for s in sc], lib=lib)
        b.set_state(x4, v4)
        b.forward_record(4, 2)
        dx0, dv0, g = b.backward(w, None)
        assert not (status_bits(b) & _capi.PBF_DEV_INDEX)
        res.append((b.positions(), dx0, dv0, np.asarray(g)))
        b.close()
    for a, c in zip(res[0], res[1]):
        assert np.array_equal(np.asarray(a).view(np.uint8), np.asarray(c).view(np.uint8))

"""The benchmarked workload at its full size: the 2,097,152-particle dam break
(128^3 lattice, 257 x 129 x 257 cells, 4 iterations), stepped on the GPU with
the default tuning and compared bit for bit with the FP32 oracle, plus the
size-independent properties of the intermediate state (the sort is a stable
permutation of the keys, the cell tables describe exactly the sorted runs)."""
import numpy as np
import pytest

import pbf_gb300 as pg
from pbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_dam_break_2m_bit_exact(gpu, oracle_mod):
    sc = scenes.plain_2m()
    sim = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    sim.set_state(sc.x4, sc.v4)
    sim.step(2)
    o = oracle_mod.Oracle(sc.params, sc.n)
    o.set_state(sc.x4, sc.v4)
    o.step(2)
    x, v = sim.get_state()
    ox, ov = o.get_state()
    assert np.array_equal(x.view(np.uint32), ox.view(np.uint32))
    assert np.array_equal(v.view(np.uint32), ov.view(np.uint32))

    keys, skeys, perm = sim.get_sort()
    okeys, oskeys, operm = o.get_sort()
    assert np.array_equal(perm, operm)
    # stable sort: sorted keys ascending, perm a permutation, ties in id order
    assert np.all(np.diff(skeys.astype(np.int64)) >= 0)
    assert np.array_equal(np.sort(perm), np.arange(sc.n, dtype=perm.dtype))
    assert np.array_equal(keys[perm], skeys)
    same = skeys[1:] == skeys[:-1]
    assert np.all(perm[1:][same] > perm[:-1][same])
    # cell tables: every occupied cell's [start, end) is its run, others empty
    start, end = sim.get_cells()
    cells = np.unique(skeys)
    first = np.searchsorted(skeys, cells, side="left")
    last = np.searchsorted(skeys, cells, side="right")
    assert np.array_equal(start[cells], first) and np.array_equal(end[cells], last)
    empty = np.ones(start.shape[0], bool)
    empty[cells] = False
    assert np.all(start[empty] == -1) and np.all(end[empty] == -1)

"""The reference application's own scene, the state snapshot format and the
highlight query.

- scenes.reference_two_blocks: Simulation::ResetParticleBuffer's two 32^3
  blocks (src/Simulation.cpp:206-246) with SPH's defaults; on the GPU a few
  substeps of it are bit-exact with the oracle.
- pbf_save_state / pbf_load_state: the file equals snapshot.write_snapshot's
  bytes, and loading restores the state bit for bit.
- pbf_highlight_neighbours: equal to the oracle's highlight pass (itself
  checked against the reference's highlight shaders in test_ref_pin.py), on a
  single scene, on batches, through host and device flag buffers.
"""
import os

import numpy as np
import pytest

import pbf_gb300 as pg
from pbf_gb300 import scenes, snapshot


# ---- host side ----------------------------------------------------------------

def test_reference_two_blocks_layout():
    s = scenes.reference_two_blocks(seed=3)
    assert s.n == 65536 and s.params.num_solver_iterations == 5 and float(s.params.h) == 2.0
    assert [int(g) for g in s.params.grid] == [128, 64, 128]
    assert not s.params.vorticity_confinement
    x = s.x4[:, :3].astype(np.float64)
    a, b = x[:32768], x[32768:]
    # ids x outermost, then z, then y; spacing 0.94; jitter within +-0.005
    ideal = np.empty_like(a)
    i = np.arange(32768)
    ideal[:, 0], ideal[:, 2], ideal[:, 1] = i // 1024, (i // 32) % 32, i % 32
    assert np.max(np.abs(a - ((32.5, 0.5, 32.5) + 0.94 * ideal))) <= 0.005 + 1e-5
    assert np.max(np.abs(b - ((95.5, 0.5, 95.5) + 0.94 * ideal * (-1, 1, -1)))) <= 0.005 + 1e-5
    assert not np.any(s.v4)
    # every particle inside the reference's walls
    assert np.all(x >= (16, 0, 16)) and np.all(x <= (112, 64, 112))
    # seeded: equal seeds give equal scenes, different seeds differ
    assert np.array_equal(s.x4, scenes.reference_two_blocks(seed=3).x4)
    assert not np.array_equal(s.x4, scenes.reference_two_blocks(seed=4).x4)


def test_snapshot_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    x = rng.standard_normal((37, 4)).astype(np.float32)
    v = rng.standard_normal((37, 4)).astype(np.float32)
    f = tmp_path / "s.pbfstate"
    snapshot.write_snapshot(f, x, v, num_scenes=2)
    raw = f.read_bytes()
    assert raw[:8] == b"PBFSTATE" and len(raw) == 24 + 32 * 37
    assert np.frombuffer(raw, "<u4", 4, 8).tolist() == [1, 37, 2, 0]
    x2, v2, ns = snapshot.read_snapshot(f)
    assert ns == 2 and np.array_equal(x2.view(np.uint32), x.view(np.uint32))
    assert np.array_equal(v2.view(np.uint32), v.view(np.uint32))


@pytest.mark.parametrize("damage", ["magic", "version", "truncated"])
def test_snapshot_rejects_damaged_files(tmp_path, damage):
    x = np.zeros((5, 4), np.float32)
    f = tmp_path / "s.pbfstate"
    snapshot.write_snapshot(f, x, x)
    raw = bytearray(f.read_bytes())
    if damage == "magic":
        raw[0] = ord("X")
    elif damage == "version":
        raw[8] = 9
    else:
        raw = raw[:-4]
    f.write_bytes(bytes(raw))
    with pytest.raises(ValueError):
        snapshot.read_snapshot(f)


def test_oracle_highlight_semantics(oracle_mod):
    """Bit 1 marks exactly the stencil candidates (runs, self excluded) of the
    selected particles; other bits above 0 are cleared."""
    x4, v4 = scenes.block((6, 5, 7), seed=2, vel_uniform=0.2)
    p = scenes.dam_params((12, 12, 12), 2)
    o = oracle_mod.Oracle(p, x4.shape[0])
    o.set_state(x4, v4)
    o.step(1)
    _, _, perm = o.get_sort()
    rank = np.empty_like(perm)
    rank[perm] = np.arange(perm.size, dtype=perm.dtype)
    flags = np.full(x4.shape[0], 6, np.uint32)
    sel = [0, 17, 101]
    flags[sel] |= 1
    out = o.highlight(flags)
    want = np.zeros(x4.shape[0], bool)
    for sid in sel:
        i = int(rank[sid])
        for b, e in o.get_runs(i):
            for j in range(int(b), int(e)):
                if j != i:
                    want[perm[j]] = True
    assert np.array_equal(out & 1, (flags & 1))
    assert np.array_equal((out >> 1) & 1 == 1, want)
    assert not np.any(out >> 2)


# ---- on the GPU ---------------------------------------------------------------

@pytest.mark.gpu
def test_reference_two_blocks_bit_exact(gpu, oracle_mod):
    s = scenes.reference_two_blocks(seed=0)
    sim = pg.SPH(s.n, tuple(s.params.grid), s.params)
    sim.set_state(s.x4, s.v4)
    sim.step(3)
    o = oracle_mod.Oracle(s.params, s.n)
    o.set_state(s.x4, s.v4)
    o.step(3)
    x, v = sim.get_state()
    ox, ov = o.get_state()
    assert np.array_equal(x.view(np.uint32), ox.view(np.uint32))
    assert np.array_equal(v.view(np.uint32), ov.view(np.uint32))
    sel = np.arange(5, s.n, 4099)
    flags = sim.highlight_neighbours(sel)
    oflags = np.zeros(s.n, np.uint32)
    oflags[sel] = 1
    assert np.array_equal(flags, o.highlight(oflags))


@pytest.mark.gpu
def test_save_load_state(gpu, tmp_path):
    x4, v4 = scenes.block((12, 10, 9), seed=4, vel_uniform=0.4)
    p = scenes.dam_params((24, 24, 24), 3)
    sim = pg.SPH(x4.shape[0], tuple(p.grid), p)
    sim.set_state(x4, v4)
    sim.step(2)
    f = tmp_path / "a.pbfstate"
    sim.save_state(f)
    x, v = sim.get_state()
    snapshot.write_snapshot(tmp_path / "b.pbfstate", x, v)
    assert f.read_bytes() == (tmp_path / "b.pbfstate").read_bytes()
    sim.step(3)
    x5, v5 = sim.get_state()
    sim.load_state(f)
    xl, vl = sim.get_state()
    assert np.array_equal(xl.view(np.uint32), x.view(np.uint32))
    assert np.array_equal(vl.view(np.uint32), v.view(np.uint32))
    sim.step(3)  # resuming from the snapshot repeats the same substeps
    xr, vr = sim.get_state()
    assert np.array_equal(xr.view(np.uint32), x5.view(np.uint32))
    assert np.array_equal(vr.view(np.uint32), v5.view(np.uint32))


@pytest.mark.gpu
def test_load_state_rejects_mismatch(gpu, tmp_path):
    x4, v4 = scenes.block((4, 4, 4), seed=1)
    p = scenes.dam_params((16, 16, 16), 2)
    sim = pg.SPH(x4.shape[0], tuple(p.grid), p)
    sim.set_state(x4, v4)
    snapshot.write_snapshot(tmp_path / "small.pbfstate", x4[:10], v4[:10])
    with pytest.raises(pg.PbfError):
        sim.load_state(tmp_path / "small.pbfstate")
    (tmp_path / "junk").write_bytes(b"not a snapshot")
    with pytest.raises(pg.PbfError):
        sim.load_state(tmp_path / "junk")
    with pytest.raises(pg.PbfError):
        sim.load_state(tmp_path / "missing")
    x, _ = sim.get_state()  # state untouched by the failed loads
    assert np.array_equal(x, x4)


@pytest.mark.gpu
@pytest.mark.parametrize("substeps", [1, 4])
def test_highlight_matches_oracle(gpu, oracle_mod, substeps):
    import torch
    x4, v4 = scenes.block((20, 14, 18), seed=6, vel_uniform=0.8)
    p = scenes.dam_params((32, 32, 32), 3)
    sim = pg.SPH(x4.shape[0], tuple(p.grid), p)
    sim.set_state(x4, v4)
    sim.step(substeps)
    o = oracle_mod.Oracle(p, x4.shape[0])
    o.set_state(x4, v4)
    o.step(substeps)
    rng = np.random.default_rng(substeps)
    flags = rng.integers(0, 8, x4.shape[0]).astype(np.uint32)
    flags[rng.random(x4.shape[0]) < 0.97] &= 6  # about 3 % selected
    want = o.highlight(flags)
    got = flags.copy()
    sim.highlight_flags(got)
    assert np.array_equal(got, want)
    dev = torch.from_numpy(flags.view(np.int32)).cuda()
    sim.highlight_flags(dev)
    assert np.array_equal(dev.cpu().numpy().view(np.uint32), want)


@pytest.mark.gpu
def test_highlight_in_a_batch(gpu, oracle_mod):
    sc = scenes.batch_scenes(3, seed=2, iterations=3, nmin=300, nmax=1500, box_min=12, box_max=20)
    b = pg.SPHBatch([s.params for s in sc], [s.n for s in sc])
    b.set_state(*scenes.concat_state(sc))
    b.step(2)
    n = sum(s.n for s in sc)
    flags = np.zeros(n, np.uint32)
    flags[::53] = 1
    got = flags.copy()
    b.highlight_flags(got)
    for k, s in enumerate(sc):
        sl = b.scene_slice(k)
        o = oracle_mod.Oracle(s.params, s.n)
        o.set_state(s.x4, s.v4)
        o.step(2)
        assert np.array_equal(got[sl], o.highlight(flags[sl])), k

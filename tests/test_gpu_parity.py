"""GPU parity: the CUDA substep against the FP32 oracle, through the C ABI.

Bar: bit-exact.  The sort permutation, the cell tables and every particle's
position, velocity and lambda must equal the oracle's bits, because both
evaluate the same IEEE-754 operation sequence in the reference's neighbour
order.  (The benchmark spec's tolerance, 1e-5 h max-abs per substep, is implied.)
"""
import ctypes as C

import numpy as np
import pytest

import pbf_gb300 as pg
from pbf_gb300 import scenes

pytestmark = pytest.mark.gpu


def run_gpu(params, x4, v4, substeps=1):
    sim = pg.SPH(x4.shape[0], tuple(params.grid), params)
    sim.set_state(x4, v4)
    sim.step(substeps)
    return sim


def run_oracle(oracle_mod, params, x4, v4, substeps=1, fp64=False):
    o = oracle_mod.Oracle(params, x4.shape[0], fp64=fp64)
    o.set_state(x4, v4)
    o.step(substeps)
    return o


def assert_bits(a, b, what):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    assert a.shape == b.shape, what
    same = a.view(np.uint32) == b.view(np.uint32)
    if not np.all(same):
        bad = np.argwhere(~same)
        i = tuple(bad[0])
        pytest.fail(f"{what}: {len(bad)} mismatching words, first at {i}: gpu={a[i]!r} oracle={b[i]!r}")


def compare_substep(gpu, o, params):
    kb, sk, pm = gpu.get_sort()
    okb, osk, opm = o.get_sort()
    assert np.array_equal(kb, okb), "cell keys"
    assert np.array_equal(sk, osk), "sorted keys"
    assert np.array_equal(pm, opm), "sort permutation"
    st, en = gpu.get_cells()
    ost, oen = o.get_cells()
    assert np.array_equal(st, ost), "cell start"
    assert np.array_equal(en, oen), "cell end"
    lam, xp = gpu.get_solver()
    olam, oxp = o.get_solver()
    assert_bits(xp, oxp, "predicted positions (sorted)")
    if params.num_solver_iterations > 0:
        assert_bits(lam, olam, "lambda of the last iteration")
    x, v = gpu.get_state()
    ox, ov = o.get_state()
    assert_bits(x, ox, "positions")
    assert_bits(v, ov, "velocities")


def test_dam_break_16k_one_substep_bit_exact(gpu, oracle_mod):
    sc = scenes.plain_16k()
    g = run_gpu(sc.params, sc.x4, sc.v4)
    o = run_oracle(oracle_mod, sc.params, sc.x4, sc.v4)
    compare_substep(g, o, sc.params)


def test_dam_break_16k_many_substeps_bit_exact(gpu, oracle_mod):
    """Bit-exact substeps compose: 40 substeps stay bit-identical."""
    sc = scenes.plain_16k()
    g = run_gpu(sc.params, sc.x4, sc.v4, 40)
    o = run_oracle(oracle_mod, sc.params, sc.x4, sc.v4, 40)
    x, v = g.get_state()
    ox, ov = o.get_state()
    assert_bits(x, ox, "positions after 40 substeps")
    assert_bits(v, ov, "velocities after 40 substeps")


def test_graph_replay_equals_eager_timing_path(gpu):
    sc = scenes.plain_16k()
    a = run_gpu(sc.params, sc.x4, sc.v4, 5)
    b = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    b.set_state(sc.x4, sc.v4)
    b.EnableTiming(True)
    b.step(5)
    t = b.OutputTiming()
    assert all(v >= 0 for v in t.values()) and t["solver"] > 0
    xa, va = a.get_state()
    xb, vb = b.get_state()
    assert_bits(xa, xb, "graph vs eager positions")
    assert_bits(va, vb, "graph vs eager velocities")


def test_deterministic_runs(gpu):
    sc = scenes.plain_16k()
    a = run_gpu(sc.params, sc.x4, sc.v4, 10).get_state()
    b = run_gpu(sc.params, sc.x4, sc.v4, 10).get_state()
    assert_bits(a[0], b[0], "run-to-run positions")
    assert_bits(a[1], b[1], "run-to-run velocities")


@pytest.mark.parametrize("n_lat", [(1, 1, 1), (2, 1, 1), (3, 5, 7), (17, 13, 19), (16, 16, 16)])
def test_ragged_sizes_bit_exact(gpu, oracle_mod, n_lat):
    x4, v4 = scenes.block(n_lat, seed=5, vel_uniform=0.5)
    p = scenes.dam_params((24, 24, 24), 3)
    g = run_gpu(p, x4, v4, 2)
    o = run_oracle(oracle_mod, p, x4, v4, 2)
    compare_substep(g, o, p)


@pytest.mark.parametrize("variant", ["no_vorticity", "ext_force", "h_0.8", "zero_iters",
                                     "walls_inset", "odd_grid"])
def test_parameter_variants_bit_exact(gpu, oracle_mod, variant):
    x4, v4 = scenes.block((20, 12, 16), seed=9, vel_uniform=1.0)
    box = (30, 20, 26)
    p = scenes.dam_params(box, 3)
    if variant == "no_vorticity":
        p.vorticity_confinement = 0
    elif variant == "ext_force":
        p.external_force = 1
        x4[:, 2] += 12.0  # put part of the block beyond GRID_SIZE.z / 2
    elif variant == "h_0.8":
        p.h = 0.8
    elif variant == "zero_iters":
        p.num_solver_iterations = 0
    elif variant == "walls_inset":
        p.wall_lo[0], p.wall_hi[0] = 2.0, 9.0
        p.wall_lo[2], p.wall_hi[2] = 1.5, 7.25
    elif variant == "odd_grid":
        p = scenes.dam_params((13.5, 7.25, 31.0), 2)
    g = run_gpu(p, x4, v4, 3)
    o = run_oracle(oracle_mod, p, x4, v4, 3)
    compare_substep(g, o, p)


def test_positions_outside_grid_bit_exact(gpu, oracle_mod):
    """Predicted positions beyond the grid on every side (keys clamp to the edge cells)."""
    x4, v4 = scenes.block((10, 10, 10), seed=2, vel_uniform=2000.0)
    p = scenes.dam_params((8, 8, 8), 2)
    g = run_gpu(p, x4, v4, 2)
    o = run_oracle(oracle_mod, p, x4, v4, 2)
    compare_substep(g, o, p)


def test_set_params_between_steps(gpu, oracle_mod):
    sc = scenes.plain_16k()
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    g.set_state(sc.x4, sc.v4)
    o = oracle_mod.Oracle(sc.params, sc.n)
    o.set_state(sc.x4, sc.v4)
    g.step(2)
    o.step(2)
    g.SetXSPHViscosity(0.05)
    g.SetNumSolverIterations(2)
    g.SetVorticityEpsilon(0.002)
    o.set_params(g.params)
    g.step(2)
    o.step(2)
    x, v = g.get_state()
    ox, ov = o.get_state()
    assert_bits(x, ox, "positions after parameter change")
    assert_bits(v, ov, "velocities after parameter change")


def test_device_buffers_zero_copy(gpu):
    import torch
    sc = scenes.plain_16k()
    g = run_gpu(sc.params, sc.x4, sc.v4, 1)
    x, v = g.get_state()
    ptr = g.GetPositionBuffer()
    assert ptr != 0 and g.GetVelocityBuffer() != 0
    t = torch.empty((sc.n, 4), dtype=torch.float32, device="cuda")
    g.get_state_into(t.data_ptr(), None, pg.PBF_DEVICE)
    assert np.array_equal(t.cpu().numpy(), x)
    # upload from device memory
    t2 = torch.from_numpy(sc.x4).cuda()
    t3 = torch.from_numpy(sc.v4).cuda()
    torch.cuda.synchronize()
    g.set_state_device(t2.data_ptr(), t3.data_ptr())
    assert np.array_equal(g.positions(), sc.x4)


def test_diagnostics_match_oracle(gpu, oracle_mod):
    sc = scenes.plain_16k()
    g = run_gpu(sc.params, sc.x4, sc.v4, 5)
    o = run_oracle(oracle_mod, sc.params, sc.x4, sc.v4, 5)
    dg = g.diagnostics()
    do = o.diagnostics()
    assert dg["candidate_pairs"] == do["candidate_pairs"]
    assert dg["mean_density_error"] == pytest.approx(do["mean_density_error"], rel=1e-5)
    assert dg["max_density_error"] == pytest.approx(do["max_density_error"], rel=1e-5)
    assert dg["kinetic_energy"] == pytest.approx(do["kinetic_energy"], rel=1e-5)
    # diagnostics re-sort the state; stepping afterwards stays bit-exact
    g.step(2)
    o.step(2)
    assert_bits(g.positions(), o.get_state()[0], "positions after diagnostics")


def test_nonfinite_input_reported(gpu):
    sc = scenes.plain_16k()
    x4 = sc.x4.copy()
    x4[5, 0] = np.nan
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    g.set_state(x4, sc.v4)
    g.step(1)
    with pytest.raises(pg.PbfError) as e:
        g.synchronize()
    assert e.value.status == 4
    assert g.device_status() & pg.PBF_DEV_NONFINITE


def test_set_params_rejects_grid_change(gpu):
    sc = scenes.plain_16k()
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    p = sc.params.copy()
    p.grid[0] = 10
    with pytest.raises(pg.PbfError):
        g.set_params(p)


@pytest.mark.parametrize("tuning", [dict(use_neighbour_lists=False),
                                    dict(use_neighbour_lists=True, list_capacity=8),
                                    dict(use_neighbour_lists=True, skin_h=0.0),
                                    dict(use_neighbour_lists=True, skin_h=0.5, list_capacity=400),
                                    dict(use_neighbour_lists=True, skin_h=0.02),
                                    dict(use_neighbour_lists=False, sweep_mode="direct"),
                                    dict(use_neighbour_lists=False, sweep_mode="masked"),
                                    dict(use_neighbour_lists=True, sweep_mode="direct", block_size=96),
                                    dict(use_neighbour_lists=True, skin_h=0.0, sweep_mode="masked"),
                                    dict(pair_list_capacity=0),
                                    dict(pair_list_capacity=1, sweep_mode="direct"),
                                    dict(pair_list_capacity=1, sweep_mode="masked"),
                                    dict(pair_list_capacity=20, use_neighbour_lists=False),
                                    dict(pair_list_capacity=33, block_size=64),
                                    dict(pair_list_capacity=4096, use_neighbour_lists=True),
                                    dict(pair_list_capacity=8, use_neighbour_lists=True, skin_h=0.3),
                                    dict(sweep_mode="coop"),
                                    dict(sweep_mode="coop", use_neighbour_lists=True),
                                    dict(coop_candidates=1),
                                    dict(coop_candidates=100),
                                    dict(coop_candidates=200, pair_list_capacity=20),
                                    dict(coop_candidates=150, sweep_mode="direct"),
                                    dict(coop_candidates=100, pair_list_capacity=0, block_size=64),
                                    dict(coop_candidates=100, use_neighbour_lists=True)])
def test_tuning_never_changes_results(gpu, oracle_mod, tuning):
    """Neighbour lists, their capacity and skin, the sweep mode and the pair
    lists (capacities 1, 8 and 20 overflow often: the scanning sweep then
    finds the entries past the capacity with a second scan, and the replaying
    sweep falls back to a scan) and the mixed sweeps (the particles with more
    than coop_candidates stencil candidates swept by warps, the rest by
    threads; ignored with skin lists) are performance knobs only.  (A scene this
    small defaults to the cooperative sweeps; the one-thread modes are set
    explicitly unless the case names one.)"""
    sc = scenes.plain_16k()
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    g.set_tuning(**{"sweep_mode": "masked", **tuning})
    g.set_state(sc.x4, sc.v4)
    g.step(30)
    o = run_oracle(oracle_mod, sc.params, sc.x4, sc.v4, 30)
    x, v = g.get_state()
    ox, ov = o.get_state()
    assert_bits(x, ox, f"positions with {tuning}")
    assert_bits(v, ov, f"velocities with {tuning}")


@pytest.mark.parametrize("extra", [dict(), dict(pair_list_capacity=0),
                                   dict(coop_candidates=100), dict(pair_list_capacity=20)])
def test_auto_sweeps_never_change_results(gpu, oracle_mod, extra):
    """PBF_SWEEP_AUTO with a trial every few substeps: each trial steps one
    real substep under each candidate configuration of the solver and
    vorticity passes (masked, direct, cooperative), so every configuration
    and every switch between them runs inside these 30 substeps, and the
    result is the oracle's bits."""
    sc = scenes.plain_16k()
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    g.set_tuning(sweep_mode="auto", auto_period=2, **extra)
    g.set_state(sc.x4, sc.v4)
    assert g.sweep_choice() == {"solver": "coop", "vorticity": "coop", "trials": 0}
    for _ in range(6):
        g.step(5)
    assert g.sweep_choice()["trials"] >= 3
    o = run_oracle(oracle_mod, sc.params, sc.x4, sc.v4, 30)
    x, v = g.get_state()
    ox, ov = o.get_state()
    assert_bits(x, ox, f"positions under automatic sweeps {extra}")
    assert_bits(v, ov, f"velocities under automatic sweeps {extra}")


def test_auto_is_the_default_and_resets(gpu):
    """Handles default to PBF_SWEEP_AUTO, starting with the cooperative
    sweeps below 32,768 particles and the mixed sweeps from there; a state
    upload restarts the trial schedule (the first trial after auto_period
    substeps)."""
    sc = scenes.plain_16k()
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    assert g.get_tuning().sweep_mode == 3
    assert g.sweep_choice()["solver"] == "coop"
    g.set_tuning(auto_period=8)
    g.set_state(sc.x4, sc.v4)
    l0 = g.kernels_launched()
    g.step(8)
    assert g.sweep_choice()["trials"] == 0
    assert g.kernels_launched() - l0 == 8 * g.kernels_per_substep()
    g.step(4)  # the trial's substeps: one per candidate
    assert g.sweep_choice()["trials"] == 1
    g.set_state(sc.x4, sc.v4)
    assert g.sweep_choice() == {"solver": "coop", "vorticity": "coop", "trials": 0}
    big = scenes.dam_break((40, 40, 40), (80, 80, 80), 4, 100, 0, "auto")
    h = pg.SPH(big.n, tuple(big.params.grid), big.params)
    assert h.sweep_choice()["solver"] == "mixed"


def test_auto_sweeps_with_the_mixed_candidate_never_change_results(gpu, oracle_mod):
    """From 32,768 particles the automatic configuration starts with the
    mixed sweeps (a warp for each particle with more than 256 stencil
    candidates) and also tries them in its trials, next to masked, direct and
    cooperative; every switch keeps the oracle's bits."""
    sc = scenes.dam_break((40, 40, 40), (80, 80, 80), 4, 100, 0, "auto_mixed")
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    g.set_tuning(sweep_mode="auto", auto_period=2)
    g.set_state(sc.x4, sc.v4)
    assert g.sweep_choice() == {"solver": "mixed", "vorticity": "mixed", "trials": 0}
    for _ in range(6):
        g.step(5)
    assert g.sweep_choice()["trials"] >= 3
    o = run_oracle(oracle_mod, sc.params, sc.x4, sc.v4, 30)
    x, v = g.get_state()
    ox, ov = o.get_state()
    assert_bits(x, ox, "positions under automatic sweeps with the mixed candidate")
    assert_bits(v, ov, "velocities under automatic sweeps with the mixed candidate")


def test_lists_exact_in_a_calm_scene(gpu, oracle_mod):
    """A stable scene (reference default epsilon = 5) where the lists are in use on
    most sweeps, over many substeps."""
    sc = scenes.plain_16k()
    p = sc.params.copy()
    p.epsilon = 5.0
    g = pg.SPH(sc.n, tuple(p.grid), p)
    g.set_tuning(use_neighbour_lists=True, skin_h=0.15, sweep_mode="masked")
    g.set_state(sc.x4, sc.v4)
    g.step(60)
    o = run_oracle(oracle_mod, p, sc.x4, sc.v4, 60)
    x, v = g.get_state()
    ox, ov = o.get_state()
    assert_bits(x, ox, "positions after 60 calm substeps")
    assert_bits(v, ov, "velocities after 60 calm substeps")


def test_block_size_and_autotune_never_change_results(gpu, oracle_mod):
    sc = scenes.plain_16k()
    o = run_oracle(oracle_mod, sc.params, sc.x4, sc.v4, 12)
    ox, ov = o.get_state()
    for blk in (32, 128, 256):
        g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
        g.set_tuning(block_size=blk, sweep_mode="masked")
        g.set_state(sc.x4, sc.v4)
        g.step(12)
        assert_bits(g.positions(), ox, f"positions with block {blk}")
    g = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    g.set_state(sc.x4, sc.v4)
    best = g.autotune(4)
    assert best["block_size"] in (128, 256)
    # the autotuner leaves the state where it was
    assert np.array_equal(g.positions(), sc.x4)
    g.step(12)
    x, v = g.get_state()
    assert_bits(x, ox, "positions after autotune")
    assert_bits(v, ov, "velocities after autotune")
    with pytest.raises(pg.PbfError):
        g.set_tuning(block_size=48)
    with pytest.raises(pg.PbfError):
        g.set_tuning(sweep_mode=4)


@pytest.mark.parametrize("after", [0, 1, 5, 12, 16])
def test_allocation_failure_is_reported_and_cleaned_up(gpu, after):
    """Host-side fault injection: the k-th device allocation reports out of
    memory; creation fails with PBF_ERR_OUT_OF_MEMORY, frees what it got, and
    the next creation works."""
    sc = scenes.plain_16k()
    lib = pg.load()
    lib.pbf_debug_fail_allocation(after)
    try:
        with pytest.raises(pg.PbfError) as e:
            pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
        assert e.value.status == 2
    finally:
        lib.pbf_debug_fail_allocation(-1)
    g = run_gpu(sc.params, sc.x4, sc.v4, 1)
    assert np.all(np.isfinite(g.positions()))

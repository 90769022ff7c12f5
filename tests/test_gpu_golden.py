"""The CUDA substep against the golden outputs of the reference's own
compute shaders (tests/golden/, generated by tests/golden/make_golden.py
from the reference checkout): sort order identical, positions within the
spec tolerance 1e-5 h, velocities and lambda within their rounding."""
import os
import sys

import numpy as np
import pytest

import pbf_gb300 as pg

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, HERE)
import pin_scenes  # noqa: E402

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", list(pin_scenes.CASES))
def test_gpu_matches_reference_golden(gpu, name):
    p, x4, v4 = pin_scenes.make(name)
    g = np.load(os.path.join(HERE, f"ref_{name}.npz"))
    sim = pg.SPH(x4.shape[0], tuple(p.grid), p)
    sim.set_state(x4, v4)
    sim.step(1)
    _, _, perm = sim.get_sort()
    assert np.array_equal(perm, g["ids"]), "sort order differs from the reference's"
    x, v = sim.get_state()
    lam, _ = sim.get_solver()
    h, dt = float(p.h), float(p.timestep)
    assert np.max(np.abs(x[:, :3] - g["x"][:, :3])) <= 1e-5 * h
    assert np.max(np.abs(v[:, :3] - g["v"][:, :3])) <= 1e-5 * h / dt
    if p.num_solver_iterations:
        assert np.max(np.abs(lam - g["lam"])) <= 2e-5


@pytest.mark.parametrize("name", list(pin_scenes.CASES))
def test_gpu_highlight_matches_reference_golden(gpu, name):
    p, x4, v4 = pin_scenes.make(name)
    g = np.load(os.path.join(HERE, f"ref_{name}.npz"))
    sim = pg.SPH(x4.shape[0], tuple(p.grid), p)
    sim.set_state(x4, v4)
    sim.step(1)
    flags = g["hl_in"].copy()
    sim.highlight_flags(flags)
    assert np.array_equal(flags, g["hl"])

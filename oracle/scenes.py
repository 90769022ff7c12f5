"""The workloads' seeded dam-break scenes built on the oracle side — TEST
INFRASTRUCTURE ONLY.

bench.py's CPU reference arm builds its scene here, so that timing the
reference path loads nothing but the oracle.  The generator
(pbf_scene_oracle.cpp) follows the same recipe as the product's
pbf_scene_block, and tests/test_oracle.py checks scenes and constants from
both byte for byte.  Constants: h = 1, lattice spacing 0.5h, g = 9.81,
dt = 0.008, epsilon = 0.01, s_corr k = 0.1 (n = 4, dq = 0.2h), XSPH c = 0.01,
vorticity epsilon = 0.0005, rho_0 = poly6 density of an unjittered interior
lattice point (self excluded); grid floor(B) + 1 cells per box side B.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import load

H = 1.0
SPACING = 0.5
GRAVITY = 9.81
DT = 0.008
EPSILON = 0.01
SCORR_K = 0.1
SCORR_DQ = 0.2
XSPH_C = 0.01
VORT_EPS = 0.0005
JITTER = 0.01


class Params(C.Structure):
    """The oracle's parameter block (pbfo::Params, the same layout as the
    product's pbf_params; tests check both)."""

    _fields_ = [
        ("one_over_rho_0", C.c_float),
        ("epsilon", C.c_float),
        ("gravity", C.c_float),
        ("timestep", C.c_float),
        ("tensile_instability_k", C.c_float),
        ("tensile_instability_scale", C.c_float),
        ("xsph_viscosity_c", C.c_float),
        ("vorticity_epsilon", C.c_float),
        ("h", C.c_float),
        ("num_solver_iterations", C.c_uint32),
        ("vorticity_confinement", C.c_uint32),
        ("external_force", C.c_uint32),
        ("grid", C.c_uint32 * 3),
        ("wall_lo", C.c_float * 3),
        ("wall_hi", C.c_float * 3),
    ]

    def copy(self) -> "Params":
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def as_dict(self) -> dict:
        return {name: (list(getattr(self, name)) if hasattr(getattr(self, name), "__len__")
                       else getattr(self, name)) for name, _ in self._fields_}


@dataclass
class Scene:
    name: str
    params: Params
    x4: np.ndarray
    v4: np.ndarray
    substeps: int
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.x4.shape[0])


def wpoly6(r: float, h: float = H) -> float:
    return float(load().pbfo_wpoly6(r, h))


def rest_density(h: float = H, spacing: float = SPACING) -> float:
    return float(load().pbfo_rest_density_lattice(h, spacing))


def dam_params(box, iterations: int, *, h: float = H, spacing: float = SPACING,
               epsilon: float = EPSILON) -> Params:
    grid = [int(math.floor(b)) + 1 for b in box]
    p = Params()
    if load().pbfo_params_default((C.c_uint32 * 3)(*grid), C.addressof(p)) != 0:
        raise ValueError(f"bad grid {grid}")
    p.h = h
    p.one_over_rho_0 = float(np.float32(1.0 / rest_density(h, spacing)))
    p.epsilon = epsilon
    p.gravity = GRAVITY
    p.timestep = DT
    p.tensile_instability_k = SCORR_K
    p.tensile_instability_scale = float(np.float32(1.0 / wpoly6(SCORR_DQ * h, h)))
    p.xsph_viscosity_c = XSPH_C
    p.vorticity_epsilon = VORT_EPS
    p.num_solver_iterations = int(iterations)
    p.vorticity_confinement = 1
    p.external_force = 0
    for a in range(3):
        p.wall_lo[a] = 0.0
        p.wall_hi[a] = float(box[a])
    return p


def block(lattice, *, spacing: float = SPACING, origin=None, jitter: float = JITTER,
          vel_uniform: float = 0.0, vel_sigma: float = 0.0, seed: int = 0):
    lat = [int(v) for v in lattice]
    n = lat[0] * lat[1] * lat[2]
    if origin is None:
        origin = (0.5 * spacing,) * 3
    x4 = np.empty((n, 4), np.float32)
    v4 = np.empty((n, 4), np.float32)
    rc = load().pbfo_scene_block((C.c_uint32 * 3)(*lat), spacing, (C.c_float * 3)(*origin), jitter,
                                 vel_uniform, vel_sigma, C.c_uint64(seed), x4.ctypes.data,
                                 v4.ctypes.data)
    if rc != 0:
        raise ValueError("pbfo_scene_block failed")
    return x4, v4


def dam_break(lattice, box, iterations: int, substeps: int, seed: int = 0,
              name: str = "dam") -> Scene:
    x4, v4 = block(lattice, seed=seed)
    return Scene(name, dam_params(box, iterations), x4, v4, substeps,
                 {"lattice": list(lattice), "box": list(box), "seed": seed})


def plain_16k(seed: int = 0) -> Scene:
    """16,384 particles (32x16x32) in a 64^3 box, 3 iterations, 200 substeps."""
    return dam_break((32, 16, 32), (64, 64, 64), 3, 200, seed, "dam_break_16k")


def plain_2m(seed: int = 0) -> Scene:
    """2,097,152 particles (128^3) in a 256x128x256 box, 4 iterations, 500 substeps."""
    return dam_break((128, 128, 128), (256, 128, 256), 4, 500, seed, "dam_break_2m")


def plain_262k(seed: int = 0) -> Scene:
    """262,144 particles (64^3) in a 128x64x128 box, 4 iterations."""
    return dam_break((64, 64, 64), (128, 64, 128), 4, 500, seed, "dam_break_262k")


def diff_32k(seed_a: int = 1, seed_b: int = 2):
    """32,768 particles (32^3) in a 64^3 box, velocities N(0, 0.25^2) from
    seed A and seed B, 64 substeps x 4 iterations."""
    xa, va = block((32, 32, 32), seed=seed_a, vel_sigma=0.25)
    _, vb = block((32, 32, 32), seed=seed_b, vel_sigma=0.25)
    p = dam_params((64, 64, 64), 4)
    return (Scene("diff_32k_A", p, xa, va, 64, {"seed": seed_a}),
            Scene("diff_32k_B", p.copy(), xa.copy(), vb, 64, {"seed": seed_b}))

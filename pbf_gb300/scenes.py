"""Scene and parameter builders for the dam-break workloads.

Every workload is a seeded block of particles on a lattice of spacing 0.5h in
the corner of a clamping box, with the constants h = 1, g = 9.81, dt = 0.008,
epsilon = 0.01, s_corr k = 0.1 (n = 4, dq = 0.2h), XSPH c = 0.01 and
vorticity epsilon = 0.0005, and rho_0 = the poly6 density of an unjittered
interior lattice point (self excluded).  Positions come from the library's
mt19937_64 generator (pbf_scene_block), so C++ and Python callers get the
same bytes.

The cell grid of a box [0, B] is floor(B) + 1 cells per axis, so that every
clamped position owns a cell (the reference's clamp is inclusive of the grid
size, shaders/radixsort/counting.glsl:55).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from ._capi import Params, check, load

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


def rest_density(h: float = H, spacing: float = SPACING) -> float:
    return float(load().pbf_rest_density_lattice(h, spacing))


def wpoly6(r: float, h: float = H) -> float:
    return float(load().pbf_wpoly6(r, h))


def dam_params(box, iterations: int, *, h: float = H, spacing: float = SPACING,
               xsph_c: float = XSPH_C, vort_eps: float = VORT_EPS, epsilon: float = EPSILON,
               scorr_k: float = SCORR_K, vorticity: bool = True) -> Params:
    """Parameters of a dam break in the box [0, box]."""
    lib = load()
    grid = [int(math.floor(b)) + 1 for b in box]
    p = Params()
    check(lib.pbf_params_default((C.c_uint32 * 3)(*grid), C.byref(p)))
    p.h = h
    p.one_over_rho_0 = float(np.float32(1.0 / rest_density(h, spacing)))
    p.epsilon = epsilon
    p.gravity = GRAVITY
    p.timestep = DT
    p.tensile_instability_k = scorr_k
    p.tensile_instability_scale = float(np.float32(1.0 / wpoly6(SCORR_DQ * h, h)))
    p.xsph_viscosity_c = xsph_c
    p.vorticity_epsilon = vort_eps
    p.num_solver_iterations = int(iterations)
    p.vorticity_confinement = 1 if vorticity else 0
    p.external_force = 0
    for a in range(3):
        p.wall_lo[a] = 0.0
        p.wall_hi[a] = float(box[a])
    return p


def block(lattice, *, spacing: float = SPACING, origin=None, jitter: float = JITTER,
          vel_uniform: float = 0.0, vel_sigma: float = 0.0, seed: int = 0):
    """Seeded lattice block (pbf_scene_block); returns (x4, v4) float32 arrays."""
    lib = load()
    lat = [int(v) for v in lattice]
    n = lat[0] * lat[1] * lat[2]
    if origin is None:
        origin = (0.5 * spacing,) * 3
    x4 = np.empty((n, 4), np.float32)
    v4 = np.empty((n, 4), np.float32)
    check(lib.pbf_scene_block((C.c_uint32 * 3)(*lat), spacing, (C.c_float * 3)(*origin), jitter,
                              vel_uniform, vel_sigma, C.c_uint64(seed), x4.ctypes.data,
                              v4.ctypes.data))
    return x4, v4


def dam_break(lattice, box, iterations: int, substeps: int, seed: int = 0, name: str = "dam",
              **kw) -> Scene:
    x4, v4 = block(lattice, seed=seed)
    return Scene(name, dam_params(box, iterations, **kw), x4, v4, substeps,
                 {"lattice": list(lattice), "box": list(box), "seed": seed})


def plain_16k(seed: int = 0) -> Scene:
    """16,384 particles (32x16x32) in a 64^3 box, 3 iterations, 200 substeps."""
    return dam_break((32, 16, 32), (64, 64, 64), 3, 200, seed, "dam_break_16k")


def plain_2m(seed: int = 0) -> Scene:
    """2,097,152 particles (128^3) in a 256x128x256 box, 4 iterations, 500 substeps."""
    return dam_break((128, 128, 128), (256, 128, 256), 4, 500, seed, "dam_break_2m")


def plain_262k(seed: int = 0) -> Scene:
    """262,144 particles (64^3) in a 128x64x128 box, 4 iterations: the 2M
    workload's density and constants at 1/8 the size (profiling captures)."""
    return dam_break((64, 64, 64), (128, 64, 128), 4, 500, seed, "dam_break_262k")


def diff_32k(seed_a: int = 1, seed_b: int = 2):
    """32,768 particles (32^3) in a 64^3 box, velocities N(0, 0.25^2) from a seed,
    64 substeps x 4 iterations.  Returns (scene_A, scene_B): same positions,
    velocities from seed A (the optimised start) and seed B (the target run)."""
    xa, va = block((32, 32, 32), seed=seed_a, vel_sigma=0.25)
    _, vb = block((32, 32, 32), seed=seed_b, vel_sigma=0.25)
    p = dam_params((64, 64, 64), 4)
    a = Scene("diff_32k_A", p, xa, va, 64, {"seed": seed_a})
    b = Scene("diff_32k_B", p.copy(), xa.copy(), vb, 64, {"seed": seed_b})
    return a, b


def batch_scene_specs(num_scenes: int = 256, seed: int = 7, nmin: int = 4096, nmax: int = 65536,
                      box_min: int = 32, box_max: int = 96):
    """Per-scene (lattice, box) of a batched workload: a target count drawn
    uniform-integer in [nmin, nmax], box sides uniform in [box_min, box_max]
    cells, and block dimensions (x = z near the cube root, y the rest) whose
    product is the target rounded to the block's shape, the block fitting
    inside its box at spacing 0.5."""
    rng = np.random.Generator(np.random.PCG64(seed))
    specs = []
    for _ in range(num_scenes):
        target = int(rng.integers(nmin, nmax + 1))
        box = [int(rng.integers(box_min, box_max + 1)) for _ in range(3)]
        cap = [max(1, int((b - 1) / SPACING)) for b in box]
        side = max(1, int(round(target ** (1 / 3))))
        bx = min(cap[0], side)
        bz = min(cap[2], side)
        by = max(1, min(cap[1], int(round(target / (bx * bz)))))
        specs.append({"lattice": [bx, by, bz], "box": box})
    return specs


def batch_scenes(num_scenes: int = 256, seed: int = 7, iterations: int = 4, substeps: int = 100,
                 nmin: int = 4096, nmax: int = 65536, box_min: int = 32, box_max: int = 96,
                 vel_uniform: float = 0.5) -> list[Scene]:
    """The batched dam breaks: per scene a seeded block (jitter U(-0.01h, 0.01h),
    velocities U(-0.5, 0.5)) in its own box, the shared constants above."""
    out = []
    for k, spec in enumerate(batch_scene_specs(num_scenes, seed, nmin, nmax, box_min, box_max)):
        x4, v4 = block(spec["lattice"], seed=seed * 100003 + k, vel_uniform=vel_uniform)
        out.append(Scene(f"batch{k}", dam_params(spec["box"], iterations), x4, v4, substeps,
                         {**spec, "seed": seed * 100003 + k}))
    return out


def concat_state(scenes_: list[Scene]):
    return (np.ascontiguousarray(np.concatenate([s.x4 for s in scenes_])),
            np.ascontiguousarray(np.concatenate([s.v4 for s in scenes_])))


def shard(scenes_: list[Scene], rank: int, world: int) -> list[int]:
    """Indices of the scenes rank `rank` of `world` steps when a batch is split
    across GPUs (independent scenes need no exchange): greedy by particle
    count, largest first, so every rank gets a near-equal share."""
    order = sorted(range(len(scenes_)), key=lambda k: -scenes_[k].n)
    load = [0] * world
    owner = [0] * len(scenes_)
    for k in order:
        r = min(range(world), key=lambda q: (load[q], q))
        owner[k] = r
        load[r] += scenes_[k].n
    return [k for k in range(len(scenes_)) if owner[k] == rank]


def shard_batch(scenes_: list[Scene], rank: int, world: int):
    """What one rank of a sharded batch steps: the indices of its scenes
    (shard), their parameters and particle counts, and their initial states
    concatenated in that order, the arguments of its own batched handle.
    Scenes are independent, so nothing crosses ranks on the data path."""
    idx = shard(scenes_, rank, world)
    mine = [scenes_[k] for k in idx]
    if not mine:
        return idx, [], [], np.zeros((0, 4), np.float32), np.zeros((0, 4), np.float32)
    x4, v4 = concat_state(mine)
    return idx, [s.params for s in mine], [s.n for s in mine], x4, v4


def reference_two_blocks(seed: int = 0) -> Scene:
    """The reference application's own scene (Simulation::ResetParticleBuffer,
    src/Simulation.cpp:206-246, with SPH's defaults, src/SPH.cpp:24-26,136-144):
    65,536 particles in two 32^3 blocks of spacing 0.94, one from
    (32.5, 0.5, 32.5) along +x, +y, +z and one from (95.5, 0.5, 95.5) along
    -x, +y, -z, each coordinate jittered by 0.01 * (U(0,1) - 0.5) (the
    reference's unseeded rand(); here a seeded generator), zero velocities, in
    the (128, 64, 128) grid with the reference's walls, h = 2 and 5 solver
    iterations, vorticity confinement off."""
    rng = np.random.Generator(np.random.PCG64(seed))
    blocks = []
    for origin, sign in (((32.5, 0.5, 32.5), (1, 1, 1)), ((95.5, 0.5, 95.5), (-1, 1, -1))):
        # id order x outermost, then z, then y (src/Simulation.cpp:214-229)
        gi, gk, gj = np.meshgrid(np.arange(32), np.arange(32), np.arange(32), indexing="ij")
        idx = np.stack([gi.ravel(), gj.ravel(), gk.ravel()], 1).astype(np.float64)
        pos = np.asarray(origin) + 0.94 * idx * np.asarray(sign, np.float64)
        pos += 0.01 * (rng.random(pos.shape) - 0.5)
        blocks.append(pos)
    pos = np.concatenate(blocks)
    x4 = np.zeros((pos.shape[0], 4), np.float32)
    x4[:, :3] = pos.astype(np.float32)
    v4 = np.zeros_like(x4)
    from .sph import default_params
    p = default_params((128, 64, 128))
    p.h = 2.0
    p.tensile_instability_scale = float(np.float32(1.0 / wpoly6(0.2, 2.0)))
    return Scene("reference_two_blocks", p, x4, v4, 0, {"seed": seed})

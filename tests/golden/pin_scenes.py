"""Scenes on which the reference's own shaders, compiled as C++ by
oracle/ref_build.py, are compared with the oracle and the GPU.

Each keeps the reference's boundary quirks out of play: the fluid block sits
away from the grid faces (except the below-floor case, which puts the
unclamped stencil centre of neighbourcells.glsl:57 to the test) and from the
reference's hard-coded walls (16, 0, 16)
.. GRID_SIZE - (16, 0, 16) (shaders/sph/updatepos.glsl:98-100), and two
isolated dummy particles occupy the first and the last cell, so findcells'
fixed start[(0,0,0)] = 0 and its never-written last `end`
(shaders/neighbourcellfinder/findcells.glsl:39-43) touch only them.
"""
import numpy as np

from pbf_gb300 import scenes

GRID = 48

CASES = {
    # name: (h, epsilon, vorticity, external force, iterations)
    "h1_eps0.01": (1.0, 0.01, True, False, 3),
    "h2_eps5": (2.0, 5.0, True, False, 3),
    "h1_eps5_novort": (1.0, 5.0, False, False, 2),
    "h1_eps0.01_extforce": (1.0, 0.01, True, True, 3),
    # the bottom layer moving down fast enough that its predicted positions
    # leave the grid (y from -0.5 to -3.7): neighbourcells.glsl:57 centres
    # their stencil on the outside cell without a clamp, so they find only
    # the floor row or nothing
    "h1_eps5_below_floor": (1.0, 5.0, True, False, 3),
}


def make(name):
    h, eps, vort, ext, iters = CASES[name]
    p = scenes.dam_params((GRID - 1,) * 3, iters, h=h, epsilon=eps, vorticity=vort)
    p.external_force = 1 if ext else 0
    for a, w in enumerate((16.0, 0.0, 16.0)):
        p.wall_lo[a] = w
        p.wall_hi[a] = GRID - w
    if name.endswith("below_floor"):
        x4, v4 = scenes.block((10, 4, 10), origin=(20.25, 0.25, 20.25), seed=3, vel_uniform=0.3)
        bottom = x4[:, 1] < 0.5
        v4[bottom, 1] = np.linspace(-100.0, -500.0, int(bottom.sum()), dtype=np.float32)
    else:
        x4, v4 = scenes.block((10, 8, 10), origin=(20.25, 3.25, 20.25), seed=3, vel_uniform=0.3)
    d = np.array([[0.5, 0.5, 0.5, 0], [GRID - 0.5, GRID - 0.5, GRID - 0.5, 0]], np.float32)
    z = np.zeros((1, 4), np.float32)
    return p, np.concatenate([d[:1], x4, d[1:]]), np.concatenate([z, v4, z])


def highlight_flags(n):
    """Highlight input: bit 0 (selected) on every 395th particle, stale bits 1
    and 2 elsewhere, which the clear pass must drop."""
    i = np.arange(n)
    f = np.zeros(n, np.uint32)
    f[i % 395 == 5] |= 1
    f[i % 5 == 0] |= 2
    f[i % 11 == 0] |= 4
    return f

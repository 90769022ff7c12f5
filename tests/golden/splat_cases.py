"""Scenes and cameras on which the splatting passes (pbf_splat) are compared
with the reference's own particledepth / thickness shaders compiled as C++
(oracle/ref_build.py) and with the CPU oracle.

Each case: particle positions (float4, grid units as the reference's position
buffer), a view and projection matrix (math layout), and the depth and
thickness image sizes.  The cameras cover the reference's start-up camera, a
mirrored projection (clockwise triangles on screen), an orthographic
projection (constant w: the depth pass's corner offset w of 1, which the
reference adds in particledepth/vertex.glsl:41, then halves the sprite
positions on screen), two projections whose clip z depends on x (sprites that
straddle the near and far planes, clipped per fragment) and a camera inside
the fluid (sprites behind the eye and cut by the near plane).
"""
import math

import numpy as np

from pbf_gb300 import scenes, splat

CASES = ["reference", "mirrored", "ortho", "skewed_a", "skewed_b", "inside"]


def _positions(kind):
    if kind == "blocks":
        s = scenes.reference_two_blocks(seed=0)
        return np.ascontiguousarray(s.x4[::16])
    rng = np.random.default_rng(11)
    x = np.zeros((3000, 4), np.float32)
    x[:, :3] = rng.uniform((40, 0, 40), (90, 40, 90), (3000, 3)).astype(np.float32)
    return x


def make(name):
    """Returns (x4, viewmat, projmat, (depth W, H), (thickness W, H))."""
    if name == "reference":
        v = splat.reference_view(320, 180)
        V, P = v.matrices()
        return _positions("blocks"), V, P, (320, 180), (128, 128)
    if name == "mirrored":
        v = splat.reference_view(200, 150)
        V, P = v.matrices()
        P = P.copy()
        P[0, 0] = -P[0, 0]
        return _positions("blocks"), V, P, (200, 150), (96, 96)
    if name == "ortho":
        V = splat.look_at((0.0, 30.0, 0.1), (0.0, 0.0, 0.0), (0.0, 0.0, -1.0))
        P = np.zeros((4, 4))
        P[0, 0], P[1, 1], P[2, 2], P[2, 3], P[3, 3] = 1 / 14.0, 1 / 14.0, -2 / 60.0, -1.0, 1.0
        return _positions("cloud"), V, P, (160, 160), (64, 64)
    if name in ("skewed_a", "skewed_b"):
        # clip z grows with view x: the near and far planes cut sprites
        near, far, skew = (12.0, 60.0, 0.5) if name == "skewed_a" else (5.0, 20.0, 0.3)
        V = splat.look_at((0.0, 8.0, 25.0), (0.0, 4.0, 0.0), (0.0, 1.0, 0.0))
        P = splat.perspective(math.radians(50.0), 4 / 3, near, far)
        P[2, 0] = skew
        return _positions("cloud"), V, P, (240, 180), (80, 80)
    if name == "inside":
        V = splat.look_at((1.0, 3.0, 1.0), (-3.0, 2.0, -4.0), (0.0, 1.0, 0.0))
        P = splat.perspective(math.radians(70.0), 16 / 9, 0.05, 40.0)
        return _positions("cloud"), V, P, (192, 108), (72, 72)
    raise KeyError(name)


def columns(m):
    return np.ascontiguousarray(np.asarray(m, np.float32).T.reshape(16))

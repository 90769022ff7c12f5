"""Headless splatting: SurfaceReconstruction's particle depth and thickness
passes (src/SurfaceReconstruction.cpp:176-231) through ``pbf_splat``, into
device buffers instead of GL framebuffers.

``reference_view`` builds the reference application's camera
(src/Simulation.cpp:42-43,103: eye (20, 10, 10), rotated 240 degrees about y
and 30 degrees about x, 45-degree perspective with near 1 and far 200), in the
column-major layout of its TransformationBlock.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from ._capi import check, load

DEPTH = 0
THICKNESS = 1


class View(C.Structure):
    """pbf_view (include/pbf.h): column-major 4x4 view and projection."""

    _fields_ = [("viewmat", C.c_float * 16), ("projmat", C.c_float * 16)]

    @staticmethod
    def of(viewmat, projmat) -> "View":
        v = View()
        vm = np.asarray(viewmat, np.float32).reshape(4, 4)
        pm = np.asarray(projmat, np.float32).reshape(4, 4)
        # accept math (row-major) 4x4 arrays: store their columns
        v.viewmat[:] = [float(a) for a in vm.T.reshape(16)]
        v.projmat[:] = [float(a) for a in pm.T.reshape(16)]
        return v

    def matrices(self):
        """(view, projection) as math 4x4 arrays."""
        return (np.array(self.viewmat[:], np.float32).reshape(4, 4).T,
                np.array(self.projmat[:], np.float32).reshape(4, 4).T)

    def columns(self):
        """(view, projection) as column-major float32[16] (the ABI layout)."""
        return np.array(self.viewmat[:], np.float32), np.array(self.projmat[:], np.float32)


def look_at(eye, center, up) -> np.ndarray:
    """Right-handed view matrix (the gluLookAt construction), math layout."""
    eye, center, up = (np.asarray(a, np.float64) for a in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def perspective(fovy: float, aspect: float, near: float, far: float) -> np.ndarray:
    """Right-handed perspective projection to clip z in [-w, w], math layout."""
    t = math.tan(fovy / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0 / (aspect * t)
    m[1, 1] = 1.0 / t
    m[2, 2] = -(far + near) / (far - near)
    m[2, 3] = -2.0 * far * near / (far - near)
    m[3, 2] = -1.0
    return m


def _rot(axis, deg):
    a = math.radians(deg)
    c, s = math.cos(a), math.sin(a)
    x, y, z = axis
    return np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                     [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                     [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])


def reference_view(width: int = 1280, height: int = 720, eye=(20.0, 10.0, 10.0), xangle=30.0,
                   yangle=240.0) -> View:
    """The reference application's start-up camera (Camera::Rotate, then
    Camera::GetViewMatrix, src/Camera.cpp:37-60) and projection for a
    width x height framebuffer."""
    rot = _rot((0.0, 1.0, 0.0), yangle) @ _rot((1.0, 0.0, 0.0), xangle)
    d = rot @ np.array([0.0, 0.0, 1.0])
    up = rot @ np.array([0.0, 1.0, 0.0])
    eye = np.asarray(eye, np.float64)
    return View.of(look_at(eye, eye + d, up),
                   perspective(math.radians(45.0), width / height, 1.0, 200.0))


def splat_device(pass_: int, positions_ptr: int, n: int, view: View, width: int, height: int,
                 out_ptr: int, stream_ptr: int = 0) -> None:
    """pbf_splat on caller device buffers (float4[n] positions, float[height][width] out)."""
    check(load().pbf_splat(int(pass_), positions_ptr, int(n), C.byref(view), int(width),
                           int(height), out_ptr, stream_ptr or None))


def splat(pass_: int, positions, view: View, width: int, height: int):
    """Splats positions (float32 (n, 4), a numpy array or a CUDA tensor) and
    returns the float32 [height, width] image (row 0 at the bottom) as a CUDA
    tensor."""
    import torch
    x = positions
    if not isinstance(x, torch.Tensor):
        x = torch.from_numpy(np.ascontiguousarray(x, np.float32))
    x = x.to(device="cuda", dtype=torch.float32).contiguous()
    if x.dim() != 2 or x.shape[1] != 4:
        raise ValueError("positions must have shape (n, 4)")
    out = torch.empty((int(height), int(width)), dtype=torch.float32, device=x.device)
    splat_device(pass_, x.data_ptr(), x.shape[0], view, width, height, out.data_ptr(),
                 torch.cuda.current_stream(x.device).cuda_stream)
    return out

"""Python mirror of the reference's ``SPH`` class (src/SPH.h) over the C ABI.

Method names, argument meaning and defaults follow src/SPH.h:40-235 so code
written against the reference reads the same:

    sph = SPH(numparticles, gridsize=(128, 64, 128))
    sph.SetRestDensity(rho0); sph.SetNumSolverIterations(4)
    sph.set_state(x4, v4)        # what Simulation::ResetParticleBuffer uploads
    sph.Run()                    # one substep (SPH::Run)
    x4 = sph.positions()         # contents of GetPositionBuffer

Errors raise :class:`PbfError` carrying the C status code.  All compute runs
in libpbf_gb300.so on the GPU; this module only marshals arguments.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import (PBF_DEVICE, PBF_HOST, Diagnostics, ParamGrads, Params, PbfError, Tuning,
                    check, load)


def default_params(gridsize=(128, 64, 128)) -> Params:
    """Reference defaults (src/SPH.cpp:136-144) for a grid, h = 1."""
    lib = load()
    p = Params()
    g = (C.c_uint32 * 3)(*[int(v) for v in gridsize])
    check(lib.pbf_params_default(g, C.byref(p)))
    return p


def _f32(v) -> float:
    return float(np.float32(v))


def _as_f4(a, n: int) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.shape == (n, 3):
        a = np.ascontiguousarray(np.concatenate([a, np.zeros((n, 1), np.float32)], axis=1))
    if a.shape != (n, 4):
        raise ValueError(f"expected shape ({n}, 4) or ({n}, 3), got {a.shape}")
    return a


class SPH:
    """One simulation handle (``pbf_sim``), the counterpart of ``SPH``."""

    def __init__(self, numparticles: int, gridsize=(128, 64, 128), params: Params | None = None,
                 lib=None):
        # lib: another build of the library with the same entry points (the
        # bounds-checked one, _capi.load_checked()); default the normal build
        self._lib = lib if lib is not None else load()
        p = params.copy() if params is not None else default_params(gridsize)
        if params is not None and tuple(p.grid) != tuple(int(g) for g in gridsize):
            gridsize = tuple(p.grid)
        self._params = p
        self._n = int(numparticles)
        h = C.c_void_p()
        check(self._lib.pbf_create(C.byref(p), self._n, C.byref(h)))
        self._h = h

    # ---- lifetime --------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.pbf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    @property
    def numparticles(self) -> int:
        return self._n

    @property
    def params(self) -> Params:
        return self._params.copy()

    def set_params(self, p: Params) -> None:
        check(self._lib.pbf_set_params(self._h, C.byref(p)), self._h)
        self._params = p.copy()

    def _update(self, **kw) -> None:
        p = self._params.copy()
        for k, v in kw.items():
            setattr(p, k, v)
        self.set_params(p)

    # ---- reference setters / getters (src/SPH.h:57-230) -------------------
    def GetRestDensity(self) -> float:
        return _f32(np.float32(1.0) / np.float32(self._params.one_over_rho_0))

    def SetRestDensity(self, rho: float) -> None:
        self._update(one_over_rho_0=_f32(np.float32(1.0) / np.float32(rho)))

    def GetCFMEpsilon(self) -> float:
        return self._params.epsilon

    def SetCFMEpsilon(self, eps: float) -> None:
        self._update(epsilon=_f32(eps))

    def GetGravity(self) -> float:
        return self._params.gravity

    def SetGravity(self, g: float) -> None:
        self._update(gravity=_f32(g))

    def GetTimestep(self) -> float:
        return self._params.timestep

    def SetTimestep(self, dt: float) -> None:
        self._update(timestep=_f32(dt))

    def GetTensileInstabilityK(self) -> float:
        return self._params.tensile_instability_k

    def SetTensileInstabilityK(self, k: float) -> None:
        self._update(tensile_instability_k=_f32(k))

    def GetTensileInstabilityScale(self) -> float:
        return self._params.tensile_instability_scale

    def SetTensileInstabilityScale(self, v: float) -> None:
        self._update(tensile_instability_scale=_f32(v))

    def GetXSPHViscosity(self) -> float:
        return self._params.xsph_viscosity_c

    def SetXSPHViscosity(self, c: float) -> None:
        self._update(xsph_viscosity_c=_f32(c))

    def GetVorticityEpsilon(self) -> float:
        return self._params.vorticity_epsilon

    def SetVorticityEpsilon(self, eps: float) -> None:
        self._update(vorticity_epsilon=_f32(eps))

    def GetNumSolverIterations(self) -> int:
        return int(self._params.num_solver_iterations)

    def SetNumSolverIterations(self, it: int) -> None:
        self._update(num_solver_iterations=int(it))

    def IsVorticityConfinementEnabled(self) -> bool:
        return bool(self._params.vorticity_confinement)

    def SetVorticityConfinementEnabled(self, flag: bool) -> None:
        self._update(vorticity_confinement=1 if flag else 0)

    def SetExternalForce(self, state: bool) -> None:
        self._update(external_force=1 if state else 0)

    # ---- tuning (no result depends on it) ---------------------------------
    def get_tuning(self) -> Tuning:
        t = Tuning()
        check(self._lib.pbf_get_tuning(self._h, C.byref(t)), self._h)
        return t

    def set_tuning(self, use_neighbour_lists=None, list_capacity=None, skin_h=None,
                   block_size=None, sweep_mode=None, pair_list_capacity=None,
                   coop_candidates=None, auto_period=None,
                   adjoint_warp_candidates=None) -> None:
        t = self.get_tuning()
        if use_neighbour_lists is not None:
            t.use_neighbour_lists = 1 if use_neighbour_lists else 0
        if list_capacity is not None:
            t.list_capacity = int(list_capacity)
        if skin_h is not None:
            t.skin_h = float(skin_h)
        if block_size is not None:
            t.block_size = int(block_size)
        if sweep_mode is not None:
            t.sweep_mode = {"direct": _capi.PBF_SWEEP_DIRECT, "masked": _capi.PBF_SWEEP_MASKED,
                            "coop": _capi.PBF_SWEEP_COOP,
                            "auto": _capi.PBF_SWEEP_AUTO}.get(sweep_mode, sweep_mode)
        if pair_list_capacity is not None:
            t.pair_list_capacity = int(pair_list_capacity)
        if coop_candidates is not None:
            t.coop_candidates = int(coop_candidates)
        if auto_period is not None:
            t.auto_period = int(auto_period)
        if adjoint_warp_candidates is not None:
            t.adjoint_warp_candidates = int(adjoint_warp_candidates)
        check(self._lib.pbf_set_tuning(self._h, C.byref(t)), self._h)

    PASSES = ("masked", "direct", "coop", "direct+coop", "mixed")

    def sweep_choice(self) -> dict:
        """The configurations the next substep runs for the solver sweeps and
        the vorticity passes, and the automatic-mode trials so far
        (pbf_get_sweep_choice)."""
        out = (C.c_uint32 * 3)()
        check(self._lib.pbf_get_sweep_choice(self._h, out), self._h)
        return {"solver": self.PASSES[out[0]], "vorticity": self.PASSES[out[1]],
                "trials": int(out[2])}

    def autotune(self, trial_substeps: int = 10) -> dict:
        """Picks the fastest tuning for the current state (pbf_autotune)."""
        t = Tuning()
        check(self._lib.pbf_autotune(self._h, int(trial_substeps), C.byref(t)), self._h)
        return {name: getattr(t, name) for name, _ in Tuning._fields_}

    # ---- state ------------------------------------------------------------
    def set_state(self, x4, v4) -> None:
        """Uploads positions and velocities (id order, (n,4) or (n,3) float32)."""
        x = _as_f4(x4, self._n)
        v = _as_f4(v4, self._n)
        check(self._lib.pbf_set_state(self._h, x.ctypes.data, v.ctypes.data, PBF_HOST), self._h)

    def set_state_device(self, x_ptr: int, v_ptr: int) -> None:
        check(self._lib.pbf_set_state(self._h, x_ptr, v_ptr, PBF_DEVICE), self._h)

    def get_state(self) -> tuple[np.ndarray, np.ndarray]:
        x = np.empty((self._n, 4), np.float32)
        v = np.empty((self._n, 4), np.float32)
        check(self._lib.pbf_get_state(self._h, x.ctypes.data, v.ctypes.data, PBF_HOST), self._h)
        return x, v

    def get_state_into(self, x_ptr, v_ptr, where=PBF_HOST) -> None:
        check(self._lib.pbf_get_state(self._h, x_ptr, v_ptr, where), self._h)

    def positions(self) -> np.ndarray:
        return self.get_state()[0]

    def velocities(self) -> np.ndarray:
        return self.get_state()[1]

    def GetPositionBuffer(self) -> int:
        """Device address of the id-order float4 position array."""
        x = C.c_void_p()
        check(self._lib.pbf_device_buffers(self._h, C.byref(x), None), self._h)
        return int(x.value)

    def GetVelocityBuffer(self) -> int:
        """Device address of the id-order float4 velocity array."""
        v = C.c_void_p()
        check(self._lib.pbf_device_buffers(self._h, None, C.byref(v)), self._h)
        return int(v.value)

    def save_state(self, path: str) -> None:
        """Binary snapshot of x, v (pbf_save_state)."""
        check(self._lib.pbf_save_state(self._h, str(path).encode()), self._h)

    def load_state(self, path: str) -> None:
        check(self._lib.pbf_load_state(self._h, str(path).encode()), self._h)

    def highlight_flags(self, flags) -> None:
        """The highlight pass on a flag buffer (the reference's highlight
        buffer, src/SPH.h:201-207), updated in place: a uint32 numpy array, or
        a contiguous int32/uint32 CUDA tensor on this handle's device.  Bit 0
        marks selected particles; bit 1 is cleared and set on every stencil
        candidate of a selected particle, from the last substep's sort."""
        if isinstance(flags, np.ndarray):
            if flags.dtype != np.uint32 or flags.shape != (self._n,) or not flags.flags.c_contiguous:
                raise ValueError("flags must be a contiguous uint32 array of one entry per particle")
            check(self._lib.pbf_highlight_neighbours(self._h, flags.ctypes.data, PBF_HOST), self._h)
            return
        import torch
        if not (isinstance(flags, torch.Tensor) and flags.is_cuda and flags.is_contiguous()
                and flags.numel() == self._n and flags.element_size() == 4):
            raise ValueError("flags must be a contiguous 4-byte CUDA tensor of one entry per particle")
        torch.cuda.current_stream(flags.device).synchronize()
        check(self._lib.pbf_highlight_neighbours(self._h, flags.data_ptr(), PBF_DEVICE), self._h)

    def highlight_neighbours(self, selected) -> np.ndarray:
        """Flags with bit 0 on the `selected` ids and bit 1 on their stencil
        candidates in the last substep."""
        flags = np.zeros(self._n, np.uint32)
        flags[np.asarray(selected, np.int64)] = 1
        self.highlight_flags(flags)
        return flags

    # ---- stepping -----------------------------------------------------------
    def Run(self) -> None:
        """One substep (SPH::Run, src/SPH.cpp:246-334); asynchronous."""
        check(self._lib.pbf_step(self._h, 1), self._h)

    def step(self, substeps: int) -> None:
        check(self._lib.pbf_step(self._h, int(substeps)), self._h)

    def synchronize(self) -> None:
        check(self._lib.pbf_synchronize(self._h), self._h)

    def set_stream(self, stream_ptr: int | None) -> None:
        check(self._lib.pbf_set_stream(self._h, stream_ptr), self._h)

    def device_status(self) -> int:
        bits = C.c_uint32()
        check(self._lib.pbf_device_status(self._h, C.byref(bits)), self._h)
        return int(bits.value)

    # ---- timing (SPH::OutputTiming, src/SPH.cpp:218-240) ---------------------
    def EnableTiming(self, enable: bool = True) -> None:
        check(self._lib.pbf_enable_timing(self._h, 1 if enable else 0), self._h)

    def OutputTiming(self) -> dict:
        ms = (C.c_float * 5)()
        check(self._lib.pbf_get_timing(self._h, ms), self._h)
        names = ("predict", "sort", "neighbour_cells", "solver", "vorticity")
        return {k: float(v) for k, v in zip(names, ms)}

    STAGES = ("predict", "sort", "cells", "lambda", "delta_p", "commit", "vorticity_a",
              "vorticity_b")

    def stage_times(self) -> tuple[dict, int]:
        """Per-stage millisecond sums since EnableTiming, and the substep count."""
        ms = (C.c_double * 8)()
        cnt = C.c_uint32()
        check(self._lib.pbf_get_stage_times(self._h, ms, C.byref(cnt)), self._h)
        return {k: float(v) for k, v in zip(self.STAGES, ms)}, int(cnt.value)

    def kernels_per_substep(self) -> int:
        return int(self._lib.pbf_kernels_per_substep(self._h))

    def kernels_launched(self) -> int:
        """Kernels launched by this handle's substeps so far (pbf_kernels_launched)."""
        return int(self._lib.pbf_kernels_launched(self._h))

    # ---- differentiation ------------------------------------------------------
    PARAM_NAMES = ("epsilon", "tensile_instability_k", "xsph_viscosity_c", "vorticity_epsilon")

    def forward_record(self, substeps: int, checkpoint_every: int = 8) -> None:
        """Steps like step() and records what backward() needs (pbf_forward_record)."""
        check(self._lib.pbf_forward_record(self._h, int(substeps), int(checkpoint_every)),
              self._h)

    def backward(self, dL_dx=None, dL_dv=None):
        """Gradients at the start of the recorded run: (dL/dx0, dL/dv0, per-scene
        parameter gradients as an (num_scenes, 4) array in PARAM_NAMES order)."""
        n = self._n
        gx = None if dL_dx is None else _as_f4(dL_dx, n)
        gv = None if dL_dv is None else _as_f4(dL_dv, n)
        dx0 = np.empty((n, 4), np.float32)
        dv0 = np.empty((n, 4), np.float32)
        ns = int(self._lib.pbf_num_scenes(self._h))
        grads = (ParamGrads * ns)()
        check(self._lib.pbf_backward(self._h, None if gx is None else gx.ctypes.data,
                                     None if gv is None else gv.ctypes.data, PBF_HOST,
                                     dx0.ctypes.data, dv0.ctypes.data, grads), self._h)
        g = np.array([[getattr(grads[k], nm) for nm in self.PARAM_NAMES] for k in range(ns)])
        return dx0, dv0, g

    def backward_device(self, gx_ptr, gv_ptr, dx0_ptr, dv0_ptr):
        """backward() on device buffers (float4, id order); returns the parameter gradients."""
        ns = int(self._lib.pbf_num_scenes(self._h))
        grads = (ParamGrads * ns)()
        check(self._lib.pbf_backward(self._h, gx_ptr, gv_ptr, PBF_DEVICE, dx0_ptr, dv0_ptr, grads),
              self._h)
        return np.array([[getattr(grads[k], nm) for nm in self.PARAM_NAMES] for k in range(ns)])

    def release_record(self) -> None:
        check(self._lib.pbf_release_record(self._h), self._h)

    # ---- debug reads of the last substep ---------------------------------------
    def get_sort(self) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        kb = np.empty(self._n, np.uint32)
        sk = np.empty(self._n, np.uint32)
        pm = np.empty(self._n, np.uint32)
        check(self._lib.pbf_get_sort(self._h, kb.ctypes.data, sk.ctypes.data, pm.ctypes.data),
              self._h)
        return kb, sk, pm

    def get_cells(self) -> tuple[np.ndarray, np.ndarray]:
        nc = int(self._lib.pbf_num_cells(self._h))
        st = np.empty(nc, np.int32)
        en = np.empty(nc, np.int32)
        check(self._lib.pbf_get_cells(self._h, st.ctypes.data, en.ctypes.data), self._h)
        return st, en

    def get_solver(self) -> tuple[np.ndarray, np.ndarray]:
        lam = np.empty(self._n, np.float32)
        xp = np.empty((self._n, 4), np.float32)
        check(self._lib.pbf_get_solver(self._h, lam.ctypes.data, xp.ctypes.data), self._h)
        return lam, xp

    def diagnostics(self) -> dict:
        d = Diagnostics()
        check(self._lib.pbf_compute_diagnostics(self._h, C.byref(d)), self._h)
        return {name: getattr(d, name) for name, _ in Diagnostics._fields_}


class SPHBatch(SPH):
    """Several independent scenes in one handle (pbf_create_batch).

    State arrays are the scenes' float4 arrays concatenated in scene order;
    every stage runs as one launch over all scenes, and each scene steps
    bit-identically to the same scene in its own :class:`SPH`.
    """

    def __init__(self, scene_params, scene_counts, lib=None):
        self._lib = lib if lib is not None else load()
        ps = list(scene_params)
        counts = [int(c) for c in scene_counts]
        if len(ps) != len(counts) or not ps:
            raise ValueError("one particle count per scene")
        arr = (Params * len(ps))(*[p.copy() for p in ps])
        cnt = (C.c_uint32 * len(counts))(*counts)
        h = C.c_void_p()
        check(self._lib.pbf_create_batch(arr, cnt, len(ps), C.byref(h)))
        self._h = h
        self._n = sum(counts)
        self._params = ps[0].copy()
        self._scene_params = [p.copy() for p in ps]
        self._counts = counts
        self._offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)

    @property
    def num_scenes(self) -> int:
        return len(self._counts)

    def scene_slice(self, k: int) -> slice:
        return slice(int(self._offsets[k]), int(self._offsets[k + 1]))

    def scene_params(self, k: int) -> Params:
        return self._scene_params[k].copy()

    def set_scene_params(self, k: int, p: Params) -> None:
        check(self._lib.pbf_set_scene_params(self._h, int(k), C.byref(p)), self._h)
        self._scene_params[k] = p.copy()
        if k == 0:
            self._params = p.copy()

    def set_params(self, p: Params) -> None:
        raise PbfError(1, "a batch takes set_scene_params")


__all__ = ["SPH", "SPHBatch", "default_params", "PbfError"]

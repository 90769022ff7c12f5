"""CPU oracle of the PBF substep path — TEST INFRASTRUCTURE ONLY.

A C++ restatement of the reference's GLSL compute shaders (pbf_oracle.hpp),
FP32 and an FP64 twin, OpenMP-parallel over particles.  Only tests/,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use
it, and only as the checker or the timed CPU baseline: the product
(pbf_gb300/) never imports, links or calls it.

Parity status: the reference runs only inside an OpenGL 4.3 context, which
neither machine here has, and it ships no tests or golden vectors.  Its
compute shaders are compiled as C++ by ref_build.py (from the reference
checkout, interface declarations rewritten, bodies as written) and the oracle
is checked against them (tests/test_ref_pin.py); their outputs are committed
as fixtures (tests/golden/).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpbf_oracle.so")
SRC = [os.path.join(HERE, "pbf_oracle.cpp"), os.path.join(HERE, "pbf_oracle.hpp"),
       os.path.join(HERE, "pbf_splat_oracle.cpp"), os.path.join(HERE, "pbf_scene_oracle.cpp"),
       os.path.join(HERE, "pbf_dual.cpp"), os.path.join(HERE, "pbf_dual.hpp")]

CXXFLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    """Compiles the oracle with g++ (no -ffast-math, contraction off)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and all(
            os.path.getmtime(LIB) >= os.path.getmtime(s) for s in SRC):
        return LIB
    tmp = LIB + ".tmp"
    cxx = os.environ.get("CXX", "g++")
    # the dual-number twin at -O3 (its tangent loops vectorise, ~4x faster);
    # no flag here changes a floating-point result (no fast-math, no contraction)
    dual_obj = os.path.join(BUILD, "pbf_dual.o")
    cmds = [[cxx] + [f for f in CXXFLAGS if f not in ("-O2", "-shared")] +
            ["-O3", "-c", "-o", dual_obj, SRC[4]],
            [cxx] + CXXFLAGS + ["-o", tmp, SRC[0], SRC[2], SRC[3], dual_obj]]
    for cmd in cmds:
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stderr)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        lib = C.CDLL(LIB)
        P = C.c_void_p
        lib.pbfo_params_size.restype = C.c_int
        lib.pbfo_create.restype = P
        lib.pbfo_create.argtypes = [P, C.c_uint32, C.c_int, C.c_int]
        lib.pbfo_destroy.argtypes = [P]
        lib.pbfo_set_params.argtypes = [P, P]
        lib.pbfo_set_state.argtypes = [P, P, P]
        lib.pbfo_get_state.argtypes = [P, P, P]
        lib.pbfo_step.restype = C.c_double
        lib.pbfo_step.argtypes = [P, C.c_uint32]
        lib.pbfo_get_sort.argtypes = [P, P, P, P]
        lib.pbfo_get_cells.argtypes = [P, P, P]
        lib.pbfo_get_solver.argtypes = [P, P, P]
        lib.pbfo_get_runs.argtypes = [P, C.c_uint32, P]
        lib.pbfo_get_consts.argtypes = [P, P]
        lib.pbfo_diagnostics.argtypes = [P, P]
        lib.pbfo_radix_sort.argtypes = [P, C.c_uint32, C.c_uint32, P, P]
        lib.pbfo_highlight.argtypes = [P, P]
        lib.pbfo_splat.argtypes = [C.c_int, P, C.c_uint32, P, P, C.c_uint32, C.c_uint32, P]
        lib.pbfo_max_threads.restype = C.c_int
        lib.pbfo_sample_substep.restype = C.c_double
        lib.pbfo_sample_substep.argtypes = [P, C.c_uint32, C.c_uint32, P, P]
        lib.pbfo_wpoly6.restype = C.c_double
        lib.pbfo_wpoly6.argtypes = [C.c_double, C.c_double]
        lib.pbfo_rest_density_lattice.restype = C.c_double
        lib.pbfo_rest_density_lattice.argtypes = [C.c_double, C.c_double]
        lib.pbfo_params_default.restype = C.c_int
        lib.pbfo_params_default.argtypes = [P, P]
        for fn in (lib.pbfo_dual_tangents, lib.pbfo_dual_tangents_fp32):
            fn.restype = C.c_int
            fn.argtypes = [P, C.c_uint32, P, P, C.c_uint32, C.c_uint32, P, P, P, P, P, P, P,
                           C.c_int]
        lib.pbfo_scene_block.restype = C.c_int
        lib.pbfo_scene_block.argtypes = [P, C.c_float, P, C.c_float, C.c_float, C.c_float,
                                         C.c_uint64, P, P]
        _lib = lib
    return _lib


def max_threads() -> int:
    return int(load().pbfo_max_threads())


class Oracle:
    """One oracle simulation (FP32, or the FP64 twin with fp64=True)."""

    def __init__(self, params, n: int, fp64: bool = False, threads: int = 0):
        self._lib = load()
        self.fp64 = bool(fp64)
        self.n = int(n)
        self._params = params
        self.ncells = int(params.grid[0]) * int(params.grid[1]) * int(params.grid[2])
        self._h = self._lib.pbfo_create(C.addressof(params), self.n, int(fp64), int(threads))
        self._rt = np.float64 if fp64 else np.float32

    def close(self):
        if self._h:
            self._lib.pbfo_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        self._params = params
        self._lib.pbfo_set_params(self._h, C.addressof(params))

    def set_state(self, x4, v4):
        x = np.ascontiguousarray(x4, np.float32)
        v = np.ascontiguousarray(v4, np.float32)
        assert x.shape == (self.n, 4) and v.shape == (self.n, 4)
        self._lib.pbfo_set_state(self._h, x.ctypes.data, v.ctypes.data)

    def get_state(self):
        x = np.empty((self.n, 4), self._rt)
        v = np.empty((self.n, 4), self._rt)
        self._lib.pbfo_get_state(self._h, x.ctypes.data, v.ctypes.data)
        return x, v

    def step(self, substeps: int = 1) -> float:
        """Runs substeps; returns wall seconds."""
        return float(self._lib.pbfo_step(self._h, int(substeps)))

    def get_sort(self):
        kb = np.empty(self.n, np.uint32)
        sk = np.empty(self.n, np.uint32)
        pm = np.empty(self.n, np.uint32)
        self._lib.pbfo_get_sort(self._h, kb.ctypes.data, sk.ctypes.data, pm.ctypes.data)
        return kb, sk, pm

    def get_cells(self):
        st = np.empty(self.ncells, np.int32)
        en = np.empty(self.ncells, np.int32)
        self._lib.pbfo_get_cells(self._h, st.ctypes.data, en.ctypes.data)
        return st, en

    def get_solver(self):
        lam = np.empty(self.n, self._rt)
        xp = np.empty((self.n, 4), self._rt)
        self._lib.pbfo_get_solver(self._h, lam.ctypes.data, xp.ctypes.data)
        return lam, xp

    def get_runs(self, i: int):
        r = np.empty(18, np.int32)
        self._lib.pbfo_get_runs(self._h, int(i), r.ctypes.data)
        return r.reshape(9, 2)

    def highlight(self, flags):
        """Highlight pass over the last substep's runs (see pbfo_highlight)."""
        f = np.ascontiguousarray(flags, np.uint32).copy()
        assert f.shape == (self.n,)
        self._lib.pbfo_highlight(self._h, f.ctypes.data)
        return f

    def consts(self):
        out = np.empty(4, np.float64)
        self._lib.pbfo_get_consts(self._h, out.ctypes.data)
        return {"k6": out[0], "kg": out[1], "kg_lambda": out[2], "h2": out[3]}

    def sample_substep(self, lo: int, hi: int):
        """Timing sample: (extrapolated s per substep, s of all-particle stages, s of slice)."""
        tf = C.c_double()
        ts = C.c_double()
        tot = self._lib.pbfo_sample_substep(self._h, int(lo), int(hi), C.addressof(tf),
                                            C.addressof(ts))
        return float(tot), tf.value, ts.value

    def diagnostics(self):
        out = np.empty(4, np.float64)
        self._lib.pbfo_diagnostics(self._h, out.ctypes.data)
        return {"mean_density_error": out[0], "max_density_error": out[1],
                "kinetic_energy": out[2], "candidate_pairs": out[3]}


DUAL_KINDS = {"v": 0, "x": 1, "epsilon": 2, "tensile_instability_k": 3, "xsph_viscosity_c": 4,
              "vorticity_epsilon": 5}


def dual_tangents(params, x4, v4, substeps: int, directions, threads: int = 0, fp32: bool = False):
    """Forward-mode derivatives of the FP64 twin (pbf_dual.cpp), or with
    fp32=True of the FP32 oracle's own trajectory: `directions` is a list of
    ("v" | "x", index, component) or (scalar name,) tuples.  Returns
    (x_N, v_N, xdot, vdot): the final state (n, 3) in double, equal to the
    FP64 twin's (or the FP32 oracle's), and its tangents (ndir, n, 3)."""
    lib = load()
    x = np.ascontiguousarray(x4, np.float32)
    v = np.ascontiguousarray(v4, np.float32)
    n = x.shape[0]
    nd = len(directions)
    kind = np.array([DUAL_KINDS[d[0]] for d in directions], np.int32)
    idx = np.array([int(d[1]) if len(d) > 1 else 0 for d in directions], np.int32)
    comp = np.array([int(d[2]) if len(d) > 2 else 0 for d in directions], np.int32)
    xo = np.empty((n, 3), np.float64)
    vo = np.empty((n, 3), np.float64)
    xd = np.empty((nd, n, 3), np.float64)
    vd = np.empty((nd, n, 3), np.float64)
    fn = lib.pbfo_dual_tangents_fp32 if fp32 else lib.pbfo_dual_tangents
    rc = fn(C.addressof(params), n, x.ctypes.data, v.ctypes.data, int(substeps),
                                nd, kind.ctypes.data, idx.ctypes.data, comp.ctypes.data,
                                xo.ctypes.data, vo.ctypes.data, xd.ctypes.data, vd.ctypes.data,
                                int(threads))
    if rc != 0:
        raise ValueError("pbfo_dual_tangents: bad argument")
    return xo, vo, xd, vd


def radix_sort(keys, numbits: int):
    """Stable sort of keys on their low numbits bits: (sorted keys, perm)."""
    lib = load()
    k = np.ascontiguousarray(keys, np.uint32)
    n = k.shape[0]
    ko = np.empty(n, np.uint32)
    po = np.empty(n, np.uint32)
    lib.pbfo_radix_sort(k.ctypes.data, n, int(numbits), ko.ctypes.data, po.ctypes.data)
    return ko, po


def splat(pass_: int, x4, viewmat, projmat, width: int, height: int):
    """SurfaceReconstruction's particle passes on the CPU (pbf_splat_oracle.cpp):
    pass 0 depth, 1 thickness; matrices column-major (16 floats).  Returns
    float32 [height, width], row 0 at the bottom."""
    x = np.ascontiguousarray(x4, np.float32)
    assert x.ndim == 2 and x.shape[1] == 4
    V = np.ascontiguousarray(viewmat, np.float32).reshape(16)
    P = np.ascontiguousarray(projmat, np.float32).reshape(16)
    out = np.empty((int(height), int(width)), np.float32)
    load().pbfo_splat(int(pass_), x.ctypes.data, x.shape[0], V.ctypes.data, P.ctypes.data,
                      int(width), int(height), out.ctypes.data)
    return out


def params_size() -> int:
    return int(load().pbfo_params_size())


# ---- the reference's own shaders compiled as C++ (oracle/ref_build.py) ---------

def ref_available() -> bool:
    """True when the reference checkout is present here (the library is built
    from its shader files; it cannot be built where the checkout is absent)."""
    from . import ref_build
    return ref_build.available()


_ref = None


def ref_load() -> C.CDLL:
    global _ref
    if _ref is None:
        from . import ref_build
        path = ref_build.build()
        if path is None:
            raise RuntimeError("the reference checkout is absent: its shaders cannot be built")
        lib = C.CDLL(path)
        P = C.c_void_p
        lib.pbfr_substep.argtypes = [P, C.c_uint32, P, P, P, P, P, P, P]
        lib.pbfr_substep.restype = C.c_int
        lib.pbfr_substep_highlight.argtypes = [P, C.c_uint32, P, P, P, P, P, P, P, P]
        lib.pbfr_substep_highlight.restype = C.c_int
        lib.pbfr_splat.argtypes = [C.c_int, P, C.c_uint32, P, P, C.c_uint32, C.c_uint32, P]
        lib.pbfr_splat.restype = C.c_int
        lib.pbfr_set_cell_fix.argtypes = [C.c_int]
        lib.pbfr_set_cell_fix.restype = None
        _ref = lib
    return _ref


def ref_substep(params, x4, v4, highlight=None, cell_fix: int = 2):
    """One SPH::Run of the reference's shaders.  Returns a dict with x, v (id
    order), sorted ids, the grid start/end textures (x fastest, then y, z),
    the packed neighbour texture (n, 3, 4) and lambda (sorted order); with
    `highlight` (uint32[n] flags, id order) also the flags after the
    clearhighlight / highlight dispatches of that substep.  `cell_fix`
    (ref_driver.cpp's pbfr_set_cell_fix): by default the end of the last
    occupied cell, which findcells never writes, is n, so that its run stays
    inside the particle buffer."""
    lib = ref_load()
    lib.pbfr_set_cell_fix(int(cell_fix))
    n = x4.shape[0]
    x = np.ascontiguousarray(x4, np.float32).copy()
    v = np.ascontiguousarray(v4, np.float32).copy()
    g = [int(a) for a in params.grid]
    cells = g[0] * g[1] * g[2]
    ids = np.empty(n, np.uint32)
    st = np.empty(cells, np.int32)
    en = np.empty(cells, np.int32)
    nbr = np.empty(12 * n, np.int32)
    lam = np.empty(n, np.float32)
    hl = None
    if highlight is not None:
        hl = np.ascontiguousarray(highlight, np.uint32).copy()
        assert hl.shape == (n,)
    lib.pbfr_substep_highlight(C.addressof(params), n, x.ctypes.data, v.ctypes.data,
                               ids.ctypes.data, st.ctypes.data, en.ctypes.data, nbr.ctypes.data,
                               lam.ctypes.data, None if hl is None else hl.ctypes.data)
    return {"highlight": hl, "x": x, "v": v, "ids": ids, "start": st.reshape(g[2], g[1], g[0]),
            "end": en.reshape(g[2], g[1], g[0]), "nbr": nbr.reshape(n, 3, 4), "lambda": lam}


def ref_splat(pass_: int, x4, viewmat, projmat, width: int, height: int):
    """SurfaceReconstruction's particle passes through the reference's own
    vertex/fragment shaders compiled as C++ (see ref_driver.cpp)."""
    lib = ref_load()
    x = np.ascontiguousarray(x4, np.float32)
    V = np.ascontiguousarray(viewmat, np.float32).reshape(16)
    P = np.ascontiguousarray(projmat, np.float32).reshape(16)
    out = np.empty((int(height), int(width)), np.float32)
    lib.pbfr_splat(int(pass_), x.ctypes.data, x.shape[0], V.ctypes.data, P.ctypes.data, int(width),
                   int(height), out.ctypes.data)
    return out

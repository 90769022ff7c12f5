"""CPU tests of the C ABI: the library loads, exports every entry point that
include/pbf.h declares, and its host-only functions behave."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from pbf_gb300 import _capi, scenes
from tests.conftest import HAS_GPU, ROOT


def declared_functions():
    names = []
    for path in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not path.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", path)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^[A-Za-z_][\w\s\*]*?\b(pbf_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_every_declared_symbol_is_exported(product_lib):
    names = declared_functions()
    assert len(names) >= 25
    for name in names:
        assert hasattr(product_lib, name), name
    # and the Python binding covers every declaration
    assert set(names) <= set(_capi.SIGNATURES), set(names) - set(_capi.SIGNATURES)


def test_abi_version_and_status_strings(product_lib):
    import re
    text = open(os.path.join(ROOT, "include", "pbf.h")).read()
    header = int(re.search(r"#define PBF_ABI_VERSION (\d+)", text).group(1))
    # a layout change of a struct crossing the ABI bumps the version: these
    # sizes belong to version 3
    assert header == 3
    assert C.sizeof(_capi.Tuning) == 36 and C.sizeof(_capi.Params) == 84
    assert product_lib.pbf_abi_version() == header
    assert product_lib.pbf_status_string(0) == b"ok"
    assert product_lib.pbf_status_string(1) == b"invalid argument"


def test_params_default_mirrors_reference(product_lib):
    p = _capi.Params()
    assert product_lib.pbf_params_default((C.c_uint32 * 3)(128, 64, 128), C.byref(p)) == 0
    # src/SPH.cpp:136-144 and src/SPH.cpp:25-26
    assert (p.one_over_rho_0, p.epsilon, p.gravity) == (1.0, 5.0, 10.0)
    assert p.timestep == np.float32(0.016)
    assert p.num_solver_iterations == 5 and p.vorticity_confinement == 0
    assert list(p.wall_lo) == [16.0, 0.0, 16.0] and list(p.wall_hi) == [112.0, 64.0, 112.0]
    assert product_lib.pbf_params_default((C.c_uint32 * 3)(0, 1, 1), C.byref(p)) == 1


def test_scene_generator_deterministic(product_lib):
    a = scenes.block((4, 3, 5), seed=11, vel_uniform=0.5, vel_sigma=0.25)
    b = scenes.block((4, 3, 5), seed=11, vel_uniform=0.5, vel_sigma=0.25)
    c = scenes.block((4, 3, 5), seed=12, vel_uniform=0.5, vel_sigma=0.25)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert not np.array_equal(a[0], c[0])
    x, v = a
    # id order: x outermost, then z, then y (src/Simulation.cpp:214-229)
    lat = x[:, :3].reshape(4, 5, 3, 3)
    assert np.all(np.abs(lat[1, 0, 0] - lat[0, 0, 0] - [0.5, 0, 0]) < 0.021)
    assert np.all(np.abs(lat[0, 1, 0] - lat[0, 0, 0] - [0, 0, 0.5]) < 0.021)
    assert np.all(np.abs(lat[0, 0, 1] - lat[0, 0, 0] - [0, 0.5, 0]) < 0.021)
    assert np.all(x[:, 3] == 0) and np.all(v[:, 3] == 0)


def test_scene_jitter_bounds(product_lib):
    x, v = scenes.block((8, 8, 8), seed=3)
    # loop order (i over x, k over z, j over y); coordinates (i, j, k)
    gi, gk, gj = np.meshgrid(np.arange(8), np.arange(8), np.arange(8), indexing="ij")
    ideal = 0.25 + 0.5 * np.stack([gi, gj, gk], -1).reshape(-1, 3)
    d = x[:, :3] - ideal.astype(np.float32)
    assert np.max(np.abs(d)) <= 0.01 + 1e-6
    assert np.all(v == 0)


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device path")
def test_create_without_device_fails_cleanly(product_lib):
    p = scenes.dam_params((16, 16, 16), 2)
    h = C.c_void_p()
    st = product_lib.pbf_create(C.byref(p), 100, C.byref(h))
    assert st == _capi.PBF_ERR_NO_DEVICE
    assert b"device" in product_lib.pbf_last_error(None)


def test_invalid_arguments_rejected_before_device(product_lib):
    h = C.c_void_p()
    assert product_lib.pbf_create(None, 10, C.byref(h)) == _capi.PBF_ERR_INVALID_ARGUMENT
    p = scenes.dam_params((16, 16, 16), 2)
    p.h = -1.0
    assert product_lib.pbf_create(C.byref(p), 10, C.byref(h)) == _capi.PBF_ERR_INVALID_ARGUMENT
    p = scenes.dam_params((16, 16, 16), 2)
    assert product_lib.pbf_create(C.byref(p), 0, C.byref(h)) == _capi.PBF_ERR_INVALID_ARGUMENT
    p.wall_lo[0] = 20.0
    assert product_lib.pbf_create(C.byref(p), 10, C.byref(h)) == _capi.PBF_ERR_INVALID_ARGUMENT
    assert product_lib.pbf_radix_sort(None, None, None, 5, 8, None) == _capi.PBF_ERR_INVALID_ARGUMENT


MIRRORS = {"pbf_params": "_capi.Params", "pbf_tuning": "_capi.Tuning",
           "pbf_param_grads": "_capi.ParamGrads", "pbf_diagnostics": "_capi.Diagnostics",
           "pbf_view": "splat.View"}


def test_struct_mirrors_match_header(tmp_path):
    """Every ctypes mirror of an include/pbf.h struct has the header's size
    and the same field offsets (a C probe compiled against the header prints
    them)."""
    import shutil
    import subprocess
    from pbf_gb300 import splat
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mods = {"_capi": _capi, "splat": splat}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "pbf.h"', "int main(void) {"]
    for cname, py in MIRRORS.items():
        mod, cls = py.split(".")
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for field, _ in getattr(mods[mod], cls)._fields_:
            lines.append(f'printf("{cname} {field} %zu\\n", offsetof({cname}, {field}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True,
                               text=True).stdout.splitlines():
        cname, key, val = line.split()
        got[(cname, key)] = int(val)
    for cname, py in MIRRORS.items():
        mod, cls = py.split(".")
        st = getattr(mods[mod], cls)
        assert C.sizeof(st) == got[(cname, "size")], f"{py} size"
        for field, _ in st._fields_:
            assert getattr(st, field).offset == got[(cname, field)], f"{py}.{field} offset"


def test_header_constants_match_python():
    """Every PBF_* constant include/pbf.h defines (macros and enumerators)
    has the same value in the Python binding, which mirrors all of them
    (pbf_gb300._capi; the splat pass numbers in pbf_gb300.splat)."""
    import re
    from pbf_gb300 import splat
    text = open(os.path.join(ROOT, "include", "pbf.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    consts = {}
    for name, val in re.findall(r"^#define (PBF_\w+) (0x[0-9a-fA-F]+|\d+)u?\s*$", text, flags=re.M):
        consts[name] = int(val, 0)
    for body in re.findall(r"enum\s*\w*\s*\{(.*?)\}", text, flags=re.S):
        for name, val in re.findall(r"(PBF_\w+)\s*=\s*(\d+)", body):
            consts[name] = int(val)
    consts.pop("PBF_ABI_VERSION", None)  # checked by test_abi_version_and_status_strings
    assert len(consts) >= 20
    alias = {"PBF_SPLAT_DEPTH": (splat, "DEPTH"), "PBF_SPLAT_THICKNESS": (splat, "THICKNESS")}
    for name, val in consts.items():
        mod, attr = alias.get(name, (_capi, name))
        assert hasattr(mod, attr), f"{name} is not mirrored in Python"
        assert getattr(mod, attr) == val, f"{name}: header {val}, Python {getattr(mod, attr)}"

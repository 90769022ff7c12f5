"""In-tree build of the CUDA library ``pbf_gb300/_build/libpbf_gb300.so``.

Every ``.cu`` file under ``pbf_gb300/csrc`` is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), host C++ with g++, all
translation units in parallel, then linked with nvcc into one shared library
with the CUDA runtime linked statically.  Objects are rebuilt only when a
source or header is newer.  ``-fmad=false`` and ``-ffp-contract=off`` keep the
compilers from fusing multiply-adds the source does not spell out: the
physics kernels' rounding sequence is part of their contract.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpbf_gb300.so")
# the bounds-checked variant (-DPBF_CHECK): index checks latch PBF_DEV_INDEX
CHECK_BUILD = os.path.join(HERE, "_build_check")
CHECK_LIB = os.path.join(CHECK_BUILD, "libpbf_gb300_check.so")
ROOT = os.path.dirname(HERE)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
    "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pbf_gb300")


def _deps() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + [os.path.join(ROOT, "include", "pbf.h")])


def _stale(out: str, srcs: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs if os.path.exists(s))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None, check: bool = False) -> str:
    """Compiles and links the library if anything changed; returns its path.
    check=True builds the bounds-checked variant (-DPBF_CHECK) instead, into
    its own directory."""
    out_dir, lib_path = (CHECK_BUILD, CHECK_LIB) if check else (BUILD, LIB)
    defs = ["-DPBF_CHECK"] if check else []
    os.makedirs(out_dir, exist_ok=True)
    nvcc = _nvcc()
    deps = _deps()
    jobs_list = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(out_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + deps):
            jobs_list.append([nvcc] + NVCC_FLAGS + defs + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(out_dir, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + deps):
            jobs_list.append([os.environ.get("CXX", "g++")] + CXX_FLAGS + defs +
                             ["-c", src, "-o", obj])
    if jobs_list:
        with ThreadPoolExecutor(max_workers=jobs or min(8, len(jobs_list))) as ex:
            for cmd, _ in zip(jobs_list, ex.map(_run, jobs_list)):
                if verbose:
                    print(" ".join(cmd))
    if jobs_list or _stale(lib_path, objs):
        tmp = lib_path + ".tmp"
        _run([nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs)
        os.replace(tmp, lib_path)
        if verbose:
            print("linked", lib_path)
    return lib_path


if __name__ == "__main__":
    import sys
    print(build(verbose=True, check="--check" in sys.argv))

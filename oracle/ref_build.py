"""Recipe: compile the reference's own substep compute shaders as C++ on the
CPU (TEST INFRASTRUCTURE ONLY), to pin the oracle against the reference's
code instead of a restatement of it.

The shader files are read where they lie in the reference checkout (default
/root/reference, or $PBF_REFERENCE); nothing of them is copied into the
repository.  Only their GLSL interface declarations are rewritten --
`layout(local_size_x...) in;`, buffer blocks, uniform samplers and images,
and `main` -- into plain declarations the driver binds; every function body,
constant and expression is compiled as written, with oracle/ref_shim/glsl.hpp
supplying the GLSL types and built-ins, `-fsingle-precision-constant` keeping
GLSL float literals float and `-ffp-contract=off` one rounding per operation.
The generated file and the library go to oracle/_ref/ (git-ignored).

Shaders used (SPH::Run, src/SPH.cpp:246-334): sph/predictpos, sph/calclambda,
sph/updatepos, sph/update, sph/vorticity, sph/clearhighlight, sph/highlight
(each prefixed with
sph/foreachneighbour, as SPH's constructor compiles them, src/SPH.cpp:63-90),
neighbourcellfinder/findcells and neighbourcells, and GetHash from
radixsort/counting.  The radix sort's counting / blockscan / addblocksum /
globalsort kernels are not run (their workgroup barriers have no sequential
equivalent); the driver sorts by GetHash with a stable sort over the same
bits, which is what those kernels compute (src/RadixSort.cpp:124-133).
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libpbf_ref.so")
SHIM = os.path.join(HERE, "ref_shim")

SPH_SHADERS = ["predictpos", "calclambda", "updatepos", "update", "vorticity", "clearhighlight",
               "highlight"]
NCF_SHADERS = ["findcells", "neighbourcells"]


def reference_root() -> str:
    return os.environ.get("PBF_REFERENCE", "/root/reference")


def available() -> bool:
    return os.path.isdir(os.path.join(reference_root(), "shaders", "sph"))


def _read(rel: str) -> str:
    with open(os.path.join(reference_root(), "shaders", rel)) as f:
        return f.read()


BUFFER = re.compile(
    r"layout\s*\([^)]*\)\s*((?:readonly|writeonly|coherent)\s+)*buffer\s+\w+\s*"
    r"\{\s*(\w+)\s+(\w+)\s*\[\s*\]\s*;\s*\}\s*;")
UNIFORM = re.compile(r"layout\s*\([^)]*\)\s*uniform\s+((?:readonly|writeonly)\s+)*(\w+)\s+(\w+)\s*;")
LOCAL = re.compile(r"layout\s*\(\s*local_size_x[^)]*\)\s*in\s*;")
MAIN = re.compile(r"void\s+main\s*\(\s*void\s*\)")


def translate(src: str) -> str:
    """Rewrites the interface declarations; leaves every body untouched."""
    src = LOCAL.sub("", src)
    src = BUFFER.sub(lambda m: f"static {m.group(2)}* {m.group(3)} = nullptr;", src)
    src = UNIFORM.sub(lambda m: f"static {m.group(2)} {m.group(3)};", src)
    src = MAIN.sub("void main_invocation()", src)
    return src


def get_hash_function() -> str:
    """GetHash of shaders/radixsort/counting.glsl:53-57, parameter qualifier dropped."""
    src = _read("radixsort/counting.glsl")
    m = re.search(r"uint\s+GetHash\s*\(\s*in\s+vec3\s+pos\s*\)\s*\{.*?\n\}", src, re.S)
    if not m:
        raise RuntimeError("GetHash not found in counting.glsl")
    return re.sub(r"\(\s*in\s+vec3", "(vec3", m.group(0))


def generate() -> str:
    fe = _read("sph/foreachneighbour.glsl")
    parts = ["// generated by oracle/ref_build.py from the reference's shader files\n"]
    for name in SPH_SHADERS:
        body = translate(fe + "\n" + _read(f"sph/{name}.glsl"))
        parts.append(f"namespace sh_{name} {{\nusing namespace glsl;\nusing namespace refglobals;\n"
                     f"{body}\n}}  // namespace sh_{name}\n")
    for name in NCF_SHADERS:
        body = translate(_read(f"neighbourcellfinder/{name}.glsl"))
        parts.append(f"namespace sh_{name} {{\nusing namespace glsl;\nusing namespace refglobals;\n"
                     f"{body}\n}}  // namespace sh_{name}\n")
    parts.append("namespace sh_hash {\nusing namespace glsl;\nusing namespace refglobals;\n"
                 + get_hash_function() + "\n}  // namespace sh_hash\n")
    return "\n".join(parts)


def build(force: bool = False) -> str | None:
    """Generates and compiles oracle/_ref/libpbf_ref.so; None when the
    reference checkout is absent (the library then cannot exist)."""
    if not available():
        return LIB if os.path.exists(LIB) else None
    os.makedirs(OUT, exist_ok=True)
    gen = os.path.join(OUT, "gen_shaders.inc")
    text = generate()
    if force or not os.path.exists(gen) or open(gen).read() != text:
        with open(gen, "w") as f:
            f.write(text)
    srcs = [gen, os.path.join(SHIM, "glsl.hpp"), os.path.join(SHIM, "ref_driver.cpp")]
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s)
                                                  for s in srcs):
        return LIB
    tmp = LIB + ".tmp"
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-fPIC", "-shared",
           "-ffp-contract=off", "-fsingle-precision-constant", "-w", "-I", OUT, "-I", SHIM,
           "-o", tmp, os.path.join(SHIM, "ref_driver.cpp")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference shader build failed:\n" + " ".join(cmd) + "\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

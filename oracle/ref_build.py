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
radixsort/counting; for SurfaceReconstruction's particle passes,
particledepth/vertex + fragment and thickness/vertex.  The radix sort's counting / blockscan / addblocksum /
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


STAGE_IN = re.compile(r"layout\s*\([^)]*\)\s*in\s+(\w+)\s+(\w+)\s*;")
STAGE_IO = re.compile(r"^[ \t]*(?:flat[ \t]+)?(?:in|out)[ \t]+(\w+)[ \t]+(\w+)[ \t]*;", re.M)
BLOCK = re.compile(r"layout\s*\([^)]*\)\s*uniform\s+\w+\s*\{([^}]*)\}\s*;")
DISCARD = re.compile(r"\bdiscard\s*;")


def translate_stage(src: str) -> str:
    """Rewrites a vertex or fragment shader's interface declarations (vertex
    inputs, stage inputs/outputs, the uniform block) into plain variables the
    driver sets and reads, and `discard;` into a flagged return; every body
    stays as written."""
    src = STAGE_IN.sub(lambda m: f"static {m.group(1)} {m.group(2)};", src)
    src = BLOCK.sub(lambda m: " ".join(f"static {d.strip()};" for d in m.group(1).split(";")
                                       if d.strip()), src)
    src = STAGE_IO.sub(lambda m: f"static {m.group(1)} {m.group(2)};", src)
    src = DISCARD.sub("{ discarded = true; return; }", src)
    src = MAIN.sub("void main_invocation()", src)
    return src


# SurfaceReconstruction's particle passes (src/SurfaceReconstruction.cpp:
# 176-231): the depth pass's two stages and the thickness pass's vertex stage
# (its fragment stage, with noise off, only discards outside the unit disc
# and writes 1; the driver restates that).
STAGE_SHADERS = [("particledepth_vs", "particledepth/vertex.glsl"),
                 ("particledepth_fs", "particledepth/fragment.glsl"),
                 ("thickness_vs", "thickness/vertex.glsl")]


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
    for ns, rel in STAGE_SHADERS:
        body = translate_stage(_read(rel))
        parts.append(f"namespace sh_{ns} {{\nusing namespace glsl;\nstatic vec4 gl_Position;\n"
                     f"static float gl_FragDepth;\nstatic int gl_InstanceID;\n"
                     f"static bool discarded;\n{body}\n}}  // namespace sh_{ns}\n")
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

"""Generates tests/golden/ref_splat.npz: the depth and thickness images of
the reference's own particledepth / thickness shaders (compiled as C++ from
the reference checkout by oracle/ref_build.py) for the cases in
splat_cases.py.  Run here, where the checkout exists:

    python tests/golden/make_splat_golden.py
"""
import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, HERE)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
import splat_cases  # noqa: E402


def main():
    arrays = {}
    for name in splat_cases.CASES:
        x4, V, P, dsz, tsz = splat_cases.make(name)
        Vc, Pc = splat_cases.columns(V), splat_cases.columns(P)
        arrays[f"{name}_depth"] = oracle.ref_splat(0, x4, Vc, Pc, *dsz)
        arrays[f"{name}_thickness"] = oracle.ref_splat(1, x4, Vc, Pc, *tsz)
    path = os.path.join(HERE, "ref_splat.npz")
    np.savez_compressed(path, **arrays)
    digest = hashlib.sha256(open(path, "rb").read()).hexdigest()
    man = os.path.join(HERE, "manifest.json")
    m = json.load(open(man))
    m.setdefault("splat", {})["ref_splat.npz"] = digest
    m["splat_generator"] = "tests/golden/make_splat_golden.py"
    json.dump(m, open(man, "w"), indent=1)
    print(path, digest)


if __name__ == "__main__":
    main()

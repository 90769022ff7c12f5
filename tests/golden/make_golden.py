"""Generates the golden fixtures: outputs of the reference's own compute
shaders (compiled as C++ from the reference checkout by oracle/ref_build.py)
for one substep of each scene in pin_scenes.py (with the end of the last
occupied cell written, see ref_driver.cpp's pbfr_set_cell_fix; the scenes'
dummy particles keep both boundary cells away from the fluid).  Run here, where the
reference checkout exists; the fixtures then travel to machines that lack it.

    python tests/golden/make_golden.py
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
import pin_scenes  # noqa: E402


def main():
    mpath = os.path.join(HERE, "manifest.json")
    # other generators' entries (make_multistep.py, make_splat_golden.py) are kept
    doc = json.load(open(mpath)) if os.path.exists(mpath) else {}
    manifest = {k: v for k, v in doc.get("sha256", {}).items()
                if k[4:-4] not in pin_scenes.CASES and os.path.exists(os.path.join(HERE, k))}
    for name in pin_scenes.CASES:
        p, x4, v4 = pin_scenes.make(name)
        hl_in = pin_scenes.highlight_flags(x4.shape[0])
        # the last cell's end, which findcells never writes, is n (cell_fix=2):
        # a fresh texture would give the last-cell dummy a negative run count
        r = oracle.ref_substep(p, x4, v4, highlight=hl_in, cell_fix=2)
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, x_in=x4, v_in=v4, x=r["x"], v=r["v"], ids=r["ids"],
                            lam=r["lambda"], hl_in=hl_in, hl=r["highlight"])
        manifest[os.path.basename(path)] = hashlib.sha256(open(path, "rb").read()).hexdigest()
    doc["generator"] = "tests/golden/make_golden.py, tests/golden/make_multistep.py"
    doc["source"] = "reference shaders compiled by oracle/ref_build.py"
    doc["sha256"] = dict(sorted(manifest.items()))
    with open(mpath, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps(manifest, indent=1))


if __name__ == "__main__":
    main()

"""Generates tests/golden/ref_multistep.npz: statistics of a multi-substep
run of the reference's own compute shaders (compiled as C++ by
oracle/ref_build.py; needs the reference checkout), for
tests/test_ref_pin.py::test_multistep_statistics_follow_the_reference.

Scene (a config-0-like dam break inside the reference's hard-coded walls):
the 32x16x32 lattice of spacing 0.5h (16,384 particles, seeded jitter
U(-0.01h, 0.01h), zero velocities) in the corner (16.25, 0.25, 16.25) of a
65^3-cell grid whose walls are the reference's (16, 0, 16) .. GRID_SIZE -
(16, 0, 16) (shaders/sph/updatepos.glsl:98-100); h = 1, epsilon = 0.01,
3 iterations, dt = 0.008, XSPH and vorticity on; SUBSTEPS substeps of
SPH::Run (src/SPH.cpp:246-334).

Per substep it records, from the reference library's state: the kinetic
energy, the mean and largest density error |rho/rho_0 - 1| (measured by the
oracle's diagnostics on that state, full neighbour runs) and the number of
particles whose packed neighbour texture held a run of 128 or more (the
count wraps in 8 bits and FOR_EACH_NEIGHBOUR drops the run,
shaders/sph/foreachneighbour.glsl:5-6).

Run from the repository root:  python tests/golden/make_multistep.py
"""
import ctypes as C
import hashlib
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from oracle import scenes as osc  # noqa: E402

GRID = 65
SUBSTEPS = 80


def scene():
    p = osc.dam_params((GRID - 1,) * 3, 3)
    for a, w in enumerate((16.0, 0.0, 16.0)):
        p.wall_lo[a] = w
        p.wall_hi[a] = GRID - w
    x4, v4 = osc.block((32, 16, 32), origin=(16.25, 0.25, 16.25), seed=0)
    return p, x4, v4


def stats(p, x4, v4):
    o = oracle.Oracle(p, x4.shape[0])
    o.set_state(x4, v4)
    d = o.diagnostics()
    o.close()
    return d["kinetic_energy"], d["mean_density_error"], d["max_density_error"]


def main():
    lib = oracle.ref_load()
    lib.pbfr_set_cell_fix(0)  # the reference exactly as written
    p, x4, v4 = scene()
    n = x4.shape[0]
    x, v = x4.copy(), v4.copy()
    nbr = np.empty(12 * n, np.int32)
    ke, mean_err, max_err, dropped, secs = [], [], [], [], []
    for s in range(SUBSTEPS):
        t = time.time()
        lib.pbfr_substep_highlight(C.addressof(p), n, x.ctypes.data, v.ctypes.data, None, None, None,
                                   nbr.ctypes.data, None, None)
        secs.append(time.time() - t)
        k, me, mx = stats(p, x, v)
        packed = nbr.reshape(n, 3, 4)[:, :, :3].reshape(n, 9)  # 3 ivec4 per particle, xyz used
        # start + (count << 24): a count of 128 or more reads negative (-1 marks an empty row)
        dropped.append(int(np.sum(np.any((packed != -1) & ((packed >> 24) < 0), axis=1))))
        ke.append(k)
        mean_err.append(me)
        max_err.append(mx)
        print(f"substep {s + 1}: KE {k:.4g}, density error mean {me:.3g} max {mx:.3g}, "
              f"particles with a dropped run {dropped[-1]}, {secs[-1]:.1f} s", flush=True)
    path = os.path.join(HERE, "ref_multistep.npz")
    np.savez_compressed(path, ke=np.array(ke), mean_err=np.array(mean_err),
                        max_err=np.array(max_err), dropped=np.array(dropped, np.int64))
    mpath = os.path.join(HERE, "manifest.json")
    m = json.load(open(mpath))
    m["sha256"]["ref_multistep.npz"] = hashlib.sha256(open(path, "rb").read()).hexdigest()
    m["sha256"] = dict(sorted(m["sha256"].items()))
    with open(mpath, "w") as f:
        json.dump(m, f, indent=1)


if __name__ == "__main__":
    main()

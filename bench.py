#!/usr/bin/env python
"""Benchmark of the PBF substep path: particle-solver-iterations per second
on the 2,097,152-particle dam break (128^3 lattice, spacing 0.5h, in a
256x128x256 box, 4 solver iterations, dt = 0.008) on one GB300.

A "step" is one substep (SPH::Run) over all particles.  The timed window is
substeps 1..K of the run (default K = 50): with the workload's constants
(epsilon = 0.01, the reference's unclamped density constraint and stencil
centre) the dam break blows up within the first 20 substeps and then
collapses into clumps of thousands of particles per cell, a different and
degenerate workload; `stable_500`
reports the same scene with the reference's default CFM epsilon (5) over
the full 500 substeps.  Timed regions:
  value    K substeps replayed from the captured CUDA graph, inputs resident
           in HBM, bracketed by CUDA events on the simulation's stream;
  e2e      K steps through the public C ABI with host buffers: every step
           uploads the state from pinned host memory (pbf_set_state), runs
           one substep (pbf_step) and reads the state back (pbf_get_state);
  kernels  the same K substeps replayed eagerly with CUDA events around
           every kernel, for the per-launch durations behind `roofline`.
Each timed run starts from the initial scene, after W warm-up substeps;
the e2e steps continue one trajectory (each uploads the state the step
before it read back).
The per-substep working set (~0.5 GB) is larger than L2, so L2 is not
flushed between steps.

--impl reference times the reference path on the host cores instead: the
oracle (a C++ restatement of pbf's GLSL compute shaders, OpenMP; the
reference itself needs an OpenGL 4.3 context, which these machines lack),
W warm-up substeps, then the same window (substeps 1..K from the initial
scene), every substep in full, as many whole substeps as fit in about four
minutes.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-solver-iterations/s"
UNIT = "particle-iters/s"
# Compulsory HBM bytes per particle of one launch (x* 16 B + lambda 4 B read
# or written once each): lambda reads x*, writes lambda; delta-p reads x* and
# lambda, writes x*.
ALG_BYTES = {"lambda": 20, "delta_p": 36}
KERNEL_NAMES = {"lambda": "k_lambda_build + k_lambda", "delta_p": "k_delta_p"}


def parse():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scene", default="plain_2m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-substeps", type=int, default=20,
                    help="full substeps of the CPU baseline sample")
    ap.add_argument("--e2e-steps", type=int, default=0, help="0: min(steps, 50)")
    ap.add_argument("--no-stable", action="store_true", help="skip the epsilon = 5 full run")
    ap.add_argument("--no-full", action="store_true",
                    help="skip the full 500-substep run of the workload itself")
    ap.add_argument("--no-batched", action="store_true", help="skip the 256-scene comparison")
    ap.add_argument("--plain-every", type=int, default=8,
                    help="step every k-th of the 256 scenes plainly for the comparison (1: all)")
    ap.add_argument("--full-budget", type=float, default=90.0,
                    help="seconds of the workload's own 500-substep run; it stops after the "
                         "25-substep segment that crosses the budget (0: run all 500)")
    ap.add_argument("--recovery-steps-eps001", type=int, default=5,
                    help="gradient-descent steps of the recovery at the workload's epsilon "
                         "(its gradients are not finite; 50 at epsilon = 5)")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the backward/forward ratio")
    ap.add_argument("--no-splat", action="store_true", help="skip the depth/thickness splatting leg")
    ap.add_argument("--no-small", action="store_true", help="skip the 16,384-particle configuration")
    ap.add_argument("--autotune", action="store_true",
                    help="fix the tuning pbf_autotune picks instead of the automatic sweep "
                         "configuration")
    ap.add_argument("--no-autotune", action="store_true",
                    help="the default (kept for older command lines)")
    ap.add_argument("--recovery", action="store_true",
                    help="the default (kept for older command lines)")
    ap.add_argument("--no-recovery", action="store_true",
                    help="skip the 64-scene parameter recovery (about a minute)")
    ap.add_argument("--substep-stages", type=int, default=0,
                    help="instead of the benchmark: one JSON line per substep 1..N of the "
                         "workload with its stage times (eager, CUDA events per stage)")
    return ap.parse_args()


def substep_stages(scene, count: int) -> None:
    """Stage milliseconds of each of the first `count` substeps of the
    workload (after W = 5 warm-up substeps and a reset), from the stage
    events of the eager timing mode (pbf_enable_timing), one JSON line each."""
    import pbf_gb300 as pg
    sim = pg.SPH(scene.n, tuple(scene.params.grid), scene.params)
    sim.set_state(scene.x4, scene.v4)
    sim.step(5)
    sim.synchronize()
    sim.set_state(scene.x4, scene.v4)
    sim.EnableTiming(True)
    prev = {k: 0.0 for k in pg.SPH.STAGES}
    for k in range(1, count + 1):
        sim.step(1)
        st, _ = sim.stage_times()
        d = {a: round(st[a] - prev[a], 3) for a in st}
        prev = st
        print(json.dumps({"substep": k, "total_ms": round(sum(d.values()), 3), **d,
                          "solver_sweeps": sim.sweep_choice()["solver"]}), flush=True)
    sim.close()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.fh,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sms.append(float(parts[1]))
                maxs.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sms.sort()
        return {"sm_mhz": sms[len(sms) // 2], "sm_max_mhz": max(maxs), "samples": len(sms),
                "reasons": sorted(reasons)}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic():
    """DRAM bytes per particle of the dominant kernels from the committed ncu
    summary (profiles/ncu_traffic.json), or None."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


def batched_vs_plain(stream, num_scenes: int = 256, substeps: int = 100, plain_every: int = 8):
    """256 dam breaks (4,096-65,536 particles, boxes 32-96 cells, 4 iterations,
    100 substeps): one batched handle (every stage one launch over all scenes,
    the substep replayed as one CUDA graph) against the scenes stepped one at a
    time, each in its own handle with its own graph, on the same stream.  Both
    start from the initial scenes after 3 warm-up substeps.  With epsilon =
    0.01 the scenes collapse and stepping all 256 plainly takes ~10 minutes,
    so by default every `plain_every`-th scene (32 of 256) is stepped plainly
    and the plain time of all 256 is that sample's time x 256 / 32
    (plain_every = 1: all of them)."""
    import torch
    import numpy as np
    import pbf_gb300 as pg
    from pbf_gb300 import scenes
    scs = scenes.batch_scenes(num_scenes, substeps=substeps)
    x4, v4 = scenes.concat_state(scs)
    batch = pg.SPHBatch([s.params for s in scs], [s.n for s in scs])
    batch.set_stream(stream.cuda_stream)
    batch.set_state(x4, v4)
    batch.step(3)
    batch.set_state(x4, v4)
    sample = list(range(0, num_scenes, plain_every))
    plain = []
    for k in sample:
        s = scs[k]
        h = pg.SPH(s.n, tuple(s.params.grid), s.params)
        h.set_stream(stream.cuda_stream)
        h.set_state(s.x4, s.v4)
        h.step(3)
        h.set_state(s.x4, s.v4)
        plain.append(h)
    torch.cuda.synchronize()
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    e[0].record(stream)
    batch.step(substeps)
    e[1].record(stream)
    torch.cuda.synchronize()
    e[2].record(stream)
    for h in plain:
        h.step(substeps)
    e[3].record(stream)
    torch.cuda.synchronize()
    tb = e[0].elapsed_time(e[1])
    tps = e[2].elapsed_time(e[3])
    tp = tps * num_scenes / len(sample)
    bx, bv = batch.get_state()
    same = True
    for h, k in zip(plain, sample):
        px, pv = h.get_state()
        sl = batch.scene_slice(k)
        same = same and np.array_equal(bx[sl].view(np.uint32), px.view(np.uint32)) and \
            np.array_equal(bv[sl].view(np.uint32), pv.view(np.uint32))
    n = int(x4.shape[0])
    it = scs[0].params.num_solver_iterations
    for h in plain:
        h.close()
    batch.close()
    return {"scenes": num_scenes, "particles": n, "substeps": substeps,
            "batched_ms": tb, "plain_ms": tp, "plain_sampled_scenes": len(sample),
            "plain_sampled_ms": tps,
            "batched_scenes_per_s": num_scenes / (tb * 1e-3),
            "plain_scenes_per_s": num_scenes / (tp * 1e-3), "speedup": tp / tb,
            "batched_particle_iters_per_s": n * it * substeps / (tb * 1e-3),
            "bit_identical_sampled_scenes": bool(same),
            "note": ("plain time of all 256 scenes estimated from every "
                     f"{plain_every}th scene stepped plainly" if plain_every > 1 else
                     "every scene stepped plainly")}


def batched_sharded(stream, rank: int, world: int, barrier, num_scenes: int = 256,
                    substeps: int = 100):
    """The 256-scene batch split across ranks by scene (scenes.shard_batch):
    one batched handle per rank over its scenes, no collective on the data
    path; the timed region (barrier and synchronise on both sides) is the
    slowest rank's.  Whole-job scenes/s = num_scenes / that time."""
    import torch
    import torch.distributed as dist
    import pbf_gb300 as pg
    from pbf_gb300 import scenes
    scs = scenes.batch_scenes(num_scenes, substeps=substeps)
    mine, params, counts, x4, v4 = scenes.shard_batch(scs, rank, world)
    b = pg.SPHBatch(params, counts) if mine else None
    if b is not None:
        b.set_stream(stream.cuda_stream)
        b.set_state(x4, v4)
        b.step(3)
        b.set_state(x4, v4)
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    if b is not None:
        b.step(substeps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    t = torch.tensor([e0.elapsed_time(e1)], device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    n_local = torch.tensor([float(x4.shape[0])], device="cuda")
    if world > 1:
        dist.all_reduce(n_local)
    it = scs[0].params.num_solver_iterations
    if b is not None:
        b.close()
    return {"scenes": num_scenes, "ranks": world, "scenes_on_rank0": len(mine) if rank == 0 else None,
            "substeps": substeps, "ms": ms, "scenes_per_s": num_scenes / (ms * 1e-3),
            "particle_iters_per_s": float(n_local.item()) * it * substeps / (ms * 1e-3),
            "note": "scenes sharded by particle count (largest first); each rank one batched "
                    "handle, no data-path collective; time = max over ranks"}


def splat_leg(stream, reps: int = 20):
    """SurfaceReconstruction's particle passes (pbf_splat) on the reference's
    own scene (65,536 particles, after 20 substeps) and camera, at the
    reference's framebuffer sizes: depth 1280 x 720, thickness 512 x 512.
    CUDA events around `reps` calls each (each call clears its image and
    synchronises)."""
    import torch
    import pbf_gb300 as pg
    from pbf_gb300 import scenes, splat
    s = scenes.reference_two_blocks(seed=0)
    sim = pg.SPH(s.n, tuple(s.params.grid), s.params)
    sim.set_stream(stream.cuda_stream)
    sim.set_state(s.x4, s.v4)
    sim.step(20)
    sim.synchronize()
    view = splat.reference_view(1280, 720)
    res = {"particles": s.n, "reps": reps}
    for name, p, (w, h) in (("depth", splat.DEPTH, (1280, 720)),
                            ("thickness", splat.THICKNESS, (512, 512))):
        out = torch.empty((h, w), dtype=torch.float32, device="cuda")
        for _ in range(3):
            splat.splat_device(p, sim.GetPositionBuffer(), s.n, view, w, h, out.data_ptr(),
                               stream.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            splat.splat_device(p, sim.GetPositionBuffer(), s.n, view, w, h, out.data_ptr(),
                               stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res[f"{name}_ms"] = ms
        res[f"{name}_size"] = [w, h]
        res[f"{name}_covered_pixels"] = int(((out < 1) if p == splat.DEPTH else (out > 0)).sum().item())
    res["particles_per_s_depth"] = s.n / (res["depth_ms"] * 1e-3)
    res["note"] = "each call includes its image clear and a stream synchronisation"
    sim.close()
    return res


def adjoint_ratio(stream, substeps: int = 64, every: int = 8, epsilon=None):
    """Backward / forward time of the differentiable scene: 32,768 particles
    (32^3 lattice) in a 64^3 box, velocities N(0, 0.25^2) from seed A, 64
    substeps x 4 iterations; loss = mean squared distance of the final
    positions to those of a run from seed-B velocities.  Forward = the
    recorded run (checkpoint every 8 substeps); backward = recomputing each
    8-substep segment with its tape plus the adjoint kernels.  `epsilon`
    replaces the CFM epsilon of both runs (None: the workload's 0.01)."""
    import torch
    import numpy as np
    import pbf_gb300 as pg
    from pbf_gb300 import scenes
    a, b = scenes.diff_32k()
    if epsilon is not None:
        a.params.epsilon = epsilon
        b.params.epsilon = epsilon
    n = a.n
    tgt = pg.SPH(n, tuple(b.params.grid), b.params)
    tgt.set_state(b.x4, b.v4)
    tgt.step(substeps)
    target = tgt.positions()
    tgt.close()
    sim = pg.SPH(n, tuple(a.params.grid), a.params)
    sim.set_stream(stream.cuda_stream)
    sim.set_state(a.x4, a.v4)
    sim.forward_record(substeps, every)  # warm-up (graph capture, tape allocation)
    x = sim.positions()
    w = (2.0 / n) * (x - target)
    w[:, 3] = 0
    sim.backward(w, None)
    fwd, bwd = [], []
    for _ in range(3):
        sim.set_state(a.x4, a.v4)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sim.forward_record(substeps, every)
        sim.synchronize()
        t1 = time.perf_counter()
        x = sim.positions()
        w = (2.0 / n) * (x - target)
        w[:, 3] = 0
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        dx0, dv0, g = sim.backward(w, None)
        t3 = time.perf_counter()
        fwd.append(t1 - t0)
        bwd.append(t3 - t2)
    loss = float(np.mean(np.sum((x[:, :3] - target[:, :3]) ** 2, axis=1)))
    f, bk = min(fwd), min(bwd)
    sim.close()
    return {"particles": n, "substeps": substeps, "iterations": a.params.num_solver_iterations,
            "checkpoint_every": every, "forward_ms": f * 1e3, "backward_ms": bk * 1e3,
            "bwd_fwd_ratio": bk / f, "loss": loss,
            "grad_norm_v0": float(np.linalg.norm(dv0[:, :3])),
            "grad_finite": bool(np.all(np.isfinite(dv0))),
            "grad_params": dict(zip(pg.SPH.PARAM_NAMES, [float(v) for v in g[0]])),
            "epsilon": float(a.params.epsilon),
            "note": "wall-clock per call, host synchronised; backward includes the "
                    "recomputation of every checkpoint segment" +
                    ("" if epsilon is not None else
                     "; with epsilon = 0.01 the 64-substep derivative overflows FP32 (the "
                     "run blows up: see adjoint_32k_epsilon_5 for finite gradients)")}


def recovery(stream, num_scenes: int = 64, substeps: int = 32, steps: int = 50, seed: int = 11,
             epsilon: float = 0.01):
    """Batched differentiable parameter recovery: 64 scenes (8,192-32,768
    particles, boxes 48-80 cells, 32 substeps x 4 iterations).  Hidden per-scene
    XSPH c ~ U(0.005, 0.02) and vorticity epsilon ~ U(0, 0.001) generate the
    target final positions; starting from c = 0.01, epsilon = 0.0005, `steps`
    Adam steps on the per-scene mean squared distance, each one batched
    forward_record + backward (checkpoint every 8 substeps)."""
    import numpy as np
    import pbf_gb300 as pg
    from pbf_gb300 import scenes
    rng = np.random.default_rng(seed)
    scs = scenes.batch_scenes(num_scenes, seed=seed, iterations=4, substeps=substeps, nmin=8192,
                              nmax=32768, box_min=48, box_max=80)
    for s_ in scs:
        s_.params.epsilon = epsilon
    hidden = np.stack([rng.uniform(0.005, 0.02, num_scenes), rng.uniform(0.0, 0.001, num_scenes)], 1)
    x4, v4 = scenes.concat_state(scs)
    batch = pg.SPHBatch([s.params for s in scs], [s.n for s in scs])
    batch.set_stream(stream.cuda_stream)

    def set_theta(th):
        for k in range(num_scenes):
            p = batch.scene_params(k)
            p.xsph_viscosity_c = float(np.float32(th[k, 0]))
            p.vorticity_epsilon = float(np.float32(th[k, 1]))
            batch.set_scene_params(k, p)

    set_theta(hidden)
    batch.set_state(x4, v4)
    batch.step(substeps)
    target = batch.positions()
    theta = np.tile([0.01, 0.0005], (num_scenes, 1))
    scale = np.array([0.015, 0.001])
    m = np.zeros_like(theta)
    vv = np.zeros_like(theta)
    lr, b1, b2 = 0.05, 0.9, 0.999
    counts = np.array([s.n for s in scs], np.float64)
    sl = [batch.scene_slice(k) for k in range(num_scenes)]
    times, losses = [], []
    nonfinite = 0
    for it in range(steps):
        t0 = time.perf_counter()
        set_theta(theta)
        batch.set_state(x4, v4)
        batch.forward_record(substeps, 8)
        x = batch.positions()
        w = np.zeros_like(x)
        loss = np.zeros(num_scenes)
        for k in range(num_scenes):
            d = x[sl[k], :3] - target[sl[k], :3]
            loss[k] = float(np.mean(np.sum(d * d, axis=1)))
            w[sl[k], :3] = (2.0 / counts[k]) * d
        _, _, g = batch.backward(w, None)
        times.append(time.perf_counter() - t0)
        losses.append(float(loss.mean()))
        grad = g[:, [2, 3]] * scale  # d loss / d (theta / scale)
        bad = ~np.all(np.isfinite(grad), axis=1)
        nonfinite += int(bad.sum())
        grad[bad] = 0.0
        m = b1 * m + (1 - b1) * grad
        vv = b2 * vv + (1 - b2) * grad * grad
        mh = m / (1 - b1 ** (it + 1))
        vh = vv / (1 - b2 ** (it + 1))
        step = lr * mh / (np.sqrt(vh) + 1e-30)
        theta = np.clip(theta - step * scale, [0.0, 0.0], [0.05, 0.005])
    err0 = np.abs(np.tile([0.01, 0.0005], (num_scenes, 1)) - hidden) / scale
    err = np.abs(theta - hidden) / scale
    batch.close()
    return {"scenes": num_scenes, "particles": int(x4.shape[0]), "substeps": substeps,
            "gd_steps": steps, "ms_per_gd_step": 1e3 * float(np.median(times)),
            "loss_first": losses[0], "loss_last": losses[-1],
            "param_error_start": {"xsph_c": float(err0[:, 0].mean()),
                                  "vorticity_epsilon": float(err0[:, 1].mean())},
            "param_error_end": {"xsph_c": float(err[:, 0].mean()),
                                "vorticity_epsilon": float(err[:, 1].mean())},
            "epsilon": epsilon, "scene_gradients_nonfinite": nonfinite,
            "note": "errors are mean |theta - hidden| / range (0.015 for c, 0.001 for eps_v)"}


def small_config(stream, with_cpu: bool):
    """The reference's CPU-runnable configuration: the 16,384-particle dam break
    (32x16x32 lattice in a 64^3 box, 3 iterations), its full 200 substeps on
    the GPU (graph replay, timed per 50 substeps: with epsilon = 0.01 the
    scene collapses into dense clumps after ~60 substeps, where every
    particle has thousands of neighbours and 16,384 threads cannot fill the
    GPU) and, when asked, through the FP32 oracle on the host cores."""
    import torch
    import pbf_gb300 as pg
    from pbf_gb300 import scenes
    sc = scenes.plain_16k()
    it = sc.params.num_solver_iterations
    sim = pg.SPH(sc.n, tuple(sc.params.grid), sc.params)
    sim.set_stream(stream.cuda_stream)
    sim.set_state(sc.x4, sc.v4)
    sim.step(3)
    sim.set_state(sc.x4, sc.v4)
    torch.cuda.synchronize()
    seg = 50
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(sc.substeps // seg + 1)]
    ev[0].record(stream)
    for k in range(sc.substeps // seg):
        sim.step(seg)
        ev[k + 1].record(stream)
    torch.cuda.synchronize()
    ms = ev[0].elapsed_time(ev[-1])
    res = {"workload": sc.name, "particles": sc.n, "solver_iterations": it,
           "substeps": sc.substeps, "ms_per_step": ms / sc.substeps,
           "value": sc.n * it * sc.substeps / (ms * 1e-3), "unit": UNIT,
           "ms_per_step_by_50": [ev[k].elapsed_time(ev[k + 1]) / seg for k in range(len(ev) - 1)],
           "sweep_choice_after": sim.sweep_choice()}
    sim.close()
    if with_cpu:
        import oracle
        o = oracle.Oracle(sc.params, sc.n)
        o.set_state(sc.x4, sc.v4)
        secs = o.step(sc.substeps)
        res["cpu_oracle"] = {"value": sc.n * it * sc.substeps / secs, "unit": UNIT,
                             "cores": oracle.max_threads(), "seconds": secs}
        o.set_state(sc.x4, sc.v4)
        secs50 = o.step(seg)
        res["cpu_oracle"]["first_50_value"] = sc.n * it * seg / secs50
    return res


def cpu_baseline(scene_name: str, substeps: int):
    """FP32 oracle on all host threads, `substeps` full substeps of the scene
    (built by the oracle's own generator)."""
    import oracle
    from oracle import scenes as oscenes
    scene = getattr(oscenes, scene_name)()
    o = oracle.Oracle(scene.params, scene.n)
    o.set_state(scene.x4, scene.v4)
    secs = o.step(substeps)
    it = scene.params.num_solver_iterations
    return {"value": scene.n * it * substeps / secs, "unit": UNIT, "cores": oracle.max_threads(),
            "kind": "port",
            "sample": f"{substeps} full substeps of the {scene.n}-particle dam break from its "
                      f"initial state ({secs:.1f} s, FP32 oracle, OpenMP)"}


def workload_config(scene, K: int, world: int) -> dict:
    """The `config` object both arms print (same keys and values)."""
    p = scene.params
    return {"workload": scene.name, "particles": scene.n,
            "solver_iterations": int(p.num_solver_iterations),
            "lattice": scene.meta.get("lattice"), "box": scene.meta.get("box"),
            "grid": [int(g) for g in p.grid], "dt": float(p.timestep),
            "epsilon": float(p.epsilon), "substeps_timed": K,
            "window": f"substeps 1-{K} of {scene.substeps}",
            "l2": "working set > L2 (no flush)",
            "parallelism": "replicas" if world > 1 else "single"}


def reference_arm(args, world: int):
    """The reference path's CPU implementation (the oracle port) on the host:
    W warm-up substeps, then the same window as the GPU arm (substeps 1..K
    from the initial scene), every substep in full.  Only the oracle is
    loaded: the scene comes from its own generator (oracle/scenes.py)."""
    import oracle
    from oracle import scenes as oscenes
    scene = getattr(oscenes, args.scene)()
    threads = oracle.max_threads()
    o = oracle.Oracle(scene.params, scene.n)
    o.set_state(scene.x4, scene.v4)
    warm = o.step(max(1, args.warmup))
    per = warm / max(1, args.warmup)
    o.set_state(scene.x4, scene.v4)
    K = args.steps
    it = scene.params.num_solver_iterations
    if per * K <= 240.0:
        secs = o.step(K)
        timed = K
        sample = (f"substeps 1-{K} of the {scene.n}-particle dam break, every substep in "
                  f"full ({secs:.1f} s wall, FP32 oracle, OpenMP)")
    else:
        # bounded: as many whole substeps of the window as fit in ~4 minutes
        timed = max(1, int(240.0 / per))
        secs = o.step(timed)
        sample = (f"substeps 1-{timed} of the {K}-substep window in full ({secs:.1f} s wall, "
                  f"FP32 oracle, OpenMP)")
    sec_per_step = secs / timed
    value = scene.n * it / sec_per_step
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
        "warmup": args.warmup, "ms_per_step": sec_per_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": workload_config(scene, K, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference = FP32 C++ restatement of pbf's GLSL shaders (the GL path needs an "
                "OpenGL 4.3 context: unavailable on this box); only the oracle library is loaded",
    }


def _sig(x, digits: int = 4):
    if isinstance(x, float):
        return float(f"{x:.{digits}g}")
    if isinstance(x, list):
        return [_sig(v, digits) for v in x]
    if isinstance(x, dict):
        return {k: _sig(v, digits) for k, v in x.items()}
    return x


def legs_summary(stable, full, batched, adjoint, adjoint5, small, recov, sharded=None) -> dict:
    """The headline figure of each leg (rounded to 4 digits)."""
    out = {}
    if sharded:
        out["batched_256_sharded"] = _sig({"ranks": sharded["ranks"],
                                           "scenes_per_s": sharded["scenes_per_s"]})
    if full:
        by = full["ms_per_step_by_25"]
        out["full_500"] = _sig({"value": full["value"], "substeps": full["substeps"],
                                "ms_per_step": full["ms_per_step"],
                                "ms_per_step_by_100": [sum(by[k:k + 4]) / len(by[k:k + 4])
                                                       for k in range(0, len(by), 4)]})
    if stable:
        out["stable_500_eps5"] = _sig({"value": stable["value"], "ms_per_step": stable["ms_per_step"]})
    if small:
        out["dam_break_16k_200"] = _sig({"value": small["value"], "ms_per_step": small["ms_per_step"],
                                         "cpu_oracle": (small.get("cpu_oracle") or {}).get("value")})
    if batched:
        out["batched_256"] = _sig({"speedup_vs_plain": batched["speedup"],
                                   "batched_scenes_per_s": batched["batched_scenes_per_s"],
                                   "bit_identical": batched["bit_identical_sampled_scenes"]})
    for key, a in (("adjoint_32k", adjoint), ("adjoint_32k_eps5", adjoint5)):
        if a:
            out[key] = _sig({"bwd_fwd": a["bwd_fwd_ratio"], "fwd_ms": a["forward_ms"],
                             "grad_finite": a["grad_finite"]})
    if recov:
        for key, r in recov.items():
            out["recovery_64_eps" + key.split("_")[-1]] = _sig({
                "ms_per_gd_step": r["ms_per_gd_step"], "loss": [r["loss_first"], r["loss_last"]],
                "c_err": [r["param_error_start"]["xsph_c"], r["param_error_end"]["xsph_c"]],
                "vort_err": [r["param_error_start"]["vorticity_epsilon"],
                             r["param_error_end"]["vorticity_epsilon"]],
                "nonfinite": r["scene_gradients_nonfinite"]})
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args, world)), flush=True)
        return 0
    from pbf_gb300 import scenes
    scene = getattr(scenes, args.scene)()
    if args.substep_stages > 0:
        substep_stages(scene, args.substep_stages)
        return 0
    if world > 1:
        # replicas: the window and e2e lines scale; the single-GPU legs
        # (full runs, batch, adjoint, splatting, the 16k configuration) would
        # only repeat on every rank
        args.no_stable = args.no_full = args.no_batched = args.no_adjoint = True
        args.no_splat = args.no_small = args.no_recovery = True

    import torch
    import torch.distributed as dist
    import pbf_gb300 as pg

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    t_leg = [time.perf_counter()]

    def leg_done(name):  # progress on stderr: wall seconds of each leg
        now = time.perf_counter()
        print(f"bench: {name} {now - t_leg[0]:.1f} s", file=sys.stderr, flush=True)
        t_leg[0] = now

    K, W = args.steps, max(3, args.warmup)
    it = scene.params.num_solver_iterations
    stream = torch.cuda.Stream()
    sim = pg.SPH(scene.n, tuple(scene.params.grid), scene.params)
    sim.set_stream(stream.cuda_stream)

    # warm-up: with --autotune, the autotuner fixes block size, sweep mode and
    # list settings on the first substeps of this scene (no setting changes
    # any result); by default the handle's automatic sweep configuration runs.
    # W substeps capture the graph; reset after
    sim.set_state(scene.x4, scene.v4)
    tuning = sim.autotune(10) if args.autotune else None
    sim.set_state(scene.x4, scene.v4)
    sim.step(W)
    sim.synchronize()
    sim.set_state(scene.x4, scene.v4)

    clocks = ClockSampler(local) if rank == 0 else None
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    launched0 = sim.kernels_launched()
    e0.record(stream)
    sim.step(K)
    e1.record(stream)
    launches = sim.kernels_launched() - launched0
    torch.cuda.synchronize()
    barrier()
    sim.synchronize()  # surfaces any device status error
    ms = e0.elapsed_time(e1)
    clk = clocks.stop() if clocks else None
    if tuning is None:
        tuning = {"sweep_mode": "auto", "after_window": sim.sweep_choice()}
    t = torch.tensor([ms], device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    value = world * scene.n * it * K / (ms * 1e-3)
    # the state at the end of the timed window (outside the timed region)
    state_after = sim.diagnostics()

    # per-kernel durations (eager, events per kernel) over the first
    # min(K, 50) substeps of the same window
    KT = min(K, 50)
    sim.set_state(scene.x4, scene.v4)
    sim.EnableTiming(True)
    sim.step(KT)
    stages, counted = sim.stage_times()
    sim.EnableTiming(False)
    # the dominant solver sweep: lambda (k_lambda_build on the first
    # iteration, k_lambda after, each scanning the stencil and recording the
    # pair lists) or delta-p (k_delta_p, replaying them)
    per_launch = {"lambda": stages["lambda"] / (counted * it),
                  "delta_p": stages["delta_p"] / (counted * it)}
    dom = max(per_launch, key=per_launch.get)
    peak, peak_kind = measured_peaks()
    achieved = ALG_BYTES[dom] * scene.n / (per_launch[dom] * 1e-3) / 1e9
    prof = profiled_traffic()
    traffic = None
    if prof and dom in prof.get("bytes_per_particle", {}):
        traffic = prof["bytes_per_particle"][dom] * scene.n
    total_stage = sum(stages.values())

    # end to end through the C ABI with pinned host buffers
    E = args.e2e_steps or min(K, 50)
    hx = [torch.from_numpy(scene.x4.copy()).pin_memory() for _ in range(2)]
    hv = [torch.from_numpy(scene.v4.copy()).pin_memory() for _ in range(2)]
    lib = pg.load()
    h = sim.handle
    barrier()
    torch.cuda.synchronize()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for k in range(E):
        a, b = k % 2, (k + 1) % 2
        pg._capi.check(lib.pbf_set_state(h, hx[a].data_ptr(), hv[a].data_ptr(), pg.PBF_HOST), h)
        pg._capi.check(lib.pbf_step(h, 1), h)
        pg._capi.check(lib.pbf_get_state(h, hx[b].data_ptr(), hv[b].data_ptr(), pg.PBF_HOST), h)
    f1.record(stream)
    torch.cuda.synchronize()
    barrier()
    e2e_ms = f0.elapsed_time(f1)
    t = torch.tensor([e2e_ms], device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_ms = float(t.item())
    e2e_value = world * scene.n * it * E / (e2e_ms * 1e-3)

    # the same scene with the reference's default epsilon: a stable run of
    # the full 500 substeps
    leg_done('window, e2e and stage timing')
    stable = None
    if not args.no_stable:
        ps = scene.params.copy()
        ps.epsilon = 5.0
        sim.set_params(ps)
        sim.set_state(scene.x4, scene.v4)
        stable_tuning = sim.autotune(10) if args.autotune else None
        sim.set_state(scene.x4, scene.v4)
        sim.step(3)
        sim.set_state(scene.x4, scene.v4)
        torch.cuda.synchronize()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        sim.step(scene.substeps)
        g1.record(stream)
        torch.cuda.synchronize()
        sim.synchronize()
        sms = g0.elapsed_time(g1)
        if stable_tuning is None:
            stable_tuning = {"sweep_mode": "auto", "after_run": sim.sweep_choice()}
        stable = {"value": scene.n * it * scene.substeps / (sms * 1e-3), "unit": UNIT,
                  "substeps": scene.substeps, "ms_per_step": sms / scene.substeps,
                  "epsilon": 5.0, "tuning": stable_tuning,
                  "note": "same scene and constants except CFM epsilon = 5 "
                          "(src/SPH.cpp:138), full run"}
        sim.set_params(scene.params)

    # the workload's own full run (epsilon = 0.01, all substeps): the fluid
    # collapses into dense clumps and corner piles after ~100 substeps, where
    # the automatic sweep configuration moves to the direct sweeps
    leg_done('stable_500')
    full = None
    if not args.no_full:
        # 25-substep segments, host-synchronised, until the budget is spent
        sim.set_state(scene.x4, scene.v4)
        torch.cuda.synchronize()
        seg = 25
        seg_ms = []
        t_start = time.perf_counter()
        while len(seg_ms) * seg < scene.substeps:
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            sim.step(seg)
            b.record(stream)
            b.synchronize()
            seg_ms.append(a.elapsed_time(b))
            if args.full_budget > 0 and time.perf_counter() - t_start > args.full_budget:
                break
        sim.synchronize()
        done = len(seg_ms) * seg
        fms = sum(seg_ms)
        full = {"value": scene.n * it * done / (fms * 1e-3), "unit": UNIT,
                "substeps": done, "of_substeps": scene.substeps, "ms_per_step": fms / done,
                "ms_per_step_by_25": seg_ms and [t / seg for t in seg_ms],
                "complete": done == scene.substeps,
                "sweep_choice_after": sim.sweep_choice(),
                "state_after": sim.diagnostics(),
                "note": "graph replay with the default automatic sweep configuration (its "
                        "trials are real substeps of the run); "
                        + ("all substeps" if done == scene.substeps else
                           f"stopped after {done} substeps at the --full-budget of "
                           f"{args.full_budget:.0f} s")}

    leg_done('full_500')
    adjoint = adjoint5 = None
    if not args.no_adjoint:
        adjoint = adjoint_ratio(stream)
        adjoint5 = adjoint_ratio(stream, epsilon=5.0)
    leg_done('adjoint')
    splats = None
    if not args.no_splat:
        splats = splat_leg(stream)

    leg_done('splat')
    recov = None
    if not args.no_recovery:
        recov = {"workload_epsilon_0.01": recovery(stream, steps=args.recovery_steps_eps001),
                 "reference_default_epsilon_5": recovery(stream, epsilon=5.0)}

    leg_done('recovery')
    batched = None
    if not args.no_batched:
        sim.close()
        torch.cuda.empty_cache()
        batched = batched_vs_plain(stream, plain_every=args.plain_every)
    leg_done('batched_256')
    sharded = None
    if world > 1:
        sim.close()
        torch.cuda.empty_cache()
        sharded = batched_sharded(stream, rank, world, barrier)

    leg_done('sharded batch')
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args.scene, args.cpu_substeps)
    leg_done('cpu baseline')
    small = None
    if not args.no_small:
        small = small_config(stream, rank == 0 and world == 1 and not args.no_cpu_baseline)

    leg_done('dam_break_16k_200')
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(scene, K, world),
            "tuning": tuning,
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": 2 * 16 * scene.n, "d2h_bytes_per_step": 2 * 16 * scene.n,
                    "ms_per_step": e2e_ms / E, "steps": E},
            "roofline": {"bound": "hbm", "kernel": KERNEL_NAMES[dom], "achieved": achieved, "peak": peak,
                         "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic,
                         "traffic_source": (None if traffic is None else
                                            f"{prof.get('source')} (ncu capture at commit "
                                            f"{prof.get('commit', 'unknown')}; per launch, scaled "
                                            f"by particles)"),
                         "alg_bytes_per_launch": ALG_BYTES[dom] * scene.n,
                         "ms_per_launch": per_launch[dom],
                         "issue_active": (prof or {}).get("issue_active", {}).get(dom),
                         "note": "neighbour sweeps are bound by instruction issue (issue_active: "
                                 "share of issue slots used, from the committed ncu capture) and "
                                 "gather latency, not by HBM"},
            "kernel_ms_per_substep": {k: v / counted for k, v in stages.items()},
            "kernel_share": {k: v / total_stage for k, v in stages.items()},
            "gpu_launches": launches,
            "detail": {"stable_500": stable, "full_500": full, "batched_256": batched,
                       "batched_256_sharded": sharded,
                       "adjoint_32k": adjoint, "adjoint_32k_epsilon_5": adjoint5,
                       "splat_reference_scene": splats, "dam_break_16k_200": small,
                       "recovery_64": recov, "state_after_window": state_after},
            "clocks": clk,
            "cpu_baseline": cpu,
            # compact figures of every leg, last on the line so that a
            # truncated tail of the output still shows them
            "legs": legs_summary(stable, full, batched, adjoint, adjoint5, small, recov, sharded),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

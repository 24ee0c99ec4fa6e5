"""Benchmark of the GB300 SPH step (one JSON line on rank 0).

Workload: the SDF-obstacle dam break, 1,048,576 particles (128x128x64 block),
h = 0.025, in a [0,4]x[0,4]x[0,1] tank with a sphere + cone obstacle on a 128^3
boundary map.  A "step" is one plain SPH step of that scene (hash, sort, cell
table, density, forces + wall terms + integration + box collision).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
  python bench.py --leg batched|learned_1m|two_scale --steps K     (one leg alone, for profiling)

--impl reference times the reference algorithm on the host cores (the oracle's
FP32 restatement: the reference itself does not build here) on the same scene.
Multi-GPU runs are independent replicas (one scene per GPU, no exchange).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s @1M: plain vs learned-4×dt at ≤1% density err; HBM GB/s"
UNIT = "particle-steps/s"
L2_BYTES = 129 * 1024 * 1024

# Algorithmic (compulsory) bytes and flops of the two neighbour kernels, per
# particle and per interacting pair:
#   k_density: reads a position (12 B of xyz + 4 B), writes rho and p: 24 B;
#              15 flop per pair within h, the particle itself included;
#   k_force:   reads position, velocity, rho and p, writes position, velocity
#              and acceleration: 56 B, plus 8 B per cell (start/end) and 12 B
#              per boundary-map node (distance, wall density, wall viscosity);
#              40 flop per interacting pair (0 < r <= h).
DENSITY_BYTES_PER_PARTICLE = 24
FORCE_BYTES_PER_PARTICLE = 56
DENSITY_FLOP_PER_PAIR = 15
FORCE_FLOP_PER_PAIR = 40
# The source files the neighbour kernels are compiled from: a DRAM traffic
# figure recorded under profiles/ holds only while their hash is unchanged.
KERNEL_SOURCES = ["cudasphnew_gb300/csrc/" + f for f in
                  ("sph_step.cu", "sph_device.cuh", "sph_internal.h", "sph_mlp_tile.cuh", "sph_corrector.h",
                   "sph_tc.cuh")] + ["include/sph.h"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="config2")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true",
                    help="skip the 64-scene batched leg and the two-scale leg")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the learned-corrector legs (16,384-particle scene and the 1M scene)")
    ap.add_argument("--leg", choices=["plain", "batched", "learned_1m", "two_scale"], default=None,
                    help="run only this leg (plain: W warm-up and K graph-launched plain steps of the scene, "
                         "library default launch shapes; batched: the 64-scene batch; learned_1m: train the "
                         "corrector on the 16,384-particle scene, then the learned leg of the 1M scene; "
                         "two_scale: the two-scale run) and print its JSON object; for profiling")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the library's default launch shapes (for profiling runs)")
    return ap.parse_args()


def dist_setup(n_gpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # noqa: F811
        dist.init_process_group("gloo")
    return rank, world, local, dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def max_over_ranks(dist, x):
    """The slowest rank's time: the job's time (replicas, no data exchange)."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(world, n, steps, ms):
    """Particle-steps per second of all replicas together over the slowest rank's time."""
    return world * n * steps / (ms / 1e3)


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            pk = json.load(f)
        return float(pk["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 20 ms (the timed
    region of the default run lasts about 0.15 s)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.samples = []
        self.proc = None
        self.gpu = gpu_index
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.time(), parts))

    def wait_running(self, timeout=5.0):
        """Returns once the first sample is in (or after `timeout` seconds),
        so that the sampling covers the region that follows."""
        t_end = time.time() + timeout
        while self.proc and not self.samples and time.time() < t_end:
            time.sleep(0.01)

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0, t1):
        inside = [s for t, s in self.samples if t0 <= t <= t1]
        window = "timed_region"
        if len(inside) < 2:
            inside = [s for _, s in self.samples]
            window = "warmup_and_timed_region"
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"],
                    "samples": 0}
        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(s[1]) for s in inside if num(s[1]) is not None]
        mx = [num(s[2]) for s in inside if num(s[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in inside for k in range(4) if s[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(inside), "window": window}


def pair_count(pos, h):
    """Ordered pairs (i, j), i != j, with |x_i - x_j| <= h: the force stage's interactions."""
    import numpy as np
    from scipy.spatial import cKDTree
    t = cKDTree(np.asarray(pos, np.float64))
    return int(t.count_neighbors(t, h)) - len(pos)


def code_of(src):
    """C/C++ source without its comments and blank lines, each line stripped:
    what the compiler sees, so an edit of comments alone keeps the hash."""
    out, i, n = [], 0, len(src)
    while i < n:
        c = src[i]
        if c in "\"'":  # a string or character literal, escapes included
            j = i + 1
            while j < n and src[j] != c and src[j] != "\n":
                j += 2 if src[j] == "\\" else 1
            out.append(src[i:j + 1])
            i = j + 1
        elif src.startswith("//", i):
            j = src.find("\n", i)
            i = n if j < 0 else j
        elif src.startswith("/*", i):
            j = src.find("*/", i + 2)
            i = n if j < 0 else j + 2
            out.append(" ")
        else:
            out.append(c)
            i += 1
    return "\n".join(line.strip() for line in "".join(out).splitlines() if line.strip())


def kernel_sources_sha16():
    """Hash of the code of the neighbour kernels' source files (see
    KERNEL_SOURCES), comments and blank lines left out."""
    import hashlib
    d = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(ROOT, f), encoding="utf-8") as fh:
            d.update(code_of(fh.read()).encode())
    return d.hexdigest()[:16]


def profiled_traffic(workload):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) of
    the density and force kernels (k_density*, k_force*) from
    profiles/traffic_<workload>.md, for the kernel sources that capture was
    made from; {} when there is no capture or the sources have changed since."""
    path = os.path.join(ROOT, "profiles", f"traffic_{workload}.md")
    out = {}
    try:
        lines = open(path).read().splitlines()
    except OSError:
        return out
    sha = kernel_sources_sha16()
    for line in lines:
        cells = [c.strip() for c in line.strip().strip("|").split("|")]
        if len(cells) >= 4 and cells[0].startswith(("k_density", "k_force")) and cells[3] == sha:
            try:
                out[cells[0]] = float(cells[1])
            except ValueError:
                pass
    return out


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), for the CPU baselines."""
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for line in r.stdout.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine() or "unknown"


def fp32_peak(sms, max_mhz):
    """Nominal FP32 rate: SMs x 128 lanes x 2 (FMA) x clock, flop/s."""
    return sms * 128 * 2 * max_mhz * 1e6


def kernel_roofline(kernel, n, C, g3, pairs, t_s, hbm_gbs, fp32, traffic=None):
    """Roofline of one launch of a neighbour kernel (k_density or k_force):
    its compulsory bytes at the measured HBM peak and its flops at the FP32
    peak; `frac` is the HBM fraction (the contract's bound), `combined_frac`
    = max(T_bytes, T_flop) / T."""
    if kernel.startswith("k_density"):
        byts = DENSITY_BYTES_PER_PARTICLE * n
        flop = DENSITY_FLOP_PER_PAIR * (pairs + n)
    else:
        byts = FORCE_BYTES_PER_PARTICLE * n + 8 * C + 12 * g3
        flop = FORCE_FLOP_PER_PAIR * pairs
    t_bytes, t_flop = byts / (hbm_gbs * 1e9), flop / fp32
    achieved = byts / t_s / 1e9
    return {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm_gbs, "unit": "GB/s",
            "frac": achieved / hbm_gbs, "traffic": traffic, "algorithmic_bytes_per_launch": byts,
            "flop_per_launch": flop, "pairs": pairs, "avg_launch_us": t_s * 1e6,
            "t_bytes_us": t_bytes * 1e6, "t_flop_us": t_flop * 1e6, "fp32_peak_tflops": fp32 / 1e12,
            "limiter": "fp32" if t_flop >= t_bytes else "hbm",
            "combined_frac": max(t_bytes, t_flop) / t_s}


def make_scene(name):
    from cudasphnew_gb300 import scenes
    return getattr(scenes, name)()


def scenes_config4():
    from cudasphnew_gb300 import scenes
    return scenes.config4()


def working_set_bytes(sc):
    n = sc.n
    C = sc.params.num_cells
    maps = 0
    if sc.boundary is not None:
        d = sc.boundary.dims()
        maps = d[0] * d[1] * d[2] * 20
    return n * (16 * 6 + 8 + 4 * 3) + 8 * (C + 1) + maps


def load_oracle():
    """The oracle's shared library (the reference algorithm restated for the
    CPU), built if needed, on all host cores."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    return oracle, cores


def reference_stepper(oracle, cores, sc):
    """A plain step of the reference on the host cores: the reference's own
    kernels compiled for the host (oracle/_ref: its compute_particle_hash,
    density, acceleration, integrate_euler and collision_handling kernels, the
    threads of each spread over the cores) when that build is available, else
    the oracle's FP32 restatement of them (bit-identical on every pinned
    scene).  Returns (step(x, v) -> (x', v'), kind, description)."""
    bm = oracle.boundary_maps(sc.boundary) if sc.boundary is not None else None
    if oracle.ref_available():
        oracle.ref_set_threads(cores)
        collide = bool(sc.options.boxCollision)

        def step(x, v):
            r = oracle.ref_step_plain(sc.params, bm, x, v, collide)
            return r["pos"], r["vel"]
        return step, "reference", ("the reference's own kernels compiled for the host, each kernel's threads "
                                   "spread over the cores with OpenMP (its gravity acts along y; the work per "
                                   "step is the scene's)")

    def step(x, v):
        r = oracle.step_plain(sc.params, sc.options, bm, x, v)
        return r["pos"], r["vel"]
    return step, "port", "FP32 restatement of the reference, OpenMP over particles"


def cpu_baseline(sc, max_seconds=20.0, max_steps=50):
    """The reference step on all host cores (reference_stepper), on a bounded
    number of full steps of the same scene."""
    oracle, cores = load_oracle()
    step, kind, what = reference_stepper(oracle, cores, sc)
    x, v = step(sc.positions, sc.velocities)  # warm-up step
    steps, t0 = 0, time.perf_counter()
    while True:
        x, v = step(x, v)
        steps += 1
        el = time.perf_counter() - t0
        if el > max_seconds or steps >= max_steps:
            break
    return {"value": sc.n * steps / el, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": kind,
            "sample": f"{steps} full steps of the {sc.n}-particle scene after 1 warm-up step ({el:.1f} s, {what})"}


def cpu_baseline_two_scale(sc, max_seconds=15.0, max_steps=20):
    """AdvanceTwoScale restated on the CPU (oracle, FP32, all host cores) on a
    bounded number of full two-scale steps of the same scene."""
    oracle, cores = load_oracle()
    T = oracle.TwoScale(sc.n)
    x, v = sc.positions, sc.velocities
    r = T.step(sc.params, sc.options, None, x, v)  # warm-up step
    x, v = r["pos"], r["vel"]
    steps, t0 = 0, time.perf_counter()
    while True:
        r = T.step(sc.params, sc.options, None, x, v)
        x, v = r["pos"], r["vel"]
        steps += 1
        el = time.perf_counter() - t0
        if el > max_seconds or steps >= max_steps:
            break
    return {"value": sc.n * steps / el, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": "port",
            "sample": f"{steps} full two-scale steps of the {sc.n}-particle scene after 1 warm-up step "
                      f"({el:.1f} s, FP32 restatement of AdvanceTwoScale, OpenMP over particles)"}


def cpu_baseline_batch(scs, max_seconds=20.0):
    """The batched workload on the CPU: every scene stepped in turn by the
    reference step on all host cores (reference_stepper), whole rounds over
    the 64 scenes until the time bound."""
    oracle, cores = load_oracle()
    steppers = [reference_stepper(oracle, cores, sc) for sc in scs]
    state = [(sc.positions, sc.velocities) for sc in scs]
    rounds, t0 = 0, time.perf_counter()
    while True:
        for k in range(len(scs)):
            state[k] = steppers[k][0](*state[k])
        rounds += 1
        el = time.perf_counter() - t0
        if el > max_seconds or rounds >= 5:
            break
    n = sum(sc.n for sc in scs)
    return {"value": n * rounds / el, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": steppers[0][1],
            "sample": f"{rounds} step(s) of each of the {len(scs)} scenes ({n} particles, {el:.1f} s, "
                      f"{steppers[0][2]})"}


def run_reference(args):
    rank, world, local, dist = dist_setup(args.gpus)
    if rank != 0:
        return
    sc = make_scene(args.config)
    # each step is one full CPU step of the workload; W warm-up steps, then K
    # timed steps, bounded to ~2 minutes of CPU time
    oracle, cores = load_oracle()
    step, kind, what = reference_stepper(oracle, cores, sc)
    x, v = sc.positions, sc.velocities
    for _ in range(args.warmup):
        x, v = step(x, v)
    steps, t0 = 0, time.perf_counter()
    while steps < args.steps:
        x, v = step(x, v)
        steps += 1
        if time.perf_counter() - t0 > 120.0:
            break
    el = time.perf_counter() - t0
    val = sc.n * steps / el
    out = {"metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
           "warmup": args.warmup, "ms_per_step": el / steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "impl": "reference",
           "config": {"workload": sc.name, "particles": sc.n, "cells": sc.params.num_cells,
                      "boundary_map": list(sc.boundary.dims()) if sc.boundary is not None else None,
                      "parallelism": "replicas" if world > 1 else "single"},
           "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "cpu": cpu_model(), "kind": kind,
                            "sample": f"{steps} of {args.steps} requested full steps after {args.warmup} "
                                      f"warm-up steps (bounded to ~2 min), {what} (the reference's application "
                                      f"does not build: Windows/GL headers, removed CUDA texture references)"},
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def time_steps(torch, stream, sim, mode, count):
    """Device time (ms) of `count` graph-launched steps of `mode` on `stream`."""
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        e0.record()
        sim.step(mode=mode, count=count)
        e1.record()
    torch.cuda.synchronize()
    sim.synchronize()
    return e0.elapsed_time(e1)


def fp64_density(oracle, sc, pos, vel):
    """Densities at the given positions, from the oracle's FP64 density pass."""
    return oracle.step_plain(sc.params, sc.options, None, pos, vel, fp64=True)["rho"]


def density_field(sc, pos, pts):
    """sum_j m W_poly6(|x - x_j|) at the sample points `pts` (float64)."""
    import numpy as np
    from scipy.spatial import cKDTree
    h = float(sc.params.compactSupport)
    k = float(sc.params.particleMass) * float(sc.params.poly6)
    tree = cKDTree(pos.astype(np.float64))
    out = np.zeros(len(pts))
    for i, lst in enumerate(tree.query_ball_point(pts, h)):
        if lst:
            d = pts[i] - pos[lst]
            out[i] = k * (np.maximum(h * h - (d * d).sum(1), 0.0) ** 3).sum()
    return out


def density_errors(oracle, sc, ref, pos, vel, pts):
    """Three density errors of a state against the FP64 reference state `ref`:
    per particle (same particle index), of the density field sampled on a
    fixed grid inside the fluid (points where the reference field exceeds
    half the rest density), and of the mean density."""
    import numpy as np
    rho = fp64_density(oracle, sc, pos.astype(np.float64), vel.astype(np.float64))
    pp = np.abs(rho - ref["rho"]) / ref["rho"]
    f = density_field(sc, pos, pts)
    inside = ref["field"] > 0.5 * float(sc.params.restDensity)
    fe = np.abs(f[inside] - ref["field"][inside]) / ref["field"][inside]
    return {"per_particle_mean": float(pp.mean()), "per_particle_max": float(pp.max()),
            "field_mean": float(fe.mean()), "field_max": float(fe.max()),
            "mean_density": float(abs(rho.mean() - ref["rho"].mean()) / ref["rho"].mean())}


def learned_leg(lib, torch, stream):
    """Learned 4x-dt corrector on the plain 16,384-particle dam break: trained on
    2,000 plain steps of dt = 1e-4, then 500 learned steps of 4e-4 from the same
    start, against 2,000 plain steps; density error against the FP64 oracle's
    own trajectory at the same time."""
    import numpy as np
    from cudasphnew_gb300 import scenes
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # FP64 reference trajectory (the error measure only)
    if not os.path.exists(oracle.LIB_PATH):
        oracle.build()
    oracle.set_threads(os.cpu_count() or 1)
    sc = scenes.config1()
    K, train_steps, learned_steps = 4, 2000, 500
    dt = float(sc.params.timeStep)
    x0, v0 = sc.positions, sc.velocities
    sim = lib.ParticleSimulation(sc.params, x0, v0, sc.options, sc.boundary)
    sim.set_stream(stream.cuda_stream)
    cfg = lib.CorrectorConfig.default(trainSteps=train_steps, stride=K, auditInterval=16, densityTolerance=0.01)
    t0 = time.perf_counter()
    rep = sim.train_corrector(cfg)
    train_wall = time.perf_counter() - t0
    model = sim.save_corrector()
    plain_pos, plain_vel = sim.positions(), sim.velocities()
    # plain timing: 2,000 steps from the start (graph captured by the warm-up)
    sim.write_state(x0, v0)
    sim.step(count=10)
    sim.write_state(x0, v0)
    ms_plain = time_steps(torch, stream, sim, lib.SPH_STEP_PLAIN, train_steps)
    # learned timing: warm-up captures the learned and the audit graph
    sim.write_state(x0, v0)
    sim.step(mode=lib.SPH_STEP_LEARNED, count=20)
    before = sim.corrector_report()
    sim.write_state(x0, v0)
    ms_learned = time_steps(torch, stream, sim, lib.SPH_STEP_LEARNED, learned_steps)
    after = sim.corrector_report()
    lpos, lvel = sim.positions(), sim.velocities()
    sim.close()
    # the uncorrected long step, for comparison (not timed)
    p4 = type(sc.params).from_buffer_copy(bytes(sc.params))
    p4.timeStep = float(np.float32(dt * K))
    p4.timeStepSubParticles = p4.timeStep
    with lib.ParticleSimulation(p4, x0, v0, sc.options, sc.boundary) as coarse:
        coarse.step(count=learned_steps)
        cpos, cvel = coarse.positions(), coarse.velocities()
    # FP64 oracle trajectory of 2,000 plain steps
    t1 = time.perf_counter()
    x, v = x0.astype(np.float64), v0.astype(np.float64)
    for _ in range(train_steps):
        r = oracle.step_plain(sc.params, sc.options, None, x, v, fp64=True)
        x, v = r["pos"], r["vel"]
    fp64_wall = time.perf_counter() - t1
    h = float(sc.params.compactSupport)
    g = np.arange(h / 2, 1.0, h)  # the unit box at spacing h
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    ref = {"rho": fp64_density(oracle, sc, x, v), "field": density_field(sc, x, pts)}
    el = density_errors(oracle, sc, ref, lpos, lvel, pts)
    ec = density_errors(oracle, sc, ref, cpos, cvel, pts)
    ep = density_errors(oracle, sc, ref, plain_pos, plain_vel, pts)
    sim_plain = train_steps * dt / (ms_plain / 1e3)
    sim_learned = learned_steps * K * dt / (ms_learned / 1e3)
    short = learned_short_horizon(lib, sc, model, cfg, oracle)
    m = float(sc.params.particleMass)
    ke = {"fp64": 0.5 * m * float((v ** 2).sum()),
          "learned_4dt": 0.5 * m * float((lvel.astype(np.float64) ** 2).sum()),
          "uncorrected_4dt": 0.5 * m * float((cvel.astype(np.float64) ** 2).sum()),
          "plain_fp32_dt": 0.5 * m * float((plain_vel.astype(np.float64) ** 2).sum())}
    return {"workload": f"{sc.name}: {sc.n} particles, plain dt {dt:g} x {train_steps} steps vs learned "
                        f"{K}x dt x {learned_steps} steps, same start and end time",
            "unit": "simulated s / wall s",
            "plain": sim_plain, "learned": sim_learned, "speedup": sim_learned / sim_plain,
            "plain_ms_per_step": ms_plain / train_steps, "learned_ms_per_step": ms_learned / learned_steps,
            "density_err_vs_fp64": {"learned_4dt": el, "uncorrected_4dt": ec, "plain_fp32_dt": ep,
                                    "reading": "the <=1% bar reads 'mean density error' as the error of the "
                                               "mean density (mean_density); per-particle and field errors at "
                                               "0.2 s are dominated by the trajectories' chaotic divergence, "
                                               "which the plain FP32 solver at dt shows too",
                                    "note": "against the FP64 oracle's 2,000-step trajectory at the same time"},
            "kinetic_energy_J": ke,
            "short_horizon_vs_fp64": short,
            "audit_interval": cfg.auditInterval, "density_tolerance": cfg.densityTolerance,
            "audits": after.audits - before.audits, "rollbacks": after.rollbacks - before.rollbacks,
            "max_audit_err": after.maxAuditError,
            "training": {"samples": rep.samples, "adam_steps": rep.optimizerSteps,
                         "loss_first_epoch": rep.firstEpochLoss, "loss_last_epoch": rep.lastEpochLoss,
                         "device_ms": rep.trainMilliseconds, "wall_s": train_wall},
            "fp64_oracle_wall_s": fp64_wall,
            "l2": "not flushed: the 16,384-particle state (~3 MB) stays L2-resident in use"}, cfg, model


def learned_short_horizon(lib, sc, model, cfg, oracle, starts=(250, 750, 1250, 1750), horizons=(4, 16)):
    """Accuracy of the learned 4xdt step against the uncorrected 4xdt step and
    the plain step at dt over short horizons (H learned steps = 4H plain
    steps) from states of the plain trajectory, each against the FP64
    oracle's own steps from the same state: the mean per-particle density
    error (the density recomputed by the FP64 density pass at the end state)
    and the RMS position error.  Before the trajectories' chaotic divergence
    dominates (some tens of steps) these compare the integrators themselves."""
    import numpy as np
    K = cfg.stride
    with lib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        states, t0 = [], 0
        for t in starts:
            sim.step(count=t - t0)
            t0 = t
            states.append((t, sim.positions(), sim.velocities()))
    p4 = type(sc.params).from_buffer_copy(bytes(sc.params))
    p4.timeStep = float(np.float32(float(sc.params.timeStep) * K))
    p4.timeStepSubParticles = p4.timeStep
    rows = []
    for H in horizons:
        for t, xs, vs in states:
            x, v = xs.astype(np.float64), vs.astype(np.float64)
            for _ in range(H * K):
                r = oracle.step_plain(sc.params, sc.options, None, x, v, fp64=True)
                x, v = r["pos"], r["vel"]
            rho64 = fp64_density(oracle, sc, x, v)
            ends = {}
            with lib.ParticleSimulation(sc.params, xs, vs, sc.options, sc.boundary) as s:
                s.step(count=H * K)
                ends["plain_dt"] = (s.positions(), s.velocities())
            with lib.ParticleSimulation(p4, xs, vs, sc.options, sc.boundary) as s:
                s.step(count=H)
                ends["uncorrected_4dt"] = (s.positions(), s.velocities())
            c = lib.CorrectorConfig.default(stride=K, auditInterval=0, densityTolerance=cfg.densityTolerance)
            with lib.ParticleSimulation(sc.params, xs, vs, sc.options, sc.boundary) as s:
                s.load_corrector(model, c)
                s.step(mode=lib.SPH_STEP_LEARNED, count=H)
                ends["learned_4dt"] = (s.positions(), s.velocities())
            row = {"start_step": t, "learned_steps": H}
            for name, (px, pv) in ends.items():
                rho = fp64_density(oracle, sc, px.astype(np.float64), pv.astype(np.float64))
                row[name] = {"density_err_mean": float((np.abs(rho - rho64) / rho64).mean()),
                             "position_rms_m": float(np.sqrt(((px - x) ** 2).sum(1).mean()))}
            rows.append(row)
    return rows


def train_corrector_16k(lib, stream):
    """The learned leg's corrector alone: trained on 2,000 plain steps of the
    16,384-particle scene (the same configuration as learned_leg)."""
    from cudasphnew_gb300 import scenes
    sc = scenes.config1()
    cfg = lib.CorrectorConfig.default(trainSteps=2000, stride=4, auditInterval=16, densityTolerance=0.01)
    with lib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.set_stream(stream.cuda_stream)
        sim.train_corrector(cfg)
        return sim.save_corrector(), cfg


def learned_leg_1m(lib, torch, stream, model, cfg, sc, steps):
    """The corrector trained on the 16,384-particle scene, run on the 1M obstacle
    scene: `steps` plain steps against steps/4 learned steps from the same start;
    density error against that plain FP32 trajectory (the FP64 oracle is too
    slow at this size)."""
    import numpy as np
    K = cfg.stride
    steps = (steps // K) * K
    dt = float(sc.params.timeStep)
    x0, v0 = sc.positions, sc.velocities
    with lib.ParticleSimulation(sc.params, x0, v0, sc.options, sc.boundary) as sim:
        sim.set_stream(stream.cuda_stream)
        sim.load_corrector(model, cfg)
        sim.step(count=3)
        sim.write_state(x0, v0)
        ms_plain = time_steps(torch, stream, sim, lib.SPH_STEP_PLAIN, steps)
        ppos, pvel = sim.positions(), sim.velocities()
        sim.write_state(x0, v0)
        sim.step(mode=lib.SPH_STEP_LEARNED, count=cfg.auditInterval + 1)
        before = sim.corrector_report()
        sim.write_state(x0, v0)
        ms_learned = time_steps(torch, stream, sim, lib.SPH_STEP_LEARNED, steps // K)
        after = sim.corrector_report()
        lpos, lvel = sim.positions(), sim.velocities()
        # densities at both end states through the plain density pass
        rho = []
        for pos, vel in ((ppos, pvel), (lpos, lvel)):
            sim.write_state(pos, vel)
            sim.Advance()
            rho.append(sim.read(lib.FIELD_DENSITY).astype(np.float64))
    e = np.abs(rho[1] - rho[0]) / rho[0]
    sim_plain = steps * dt / (ms_plain / 1e3)
    sim_learned = steps * dt / (ms_learned / 1e3)
    return {"workload": f"{sc.name}: {sc.n} particles, {steps} plain steps vs {steps // K} learned steps, "
                        f"model trained on the 16,384-particle scene",
            "unit": "simulated s / wall s", "plain": sim_plain, "learned": sim_learned,
            "speedup": sim_learned / sim_plain,
            "learned_particle_steps_per_s": sc.n * (steps // K) / (ms_learned / 1e3),
            "plain_particle_steps_per_s": sc.n * steps / (ms_plain / 1e3),
            "mean_density_err_vs_plain_fp32": float(e.mean()), "max_density_err_vs_plain_fp32": float(e.max()),
            "audits": after.audits - before.audits, "rollbacks": after.rollbacks - before.rollbacks}


def plain_leg(lib, torch, stream, sc, warmup, steps):
    """W warm-up and K graph-launched plain steps of `sc` with the library's
    default launch shapes (the command the ncu captures under profiles/ run)."""
    with lib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.set_stream(stream.cuda_stream)
        sim.step(count=max(warmup, 1))
        ms = time_steps(torch, stream, sim, lib.SPH_STEP_PLAIN, steps)
        tuning = sim.tuning().as_dict()
    return {"workload": sc.name, "particles": sc.n, "steps": steps, "warmup": max(warmup, 1),
            "ms_per_step": ms / steps, "tuning": tuning}


def with_skin(sc, skin):
    """The scene's options with another neighbourSkin (0: the neighbour search
    in every step)."""
    o = type(sc.options).from_buffer_copy(bytes(sc.options))
    o.neighbourSkin = skin
    return o


def lists_leg(lib, torch, stream, sc, steps, tuning, late_start=1000, late_steps=200):
    """The reused neighbour lists against the per-step search on the same
    scene and launch shapes: the first `steps` steps from the initial state,
    and a later window (`late_steps` steps after `late_start` steps, when the
    fluid moves fast and the lists are built every few steps)."""
    import numpy as np
    out = {"skin": float(sc.options.neighbourSkin),
           "rebuild_distance_m": 0.45 * float(sc.options.neighbourSkin) * float(sc.params.compactSupport)}
    for label, skin in (("lists", float(sc.options.neighbourSkin)), ("per_step_search", 0.0)):
        with lib.ParticleSimulation(sc.params, sc.positions, sc.velocities, with_skin(sc, skin),
                                    sc.boundary) as sim:
            sim.set_stream(stream.cuda_stream)
            sim.set_tuning(**{k: v for k, v in tuning.items() if k in ("densityBlock", "forceBlock", "kahan")})
            sim.step(count=3)
            sim.write_state(sc.positions, sc.velocities)
            b0 = sim.neighbour_builds()
            ms = time_steps(torch, stream, sim, lib.SPH_STEP_PLAIN, steps)
            b1 = sim.neighbour_builds()
            sim.step(count=max(late_start - steps, 1))
            b2 = sim.neighbour_builds()
            ms_late = time_steps(torch, stream, sim, lib.SPH_STEP_PLAIN, late_steps)
            b3 = sim.neighbour_builds()
            vmax = float(np.linalg.norm(sim.velocities(), axis=1).max())
        out[label] = {"first_steps": steps, "ms_per_step": ms / steps, "builds": b1 - b0,
                      "late_window": f"steps {late_start}..{late_start + late_steps}",
                      "late_ms_per_step": ms_late / late_steps, "late_builds": b3 - b2,
                      "late_max_speed_m_s": vmax}
    return out


def batched_leg(lib, torch, stream, steps=200, peaks=None):
    """The 64-scene batched workload (about 4.4M particles, seeded sizes and
    sphere obstacles): one handle, one launch per stage, one CUDA graph per
    step, autotuned; beside it the same scenes as 64 separate handles stepped
    one after another (each with its own graph).  With `peaks` (HBM GB/s, its
    source, FP32 flop/s) the batched density and force launches get a
    roofline each, accounted as for one scene summed over the scenes."""
    import numpy as np
    from cudasphnew_gb300 import scenes
    scs = scenes.config4()
    n = sum(sc.n for sc in scs)
    lists = float(scs[0].options.neighbourSkin) > 0
    launches = 8 if lists else 6  # with the lists: the decision kernel and the two density forms
    roofs = None
    with lib.ParticleSimulation.batch(scs, scs[0].options) as sim:
        sim.set_stream(stream.cuda_stream)
        sim.step(count=3)
        tuning = sim.autotune(reps=3).as_dict()
        sim.step(count=3)
        ms = time_steps(torch, stream, sim, lib.SPH_STEP_PLAIN, steps)
        fp, fc = sim.scene_ranges()
        cells = int(fc[-1])
        if peaks is not None:
            hbm, hbm_kind, fp32 = peaks
            sim.step(count=1)
            pos_now = sim.positions()
            t_d = sim.time_kernel("density", 20) / 1e6
            t_f = sim.time_kernel("force", 20) / 1e6
            pairs = sum(pair_count(pos_now[fp[k]:fp[k + 1]], float(sc.params.compactSupport))
                        for k, sc in enumerate(scs))
            g3 = sum(int(np.prod(sc.boundary.dims())) for sc in scs if sc.boundary is not None)
            roofs = {}
            kd, kf = ("k_density_lists", "k_force_lists") if lists else ("k_density", "k_force")
            for key, kern, t in (("roofline_density", kd, t_d), ("roofline_force", kf, t_f)):
                r = kernel_roofline(kern, n, cells, g3, pairs, t, hbm, fp32)
                r["peak_source"] = hbm_kind
                r["timing"] = (f"20 back-to-back launches of the batched {kern} (all 64 scenes in one launch) "
                               f"on one step's sorted state, CUDA events on the library's stream")
                r["accounting"] = ("per-scene bytes and flops of the single-scene roofline summed over the scenes "
                                   "(every scene's map counted once per launch)")
                roofs[key] = r
    # the same scenes without batching, a bounded number of steps each
    k = max(steps // 10, 5)
    sims = [lib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) for sc in scs]
    try:
        for x in sims:
            x.set_stream(stream.cuda_stream)
            x.step(count=3)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            e0.record()
            for _ in range(k):
                for x in sims:
                    x.step(count=1)
            e1.record()
        torch.cuda.synchronize()
        ms_sep = e0.elapsed_time(e1)
    finally:
        for x in sims:
            x.close()
    return {"workload": f"{len(scs)} dam breaks, {n} particles (log-uniform 4,096..262,144 per scene), "
                        f"{cells} cells, one 64^3 sphere map each",
            "unit": UNIT, "steps": steps, "value": n * steps / (ms / 1e3), "ms_per_step": ms / steps,
            "launches_per_step": launches, "graph": "one CUDA graph launch per step", "tuning": tuning,
            "neighbour_lists": "reused, one build decision per scene" if lists else "per-step search",
            "separate_handles": {"value": n * k / (ms_sep / 1e3), "ms_per_step": ms_sep / k, "steps": k,
                                 "launches_per_step": launches * len(scs)},
            "l2": "no flush: working set of the 4.4M-particle batch far exceeds L2", **(roofs or {})}


def two_scale_leg(lib, torch, stream, steps=500, peaks=None):
    """The 262,144-particle two-scale run (AdvanceTwoScale with persistent
    children and merge-back), against the plain step of the same scene.
    With `peaks` (HBM GB/s, its source, FP32 flop/s): stage times of a few
    more two-scale steps (CUDA events between the stages, eager launches)
    and a roofline of the fine level's density and force stages."""
    import numpy as np
    from scipy.spatial import cKDTree
    from cudasphnew_gb300 import scenes
    sc = scenes.config3()
    fine = None
    with lib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary) as sim:
        sim.set_stream(stream.cuda_stream)
        sim.step(mode=lib.SPH_STEP_TWO_SCALE, count=5)
        ms = time_steps(torch, stream, sim, lib.SPH_STEP_TWO_SCALE, steps)
        c = sim.counts()
        if peaks is not None:
            hbm, hbm_kind, fp32 = peaks
            k = 20
            sim.set_stage_timing(k)
            sim.step(mode=lib.SPH_STEP_TWO_SCALE, count=k)
            t = sim.stage_times()
            sim.set_stage_timing(0)
            stage_us = {name: 1e3 * v[0] / v[1] for name, v in t.items() if v[1] > 0}
            cf = sim.counts()
            ids = sim.read(lib.FIELD_SUB_IDS)
            xs = sim.read(lib.FIELD_SUB_VERTEX_DATA)
            n_reg, n_sub = 8 * cf.numParticlesSplit, cf.numSubParticles
            hs = float(sc.params.compactSupportSub)
            every = cKDTree(xs[ids[:n_sub]].astype(np.float64))
            regular = cKDTree(xs[ids[:n_reg]].astype(np.float64))
            pairs = int(regular.count_neighbors(every, hs)) - n_reg  # regular child i, any child j != i
            cells = int(np.prod(list(sc.params.gridDimSubParticles)))
            fine = {"stage_us": stage_us, "steps": k, "regular_children": n_reg, "children": n_sub}
            for key, kern, stage in (("roofline_sub_density", "k_density", "sub_density"),
                                     ("roofline_sub_force", "k_force", "sub_force")):
                nk = n_reg if stage == "sub_density" else n_sub
                r = kernel_roofline(kern, nk, cells if stage == "sub_force" else 0, 0, pairs,
                                    stage_us[stage] / 1e6, hbm, fp32)
                r["kernel"] = "k_ts_subdensity" if stage == "sub_density" else "k_ts_subforce"
                r["peak_source"] = hbm_kind
                r["timing"] = (f"stage interval '{stage}' (CUDA events around the launch, gaps included), "
                               f"mean of {k} eager two-scale steps")
                r["accounting"] = ("the plain step's per-particle bytes and per-pair flops applied to the fine "
                                   "level (density: regular children; force: every child, which it integrates, "
                                   "plus the fine cell table; no boundary maps at the fine level)")
                fine[key] = r
        ms_plain = time_steps(torch, stream, sim, lib.SPH_STEP_PLAIN, steps)
    return {"workload": f"{sc.name}: {sc.n} coarse particles, split region [0.4, 0.6]^3, children merged back "
                        f"on exit", "unit": UNIT, "steps": steps,
            "value": sc.n * steps / (ms / 1e3), "ms_per_step": ms / steps,
            "children_at_end": c.numSubParticles, "split_at_end": c.numParticlesSplit,
            "boundary_at_end": c.numParticlesBoundary,
            "plain_ms_per_step": ms_plain / steps,
            "graph": "one CUDA graph launch per step; counts stay on the device", "fine_level": fine}


def run_ours(args):
    import numpy as np
    import torch

    rank, world, local, dist = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from cudasphnew_gb300 import _build, lib
    _build.build()
    lib.load()
    sc = make_scene(args.config)
    n = sc.n
    stream = torch.cuda.Stream()
    if args.leg is not None:
        if rank == 0:
            if args.leg == "plain":
                res = plain_leg(lib, torch, stream, sc, args.warmup, args.steps)
            elif args.leg == "batched":
                res = batched_leg(lib, torch, stream, steps=args.steps)
            elif args.leg == "two_scale":
                res = two_scale_leg(lib, torch, stream, steps=args.steps)
            else:
                model, lcfg = train_corrector_16k(lib, stream)
                res = learned_leg_1m(lib, torch, stream, model, lcfg, sc, args.steps)
            print(json.dumps({"leg": args.leg, **res}), flush=True)
        return
    sim = lib.ParticleSimulation(sc.params, sc.positions, sc.velocities, sc.options, sc.boundary)
    sim.set_stream(stream.cuda_stream)

    # ---- warm-up (also captures the step graph) ---------------------------
    clocks = ClockSampler(local)
    clocks.start()
    sim.step(count=max(args.warmup, 3))
    sim.synchronize()
    if args.no_autotune:
        tuning = sim.tuning().as_dict()
    else:
        tuning = sim.autotune(reps=5).as_dict()  # launch shapes; state untouched
    sim.step(count=3)  # re-capture the step graph with the chosen shapes
    sim.synchronize()

    # ---- timed region: K graph-launched steps, device-resident ----------
    builds0 = sim.neighbour_builds()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    clocks.wait_running()
    barrier(dist)
    torch.cuda.synchronize()
    t_wall0 = time.time()
    with torch.cuda.stream(stream):
        e0.record()
        sim.step(count=args.steps)
        e1.record()
    torch.cuda.synchronize()
    t_wall1 = time.time()
    barrier(dist)
    sim.synchronize()  # raises on a latched device error
    builds_timed = sim.neighbour_builds() - builds0
    ms = max_over_ranks(dist, e0.elapsed_time(e1))
    clocks.stop()
    clk = clocks.summary(t_wall0, t_wall1)
    value = whole_job_value(world, n, args.steps, ms)

    # ---- per-kernel times (stage events on the same stream) ---------------
    kt = min(args.steps, 200)
    sim.set_stage_timing(kt)
    for _ in range(kt):
        sim.Advance()
    stages = sim.stage_times()
    sim.set_stage_timing(0)
    # the neighbour kernels' own launch times: back-to-back launches on the
    # last step's sorted state (the stage events above also hold launch gaps)
    sim.step(count=1)
    pos_now = sim.positions()  # the state both timed kernels work on
    density_avg_s = sim.time_kernel("density", 50) / 1e6
    force_avg_s = sim.time_kernel("force", 50) / 1e6
    peak, peak_kind = load_peaks()
    C = sc.params.num_cells
    g3 = int(np.prod(sc.boundary.dims())) if sc.boundary is not None else 0
    pairs = pair_count(pos_now, float(sc.params.compactSupport))
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32 = fp32_peak(sms, clk.get("sm_max_mhz") or 2070.0)
    traffic = profiled_traffic(sc.name)
    # the kernels a plain step of this handle runs: the list forms when the
    # scene reuses neighbour lists
    lists_on = float(sc.options.neighbourSkin) > 0
    kd, kf = ("k_density_lists", "k_force_lists") if lists_on else ("k_density", "k_force")
    roofs = {k: kernel_roofline(k, n, C, g3, pairs, t, peak, fp32, traffic.get(k))
             for k, t in ((kd, density_avg_s), (kf, force_avg_s))}
    for r in roofs.values():
        r["peak_source"] = peak_kind
        r["timing"] = (f"50 back-to-back launches of {r['kernel']} on one step's sorted state, CUDA events on "
                       f"the library's stream")
        r["traffic_source"] = (f"profiles/traffic_{sc.name}.md (ncu dram__bytes_read.sum + "
                               f"dram__bytes_write.sum, one launch, same kernel sources)"
                               if r["traffic"] is not None else "no ncu capture of the current kernel sources")
    dominant = max(roofs, key=lambda k: roofs[k]["avg_launch_us"])

    # ---- e2e: host buffers through the C ABI, copies inside the region ----
    pin_pos = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    pin_vel = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    pin_out = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)
    pin_pos.numpy()[:] = sim.positions()
    pin_vel.numpy()[:] = sim.velocities()
    L = lib.load()
    import ctypes
    e2e_steps = max(1, min(args.steps, 100))
    pin_out2 = torch.empty((n, 3), dtype=torch.float32, pin_memory=True)

    def e2e_loop(read):
        torch.cuda.synchronize()
        barrier(dist)
        t0 = time.perf_counter()
        for k in range(e2e_steps):
            out = pin_out if k % 2 == 0 else pin_out2
            lib.check(L.sph_write(sim._h, lib.FIELD_VERTEX_DATA, ctypes.c_void_p(pin_pos.data_ptr()), n * 12))
            lib.check(L.sph_write(sim._h, lib.FIELD_VELOCITY, ctypes.c_void_p(pin_vel.data_ptr()), n * 12))
            lib.check(L.sph_step(sim._h, lib.SPH_STEP_PLAIN))
            lib.check(read(sim._h, lib.FIELD_VERTEX_DATA, ctypes.c_void_p(out.data_ptr()), n * 12))
        lib.check(L.sph_synchronize(sim._h))  # the last read-back is inside the timed region
        el = max_over_ranks(dist, time.perf_counter() - t0)
        barrier(dist)
        return world * n * e2e_steps / el

    # blocking: each step's read-back waits; pipelined: sph_read_async, so a
    # step's uploads (issued while the previous step and its read-back are
    # still queued) run beside them over the host link
    e2e_blocking = e2e_loop(L.sph_read)
    e2e_value = e2e_loop(L.sph_read_async)
    sim.close()

    lists = None
    if rank == 0 and float(sc.options.neighbourSkin) > 0:
        lists = lists_leg(lib, torch, stream, sc, args.steps, tuning)
    batched = two_scale = None
    if rank == 0 and not args.no_batched:
        batched = batched_leg(lib, torch, stream, peaks=(peak, peak_kind, fp32))
        two_scale = two_scale_leg(lib, torch, stream, peaks=(peak, peak_kind, fp32))
    learned = learned_1m = None
    if rank == 0 and not args.no_learned:
        learned, lcfg, model = learned_leg(lib, torch, stream)
        # the scene's 500 plain steps against 125 learned ones, whatever --steps is: the
        # learned run then holds several audits (one per auditInterval learned steps)
        learned_1m = learned_leg_1m(lib, torch, stream, model, lcfg, sc, 500)

    if rank != 0:
        return
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": sc.name, "particles": n, "cells": C,
                      "boundary_map": list(sc.boundary.dims()) if sc.boundary is not None else None,
                      "parallelism": "replicas" if world > 1 else "single",
                      "l2": f"no flush: per-step working set {working_set_bytes(sc) / 2**20:.0f} MiB "
                            f"> {L2_BYTES / 2**20:.0f} MiB L2",
                      "graph": "one CUDA graph launch per step", "tuning": tuning},
           "clocks": clk,
           "gpu_launches": (8 if float(sc.options.neighbourSkin) > 0 else 6) * args.steps,
           "neighbour_lists": {"skin": float(sc.options.neighbourSkin), "builds_in_timed_region": builds_timed,
                               "note": "the neighbour candidates within (1 + skin) h are rebuilt when a "
                                       "particle has moved 0.45 skin h since the last build; a step that "
                                       "builds none keeps the working order and skips the hash, sort and "
                                       "cell tables (sph_read_cells builds them on demand, bit-exact)",
                               "comparison": lists},
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 2 * n * 12,
                   "d2h_bytes_per_step": n * 12, "steps": e2e_steps,
                   "path": "per step sph_write(VD) + sph_write(VEL) from pinned host buffers, sph_step, "
                           "sph_read_async(VD) into a pinned host buffer; one sph_synchronize at the end, "
                           "inside the timed region",
                   "blocking_value": e2e_blocking,
                   "blocking_path": "the same with sph_read (each read-back waited for)"},
           "roofline": roofs[dominant],
           "roofline_density": roofs[kd],
           "roofline_force": roofs[kf],
           "stages_us": {k: round(v[0] / v[1] * 1e3, 2) for k, v in stages.items() if v[1] > 0}}
    if batched is not None:
        out["batched"] = batched
        out["two_scale"] = two_scale
    if learned is not None:
        out["learned"] = learned
        out["learned_1m"] = learned_1m
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(sc)
        if batched is not None:
            batched["cpu_baseline"] = cpu_baseline_batch(scenes_config4())
            two_scale["cpu_baseline"] = cpu_baseline_two_scale(make_scene("config3"))
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

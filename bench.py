#!/usr/bin/env python
"""Benchmark of the SPH substep pipeline on GB300.

Default workload: the 1,048,576-particle dam break (128x64x128 lattice at
spacing 0.1 in a 25.6x12.8x25.6 box, r 0.175, dt 1/120 in 2 substeps). One
step = one dt = 2 substeps = one FluidSimBase::update(dt).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints ONE JSON line (rank 0). `value` = particle-steps/s of the whole job
with the state resident in HBM (CUDA events on the library's stream, L2
flushed before every timed step); `e2e` = the same metric through the public
API with the state in pinned host memory (upload + step + download every
step). For N>1 every rank runs an independent replica of the scene (the path
has no cross-scene exchange): weak scaling, max time over ranks.

At N=1 the same line also carries the two other forms of one GPU:
  "batched": 256 independent scenes (9.4M particles) advanced by one set of
             segmented launches per substep, against the same scenes stepped
             back to back as plain single-scene launches;
  "served":  a Poisson stream of scene requests at 200 req/s for
             --serve-seconds (default 60) through the library's serving loop
             (HBM-budget admission, continuous batching), with p50/p99
             per-step latency, against --serial-sample (default 100) of the
             stream's requests run one after another as plain launches.
--no-batched / --no-served leave them out; --workload batched_256 / served
run one of them alone.

--impl reference times the reference CPU implementation of the path on the
host cores (the oracle's restatement, all hardware threads; the reference's
own build where it exists here) on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = pathlib.Path(__file__).resolve().parent
PKG = ROOT / "fluid-simulation-3d_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s"
UNIT = "particle-steps/s"
# Compulsory unique bytes per particle of each kernel of a substep (reads +
# writes of its inputs and outputs once), for the roofline.
ALG_BYTES = {
    "predict_hash": 44,   # pos 16 + vel 16 in; key/rank 8 + count 4 out
    "spatial": 172,       # scan 12 per key-table entry + scatter 24 + reorder 96
                          # + cell table ~40 (216 B of row runs per cell, ~5.4
                          # particles a cell); spatial_bytes() gives the scene's
    "density": 44,        # pred 16 + start 4 in; dens_a 8 + dens_b 16 out
    "pressure": 76,       # pred 16, start 4, dens_a 8, dens_b 16, vel 16 in; velp 16 out
    "viscosity": 84,      # pred 16, start 4, velp 16, pos 16 in; pos 16 + vel 16 out
    # (pred and velp travel together as the 32-byte rec_v record; its pred
    # half is a copy, so it is not counted as compulsory)
}
# Whole-substep compulsory traffic per particle: the sum of the per-kernel
# algorithmic bytes of an idealised substep (predict+hash 68, counting sort
# 20, reorder 68, density 24, forces 56, integrate 64).
SUBSTEP_ALG_BYTES = 300


def spatial_bytes(grid: bool, entries: int, n: int) -> float:
    """Algorithmic bytes per particle of the sort phase for a key table of
    `entries` entries: a grid table (one entry per cell) needs no cell-table
    kernel, a bucket table (n entries) does."""
    return 12.0 * entries / n + 24 + 96 + (0 if grid else 40)
PHASES = ["predict_hash", "spatial", "density", "pressure", "viscosity"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["native", "reference"], default="native")
    ap.add_argument("--workload", default="dam_break_1m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--serve-seconds", type=float, default=60.0)
    ap.add_argument("--serial-sample", type=int, default=100)
    ap.add_argument("--no-batched", action="store_true",
                    help="leave the batched (config 2) block out of the default line")
    ap.add_argument("--no-served", action="store_true",
                    help="leave the served (config 3) block out of the default line")
    ap.add_argument("--e2e-steps", type=int, default=None)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x: float, world: int, device) -> float:
    """The largest `x` of all ranks (the job lasts as long as its slowest
    replica); `x` itself for one rank."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as tdist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(n_local: int, steps: int, total_ms: float, world: int,
                       device):
    """Whole-job particle-steps/s of `world` independent replicas (weak
    scaling): every rank advanced n_local particles `steps` times in its own
    `total_ms`; returns (value, job ms = max over ranks)."""
    job_ms = max_over_ranks(total_ms, world, device)
    return world * n_local * steps / (job_ms / 1000.0), job_ms


def peaks():
    try:
        with open(ROOT / "MEASURED_PEAKS.json") as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(workload, kernel):
    """DRAM bytes per launch per particle from a committed ncu summary."""
    try:
        with open(ROOT / "profiles" / "dram_traffic.json") as f:
            d = json.load(f)
        return d[workload][kernel]
    except Exception:
        return None


def ncu_issue(workload, kernel):
    """Issue-slot use of a kernel from the same ncu summary: percent of
    cycles with an instruction issued, active lanes per instruction and warp
    instructions per particle (what bounds a kernel that is not HBM-bound)."""
    try:
        with open(ROOT / "profiles" / "dram_traffic.json") as f:
            d = json.load(f)
        return d["issue"][workload][kernel]
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed
    region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, interval_ms=200):
        self.gpu = gpu_index
        self.interval_ms = int(interval_ms)
        self.proc = None
        self.tmp = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self, wait_live=False):
        """Start sampling; with wait_live, return once the first sample is
        written (at most 3 s), so a short region that follows is covered."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", str(self.interval_ms)],
                stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        t0 = time.perf_counter()
        while wait_live and time.perf_counter() - t0 < 3.0:
            self.tmp.flush()
            if os.path.getsize(self.tmp.name) > 0:
                break
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.tmp.flush()
        self.tmp.seek(0)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.tmp.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.tmp.name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# FP32 operations counted per pair test (the density pass's candidate test:
# 3 subtractions + the 3-term distance, 1 compare) and per neighbour (density
# term 5, pressure term 25, viscosity term 15, each with its own distance).
FLOPS_PER_CANDIDATE = 9
FLOPS_PER_NEIGHBOUR = 45 + 2 * 8


def pair_stats(sc, sample=4096, seed=0):
    """Mean candidates (particles of the 27 neighbour cells, self included)
    and neighbours (other particles within r) per particle, over a seeded
    sample of the scene's initial state."""
    from scipy.spatial import cKDTree
    pos = np.ascontiguousarray(sc["pos"], np.float32)
    r = np.float32(sc["params"].radius)
    cells = np.floor(pos / r).astype(np.int64)
    lo = cells.min(axis=0) - 1
    dims = cells.max(axis=0) - lo + 2
    key = ((cells[:, 2] - lo[2]) * dims[1] + (cells[:, 1] - lo[1])) * dims[0] + (cells[:, 0] - lo[0])
    uniq, counts = np.unique(key, return_counts=True)
    rng = np.random.default_rng(seed)
    idx = rng.choice(pos.shape[0], min(sample, pos.shape[0]), replace=False)
    cand = np.zeros(idx.shape[0], np.int64)
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                k = key[idx] + (dz * dims[1] + dy) * dims[0] + dx
                at = np.clip(np.searchsorted(uniq, k), 0, uniq.shape[0] - 1)
                cand += np.where(uniq[at] == k, counts[at], 0)
    tree = cKDTree(pos.astype(np.float64))
    nb = np.array([len(v) - 1 for v in tree.query_ball_point(pos[idx].astype(np.float64), float(r))])
    return float(cand.mean()), float(nb.mean())


def nominal_fp32_tflops(device=0):
    """SMs x 128 FP32 lanes x 2 (FMA) x max SM clock: the CUDA-core peak."""
    import torch
    props = torch.cuda.get_device_properties(device)
    try:
        with open(ROOT / "MEASURED_PEAKS.json") as f:
            mhz = float(json.load(f)["sm_max_mhz"])
    except Exception:
        mhz = 2070.0
    return props.multi_processor_count * 128 * 2 * mhz * 1e6 / 1e12


def load_workload(name):
    from fluidsim import scenes
    if name not in scenes.WORKLOADS:
        raise SystemExit(f"unknown workload {name}")
    return scenes.WORKLOADS[name]()


def cpu_port_rate(sc, max_steps, budget_s, threads=0, warm_steps=0):
    """Oracle restatement (Jacobi, all host threads) on the full scene: after
    `warm_steps` untimed steps from the scene (the warm-up steps the GPU arm
    takes before its timed steps, so both time the same part of the flow),
    steps until `max_steps` or `budget_s`; returns (particle-steps/s, steps
    timed, seconds, threads)."""
    import oracle
    oracle.build()
    p, n, S = sc["params"], sc["pos"].shape[0], sc["substeps"]
    dt = np.float32(np.float32(sc["dt"]) / np.float32(S))
    pos, vel = sc["pos"].copy(), sc["vel"].copy()
    th = threads or oracle.hw_threads()
    for _ in range(warm_steps):
        for _ in range(S):
            pos, vel, _ = oracle.substep_f32(p, pos, vel, dt, nthreads=th, debug=False)
    t0 = time.perf_counter()
    steps = 0
    while steps < max_steps:
        for _ in range(S):
            pos, vel, _ = oracle.substep_f32(p, pos, vel, dt, nthreads=th, debug=False)
        steps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    el = time.perf_counter() - t0
    return n * steps / el, steps, el, th


def time_render(sim, sc, stream, warmup, width=1920, height=1080, frames=10):
    """Headless render (sph_render) of the scene's last state at 1080p from a
    camera that sees the whole box: device ms per frame (splat + resolve,
    CUDA events on the library's stream) and ms per frame with the RGBA8 and
    depth images read back to host memory."""
    import torch

    from fluidsim import render
    hx, hy, hz = (0.5 * b for b in sc["params"].bound)
    v = render.view((0.9 * hx, 1.1 * hy, 1.9 * hz), (-0.2 * hx, -0.6 * hy, -0.2 * hz),
                    width, height)
    lib, h, st = sim._lib, sim.handle, sim._stream
    vref = ctypes.byref(v)
    for _ in range(max(warmup, 1)):
        if lib.sph_render(h, vref, None, None, st) != 0:
            raise RuntimeError("render failed")
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(frames):
        lib.sph_render(h, vref, None, None, st)
    e1.record(stream)
    torch.cuda.synchronize()
    dev_ms = e0.elapsed_time(e1) / frames
    rgba = torch.empty((height, width, 4), dtype=torch.uint8, pin_memory=True).numpy()
    depth = torch.empty((height, width), dtype=torch.float32, pin_memory=True).numpy()
    t0 = time.perf_counter()
    for _ in range(frames):
        lib.sph_render(h, vref, rgba.ctypes.data, depth.ctypes.data, st)
    host_ms = (time.perf_counter() - t0) * 1000.0 / frames
    n = sc["pos"].shape[0]
    return {"width": width, "height": height, "particles": n,
            "ms_per_frame": dev_ms, "frames_per_s": 1000.0 / dev_ms,
            "ms_per_frame_with_readback": host_ms,
            "covered_frac": float((depth < 1.0).mean()),
            "readback_bytes": 8 * width * height,
            "timing": "device: CUDA events around the frames on the library's stream; "
                      "with readback: wall clock, RGBA8 + depth copied to pinned memory"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    sc = load_workload(args.workload)
    n = sc["pos"].shape[0]
    import oracle
    oracle.build()
    th = oracle.hw_threads()
    # W untimed steps from the scene, then K timed ones: the part of the flow
    # the GPU arm times
    rate, steps, el, th = cpu_port_rate(sc, args.steps, budget_s=150.0, threads=th,
                                        warm_steps=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "steps_timed": steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * el / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded dam-break lattice)",
        "config": {"workload": args.workload, "particles": n,
                   "substeps": sc["substeps"], "dt": sc["dt"]},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": th, "kind": "port",
                         "sample": f"{steps} full steps ({steps * sc['substeps']} "
                                   f"substeps) of the {n}-particle scene after "
                                   f"{args.warmup} untimed ones, Jacobi restatement "
                                   f"of physicsWorld.cc:39-111 on {th} threads"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_native(args):
    import torch
    import torch.distributed as tdist

    import build_lib
    import fluidsim

    rank, world, local = dist_env()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device (no CPU fallback)")
    torch.cuda.set_device(local)
    if world > 1:
        tdist.init_process_group("nccl", device_id=torch.device("cuda", local))
    if not fluidsim.LIB_PATH.exists():
        build_lib.build()
    sc = load_workload(args.workload)
    n = sc["pos"].shape[0]
    S = sc["substeps"]
    dt = float(sc["dt"])
    stream = torch.cuda.current_stream()
    sim = fluidsim.FluidSimulation(sc["params"], stream=stream)
    sim.InitializeData(n, sc["pos"], sc["vel"])
    tuning = None
    if not args.no_autotune:
        tuning, tuned_ms = sim.autotune(dt, S, steps_per_trial=2)
        sim.upload(sc["pos"], sc["vel"])  # timed steps start from the scene

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed_pass(profiled):
        """K steps, L2 flushed before each, CUDA events around each step on
        the library's stream. With `profiled` the library also records
        events between its kernel phases (phase_times); those event nodes
        drain the GPU between kernels (about 4% of a step), so the headline
        pass runs without them and a second pass of the same steps supplies
        the per-kernel times. Both passes start from the scene's initial
        state, so they time the same (deterministic) trajectory: the flow
        changes the neighbour counts, and with them every kernel's cost."""
        sim.profile_enable(profiled)
        sim.upload(sc["pos"], sc["vel"])
        for _ in range(args.warmup):
            sim.step_async(dt, S)
        torch.cuda.synchronize()
        ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        phase = np.zeros(6)
        launches0 = sim.kernel_launches()
        if world > 1:
            tdist.barrier()
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.zero_()  # L2 flush between timed steps (outside the events)
            ev0[k].record(stream)
            sim.step_async(dt, S)
            ev1[k].record(stream)
            if profiled:
                phase += np.array(sim.phase_times())
        torch.cuda.synchronize()
        if world > 1:
            tdist.barrier()
        wall = time.perf_counter() - wall0
        launches = sim.kernel_launches() - launches0
        total_ms = float(sum(a.elapsed_time(b) for a, b in zip(ev0, ev1)))
        return total_ms, wall, launches, phase

    # clocks over the GPU work of the timed, profiled and end-to-end passes
    # (the timed pass alone is shorter than one sampling interval)
    clocks = ClockSampler(local, interval_ms=20)
    clocks.start(wait_live=True)
    rank_ms, wall, launches, _ = timed_pass(False)
    value, total_ms = replica_throughput(n, args.steps, rank_ms, world, "cuda")
    prof_ms, _, _, phase = timed_pass(True)
    prof_ms = max_over_ranks(prof_ms, world, "cuda")
    sim.profile_enable(False)
    assert sim.status() == 0, "device status flags raised"

    # --- e2e through the public API with the state in pinned host memory
    e2e_steps = args.e2e_steps or args.steps
    pos_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    vel_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    pos_h[:] = sc["pos"]
    vel_h[:] = sc["vel"]
    dens_h = None

    def e2e_step():
        sim.upload(pos_h, vel_h)
        sim.step_async(dt, S)
        if sim._lib.sph_download(sim.handle, pos_h.ctypes.data, vel_h.ctypes.data,
                                 dens_h, sim._stream) != 0:
            raise RuntimeError("download failed")

    # The same trajectory as the timed passes: W warm-up steps from the
    # scene, then K timed steps (the flow changes the neighbour counts, and
    # with them every kernel's cost: the first steps from the lattice run
    # about 10% slower than later ones). The L2 is flushed before each timed
    # step, outside its timing; each step ends with the download's
    # synchronisation.
    for _ in range(args.warmup):  # also the first touches of the pinned buffers
        e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        tdist.barrier()
    e2e_local = 0.0
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        torch.cuda.synchronize()
        e2e_local += time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_local, world, "cuda")
    e2e_value = world * n * e2e_steps / e2e_s
    clk = clocks.stop()
    if clk:
        clk["window"] = ("20 ms samples over the timed, profiled and end-to-end "
                         "passes (warm-up steps included)")
    render_block = time_render(sim, sc, stream, args.warmup)
    sim_tuning = sim.tuning()
    sim.close()

    if rank != 0:
        if world > 1:
            tdist.destroy_process_group()
        return 0

    # roofline of the dominant kernel (per launch, from live CUDA events)
    names = ["predict_hash", "spatial", "density", "pressure", "viscosity"]
    launches_per_phase = {"predict_hash": args.steps, "spatial": args.steps * S,
                          "density": args.steps * S, "pressure": args.steps * S,
                          "viscosity": args.steps * S}
    per_launch_ms = {nm: phase[i] / launches_per_phase[nm] for i, nm in enumerate(names)}
    share = {nm: phase[i] / max(phase[:5].sum(), 1e-12) for i, nm in enumerate(names)}
    dom = max(["density", "pressure", "viscosity"], key=lambda k: per_launch_ms[k])
    peak, peak_kind = peaks()
    grid, entries = fluidsim.simulation.key_table(sc["params"], n, sim_tuning["table"])
    alg = dict(ALG_BYTES, spatial=spatial_bytes(grid, entries, n))
    achieved = alg[dom] * n / (per_launch_ms[dom] / 1000.0) / 1e9
    tr = ncu_traffic(args.workload, dom)
    # every phase against the same peak: the sort (scan, scatter, reorder,
    # cell table), density and the two force kernels; the prediction is
    # fused into the viscosity kernel while it is carried between steps
    phase_roofline = {}
    for nm in ["spatial", "density", "pressure", "viscosity"]:
        ach = alg[nm] * n / (per_launch_ms[nm] / 1000.0) / 1e9
        parts = {"spatial": ["reorder"] + ([] if grid else ["cell_table"])}.get(nm, [nm])
        tp = [ncu_traffic(args.workload, k) for k in parts]
        phase_roofline[nm] = {
            "ms_per_launch": per_launch_ms[nm], "alg_bytes_per_particle": alg[nm],
            "achieved_GBps": ach, "frac": ach / peak,
            "dram_bytes_per_particle": (sum(tp) if all(x is not None for x in tp) else None),
            "dram_bytes_of": "+".join(parts)}
    ms_step = total_ms / args.steps
    sub_ms = ms_step / S
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded dam-break lattice, no dataset)",
        "config": {"workload": args.workload, "particles": n, "substeps": S,
                   "dt": dt, "parallelism": f"replicas{world}" if world > 1 else "single",
                   "l2": "flushed (256 MiB write) before every timed step",
                   "tuning": tuning or sim_tuning,
                   "key_table": {"form": "grid" if grid else "buckets", "entries": entries}},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_kind,
                     "alg_bytes_per_particle": alg[dom],
                     "traffic": (tr * n if tr is not None else None),
                     "timing": "CUDA events around each kernel phase on the "
                               "library's stream, over a second pass of the "
                               "same steps (profiled_ms_per_step)",
                     "issue": ncu_issue(args.workload, dom)},
        "profiled_ms_per_step": prof_ms / args.steps,
        "substep": {"ms": sub_ms,
                    "alg_GBps_at_300B": SUBSTEP_ALG_BYTES * n / (sub_ms / 1000) / 1e9,
                    "frac_at_300B": SUBSTEP_ALG_BYTES * n / (sub_ms / 1000) / 1e9 / peak,
                    "phase_ms_per_launch": per_launch_ms, "phase_share": share,
                    "phase_roofline": phase_roofline},
        "e2e": {"value": e2e_value, "unit": UNIT, "steps": e2e_steps,
                "warmup": args.warmup,
                "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 24 * n,
                "timing": "host wall clock around each sph_upload + sph_step + sph_download "
                          "from pinned host buffers (the download synchronises), summed "
                          "over the timed steps; the same trajectory as the timed passes "
                          "(W warm-up steps from the scene, then K steps); L2 flushed before "
                          "each step, outside its timing"},
        "wall_s": wall,
        "render": render_block,
    }
    if clk:
        line["clocks"] = clk
    try:
        cand, nbrs = pair_stats(sc)
        substeps_s = n * S * args.steps / (total_ms / 1000.0) / world  # per rank
        flops = FLOPS_PER_CANDIDATE * cand + FLOPS_PER_NEIGHBOUR * nbrs
        peak32 = nominal_fp32_tflops(local)
        line["pairs"] = {
            "candidates_per_particle": cand, "neighbours_per_particle": nbrs,
            "measured_on": "4096 particles of the initial state",
            "pair_tests_per_s": world * substeps_s * (cand + 2 * nbrs),
            "fp32_flops_per_particle_substep": flops,
            "fp32_tflops": world * substeps_s * flops / 1e12,
            "fp32_frac": substeps_s * flops / 1e12 / peak32,
            "fp32_peak_tflops": peak32, "fp32_peak_source": "nominal (SMs x 128 x 2 x max clock)"}
    except Exception as e:  # scipy missing: leave the block out
        print(f"pair statistics skipped: {e}", file=sys.stderr)
    if not args.no_cpu_baseline and world == 1:
        rate, steps, el, th = cpu_port_rate(sc, max_steps=16, budget_s=12.0,
                                            warm_steps=args.warmup)  # ~10-15 s
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": th, "kind": "port",
            "sample": f"{steps} full steps of the {n}-particle scene after "
                      f"{args.warmup} untimed ones ({steps * S} substeps), "
                      f"{el:.1f} s on {th} threads"}
    if world == 1 and not args.no_batched:
        # config 2, one GPU's form (each block samples its own clocks); a
        # block that fails is reported in the line, which is still printed
        ck = ClockSampler(local)
        ck.start()
        try:
            line["batched"] = batched_block(args, stream)
        except Exception as e:  # noqa: BLE001 -- reported, not hidden
            line["batched"] = {"error": f"{type(e).__name__}: {e}"}
        line["batched"]["clocks"] = ck.stop()
    if world == 1 and not args.no_served:
        ck = ClockSampler(local)
        ck.start()
        try:
            line["served"] = served_block(args)
        except Exception as e:  # noqa: BLE001 -- reported, not hidden
            line["served"] = {"error": f"{type(e).__name__}: {e}"}
        line["served"]["clocks"] = ck.stop()
    print(json.dumps(line), flush=True)
    if world > 1:
        tdist.destroy_process_group()
    return 0


def batched_block(args, stream):
    """Config 2: 256 independent scenes (n log-uniform in [4096, 131072], box
    aspect U[0.5,2], 20-60% fill, dt 1/60 in 3 substeps) advanced by one set
    of segmented launches per substep (a captured graph per step), against
    the same scenes stepped back to back as separate single-scene handles on
    the same stream. Both time the same K steps from the scenes' initial
    states, L2 flushed before each timed step."""
    import torch

    import fluidsim
    from fluidsim import scenes

    scs = scenes.batched_scenes(256)
    total = sum(s["pos"].shape[0] for s in scs)
    steps = args.steps
    b = fluidsim.Batch(total, 512, stream=stream)
    for s in scs:
        b.add(s["params"], s["pos"], s["vel"], s["dt"])
    tuning, tuned_ms = b.autotune(3, steps_per_trial=1)
    for _ in range(args.warmup):
        b.step(3)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    e0 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    e1 = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    launches0 = b.kernel_launches()
    torch.cuda.synchronize()
    for k in range(steps):
        flush.zero_()
        e0[k].record(stream)
        b.step(3)
        e1[k].record(stream)
    torch.cuda.synchronize()
    bt = sum(a.elapsed_time(c) for a, c in zip(e0, e1)) / 1000.0
    launches = b.kernel_launches() - launches0
    b.close()
    # back-to-back plain launches of the same scenes
    sims = []
    for s in scs:
        sim = fluidsim.FluidSimulation(s["params"], stream=stream)
        sim.InitializeData(s["pos"].shape[0], s["pos"], s["vel"])
        sim.set_tuning(**tuning)
        sims.append(sim)
    for _ in range(args.warmup):
        for sim, s in zip(sims, scs):
            sim.step_async(s["dt"], 3)
    torch.cuda.synchronize()
    for k in range(steps):
        flush.zero_()
        e0[k].record(stream)
        for sim, s in zip(sims, scs):
            sim.step_async(s["dt"], 3)
        e1[k].record(stream)
    torch.cuda.synchronize()
    pt = sum(a.elapsed_time(c) for a, c in zip(e0, e1)) / 1000.0
    for sim in sims:
        sim.close()
    del flush
    value = total * steps / bt
    plain = total * steps / pt
    return {
        "workload": "batched_256", "scenes": len(scs), "particles": total,
        "substeps": 3, "steps": steps, "warmup": args.warmup,
        "value": value, "unit": UNIT, "ms_per_step": 1000 * bt / steps,
        "gpu_launches": int(launches), "tuning": tuning, "autotune_ms": tuned_ms,
        "plain_back_to_back": {"value": plain, "ms_per_step": 1000 * pt / steps},
        "batched_over_plain": value / plain,
        "l2": "flushed (256 MiB write) before every timed step",
        "timing": "CUDA events around each step on the library's stream"}


def served_requests(seconds, rate=200.0, seed=3):
    """The request stream of config 3: Poisson arrivals at `rate` per second
    for `seconds`; each request is (rid, arrival, seed of its scene). The
    scene (fluidsim.scenes.request_scene: n log-uniform in [8192, 524288], K
    uniform in [60, 600], dam break or falling block) is built from its seed
    when it is needed, so the stream's ~12,000 requests are not held in host
    memory at once."""
    rng = np.random.default_rng(seed)
    out, t = [], 0.0
    while True:
        t += rng.exponential(1.0 / rate)
        if t > seconds:
            return out
        out.append((len(out), t, int(rng.integers(1 << 62))))


def request_of(desc):
    from fluidsim import scenes
    rid, arrival, seed = desc
    sc = scenes.request_scene(np.random.default_rng(seed))
    return rid, arrival, sc


def served_block(args, budget=64 << 30, rate=200.0, server_queue=8):
    """Config 3: the Poisson stream (200 req/s for --serve-seconds) through
    the library's own serving loop (sph_server_*: continuous batching on a
    worker thread, admission by the 64 GiB HBM budget). The client submits
    each request once it has arrived and while the server holds fewer than
    `server_queue` jobs waiting for admission (the rest wait, as built scenes
    or not yet built, in arrival order), and collects finished jobs as they
    complete. The measurement window is the stream itself: when its last
    arrival time has passed, the server's statistics are read (particle-steps
    run, per-step latency p50/p99 as the jobs saw it) and the jobs still
    queued or resident are cancelled -- at 200 req/s the stream offers about
    six times what one GPU serves, so a backlog remains, and it is reported.
    The serial baseline runs the stream's first --serial-sample requests one
    after another, each alone on its own single-scene handle (K steps)."""
    import concurrent.futures as cf
    import ctypes
    import collections

    from fluidsim import server

    descs = served_requests(args.serve_seconds, rate)
    srv = server.NativeServer(budget, max_scenes=8192, substeps=3)
    lib, h = srv._lib, srv._h
    pool = cf.ThreadPoolExecutor(4)
    ahead = collections.deque()
    nxt = 0
    live = {}  # job -> (rid, n, K, arrival)
    done_lat, done_work = [], 0
    submitted = 0
    t0 = time.perf_counter()
    last_poll = 0.0
    while True:
        now = time.perf_counter() - t0
        if now >= args.serve_seconds:
            break
        while len(ahead) < 32 and nxt < len(descs):
            ahead.append(pool.submit(request_of, descs[nxt]))
            nxt += 1
        busy = False
        if ahead and descs[submitted][1] <= now and srv.stats()["queued"] < server_queue:
            rid, arrival, sc = ahead.popleft().result()
            job = srv.submit(sc["params"], sc["pos"], sc["vel"], sc["dt"], sc["steps"])
            live[job] = (rid, sc["pos"].shape[0], sc["steps"], arrival)
            submitted += 1
            busy = True
        if now - last_poll > 0.05:
            last_poll = now
            for job in list(live):
                if lib.sph_server_wait(h, job, None, None, None, ctypes.c_double(0.0)) == 0:
                    rid, n, k, arrival = live.pop(job)
                    done_lat.append(time.perf_counter() - t0 - arrival)
                    done_work += n * k
        if not busy:
            time.sleep(0.001)
    st = srv.stats()
    for job in list(live):
        srv.cancel(job)
    srv.close()
    pool.shutdown(wait=True, cancel_futures=True)
    # offered load of the whole stream (n * K of every request)
    from fluidsim import scenes
    offered = sum(n * k for n, k in (scenes.request_size(np.random.default_rng(d[2]))
                                     for d in descs)) / args.serve_seconds
    # serial plain launches of the stream's first requests
    t1 = time.perf_counter()
    work = 0
    for d in descs[: args.serial_sample]:
        _, _, sc = request_of(d)
        req = server.Request(d[0], sc["params"], sc["pos"], sc["vel"], sc["dt"],
                             sc["substeps"], sc["steps"])
        server.run_alone(req)
        work += req.n * req.steps
    serial_s = time.perf_counter() - t1
    serial = work / serial_s
    lat = np.asarray(done_lat) if done_lat else np.zeros(1)
    rate_served = st["particle_steps_per_s"]
    return {
        "workload": "served", "rate_per_s": rate, "seconds": args.serve_seconds,
        "requests_arrived": len(descs), "requests_submitted": submitted,
        "requests_completed": len(done_lat), "requests_cancelled_at_end": len(live),
        "budget_bytes": budget, "capacity_particles": st["capacity_particles"],
        "server": "sph_server (native loop on a worker thread), substeps 3",
        "value": rate_served, "unit": UNIT, "offered_particle_steps_per_s": offered,
        "p50_step_ms": st["p50_step_ms"], "p99_step_ms": st["p99_step_ms"],
        "batched_steps": st["steps"], "particle_steps": st["particle_steps"],
        "wall_s": st["wall_s"],
        "worker_s": {"in_steps": st["step_s"], "admitting": st["admit_s"],
                     "retiring": st["retire_s"],
                     "note": "admission staging overlaps the step it follows"},
        "completion_s_p50": float(np.percentile(lat, 50)),
        "completion_s_p99": float(np.percentile(lat, 99)),
        "serial_plain": {"value": serial, "sample_requests": args.serial_sample,
                         "seconds": serial_s,
                         "how": "each request alone on its own single-scene handle, "
                                "K steps, one after another"},
        "served_over_serial": rate_served / serial,
        "timing": "wall clock: the server's first admission to the end of its last "
                  "step inside the window (sph_server_get_stats)"}


def run_batched(args):
    """--workload batched_256: the batched block alone, as its own line."""
    import torch

    rank, _, local = dist_env()
    if rank != 0:  # one GPU's form: under torchrun rank 0 alone runs it
        return 0
    torch.cuda.set_device(local)
    blk = batched_block(args, torch.cuda.current_stream())
    print(json.dumps({
        "metric": METRIC, "value": blk["value"], "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": blk["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded scenes)",
        "config": {"workload": "batched_256", "scenes": blk["scenes"],
                   "particles": blk["particles"], "substeps": 3,
                   "tuning": blk["tuning"], "l2": blk["l2"]},
        "gpu_launches": blk["gpu_launches"], "batched": blk}), flush=True)
    return 0


def run_served(args):
    """--workload served: the served block alone, as its own line."""
    import torch

    rank, _, local = dist_env()
    if rank != 0:  # one GPU's form: under torchrun rank 0 alone runs it
        return 0
    torch.cuda.set_device(local)
    blk = served_block(args)
    print(json.dumps({
        "metric": METRIC, "value": blk["value"], "unit": UNIT,
        "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded request stream)",
        "config": {"workload": "served", "rate_per_s": blk["rate_per_s"],
                   "seconds": blk["seconds"], "budget_bytes": blk["budget_bytes"]},
        "p50_step_ms": blk["p50_step_ms"], "p99_step_ms": blk["p99_step_ms"],
        "served": blk}), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched_256":
        return run_batched(args)
    if args.workload == "served":
        return run_served(args)
    return run_native(args)


if __name__ == "__main__":
    sys.exit(main())

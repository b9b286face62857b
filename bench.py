#!/usr/bin/env python
"""Benchmark of the GB300 FDTD engine on the benchmark scenes.

Default workload: the 3-D dielectric + CPML scene on a 256^3 grid (24 seeded
spheres/blocks, eps in [1, 12], 10-cell CPML, Bandpass Ex point source),
FP64.  One benchmark step = one full FDTD time step (E and H half-steps) of
the whole grid.  Prints ONE JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload cube|dispersive|air2d] [--n 256] [--precision fp64]

Multi-GPU (torchrun, one process per GPU): the grid does not split across
GPUs in this engine, so every rank advances its own replica of the scene
(weak scaling); value = cells * steps summed over ranks / max rank time.

``--impl reference`` times the CPU oracle (a C restatement of the
reference's OpenMP per-point update loop, oracle/gmes_oracle.c) on the host
cores, on the same scene: the reference's own build (Cython + SWIG) cannot
be built on the GPU host.
"""

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Gcell-updates/s & HBM GB/s vs 8 TB/s; batched p50/p99 job latency"
UNIT = "Gcell-updates/s"


def parse():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", choices=("cube", "dispersive", "air2d", "serving", "design2d"),
                    default="cube")
    ap.add_argument("--batch", type=int, default=64, help="design2d: designs per gradient call")
    ap.add_argument("--block-steps", type=int, default=0,
                    help="design2d, fp32: steps per kernel launch (0: temporally blocked "
                         "default, 1: one step per launch)")
    ap.add_argument("--segment", type=int, default=0,
                    help="design2d: √N-checkpoint segment length (0: record the history "
                         "in the forward when it fits, else ceil(sqrt(steps)))")
    ap.add_argument("--jobs", type=int, default=64, help="serving: number of jobs")
    ap.add_argument("--rate", type=float, default=0.0,
                    help="serving: Poisson arrival rate in jobs/s (0: all at t = 0)")
    ap.add_argument("--max-job-steps", type=int, default=5000)
    ap.add_argument("--size-scale", type=float, default=1.0)
    ap.add_argument("--no-bound", action="store_true",
                    help="serving: skip the measured batching bound")
    ap.add_argument("--no-serving", action="store_true",
                    help="default run: skip the bounded serving sample")
    ap.add_argument("--serving-jobs", type=int, default=24,
                    help="default run: jobs of the bounded serving sample")
    ap.add_argument("--n", type=int, default=None, help="grid side (cube 256, dispersive 192)")
    ap.add_argument("--precision", default="fp64",
                    choices=("fp64", "df64", "fp32", "fp64_strict"))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0,
                    help="target length of the CPU-baseline sample")
    ap.add_argument("--quiet-extras", action="store_true",
                    help="only the timed loop (for profiling runs)")
    return ap.parse_args()


def build_sim(args, precision):
    from gmes_gb300 import workloads as W
    if args.workload == "cube":
        n = args.n or 256
        sim, full_steps = W.cube(n=n, precision=precision)
        cfg = {"workload": f"cube{n}_dielectric_cpml", "grid": [n, n, n], "objects": 24,
               "pml_cells": 10, "source": "Bandpass(0.5, 0.2) Ex point", "job_steps": full_steps}
    elif args.workload == "dispersive":
        n = args.n or 192
        sim, full_steps = W.dispersive(n=n, precision=precision)
        cfg = {"workload": f"cube{n}_drude_lorentz_dcp_upml", "grid": [n, n, n],
               "pml_cells": 12,
               "source": "TFSF plane wave +z, x-polarised, Bandpass(0.5, 0.2), box 90% of the "
                         "PML-free interior",
               "courant_ratio": 0.6, "job_steps": full_steps}
    else:
        sim, full_steps = W.air2d(precision=precision)
        cfg = {"workload": "air2d_tmz_200x200_cpml", "grid": [200, 200, 1],
               "source": "Continuous(0.8) Ez point", "job_steps": full_steps}
    return sim, cfg


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "of measured"
        except (KeyError, ValueError):
            pass
    return 6800.0, "of fallback"


def _profile_entry(name, workload_key, precision, side):
    """An entry of a committed ncu summary: the H half-step's own entry
    (key suffix /H) when the H half is the dominant kernel and has one,
    else the workload's entry (the E half-step)."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    try:
        data = json.loads(p.read_text())
    except ValueError:
        return None
    key = f"{workload_key}/{precision}"
    if side == "H" and f"{key}/H" in data:
        return data[f"{key}/H"]
    return data.get(key)


def ncu_traffic(workload_key, precision, side="E"):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary."""
    return _profile_entry("traffic.json", workload_key, precision, side)


def ncu_pipe(workload_key, precision, side="E"):
    """The busiest execution pipe of the dominant kernel (committed ncu summary).

    Where a kernel is bound by an arithmetic pipe rather than by DRAM (the
    FP64 cell kernel: FP64 pipe), this says which pipe and how busy it was.
    """
    return _profile_entry("pipes.json", workload_key, precision, side)


def fp64_pipe_ceiling(workload_key, precision, value, clocks):
    """The FP64 pipe's bound on the step rate, beside the HBM roofline.

    GB300 issues one FP64 warp-instruction per 16 SM cycles (1.0 TFLOP/s
    FP64 FMA measured: 2 lanes per clock per SM), so with n FP64
    instructions per cell and half-step (committed ncu count, both halves)
    the step rate cannot pass SMs x clock / 16 x 32 / (2 n) cells per second.
    """
    if precision not in ("fp64",):
        return None
    e = ncu_pipe(workload_key, precision, "E")
    if not e or "fp64_inst_per_cell" not in e:
        return None
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    per_step = 2 * float(e["fp64_inst_per_cell"])
    ceiling = sms * mhz * 1e6 / 16 * 32 / per_step / 1e9
    return {"ceiling_gcells": round(ceiling, 3), "fraction_of_ceiling": round(value / ceiling, 4),
            "fp64_inst_per_cell_step": per_step, "sms": sms, "sm_mhz": mhz,
            "note": "the FP64 step is bound by the FP64 pipe, not HBM; roofline.frac stays "
                    "the HBM fraction"}


# ---------------------------------------------------------------------------
# algorithmic bytes
# ---------------------------------------------------------------------------
def half_bytes(scene, precision, engine=None):
    """Algorithmic DRAM bytes of each half-step: (E half, H half).

    E half: read+write every E value, read every H value, read the E class
    ids, read+write the E state slots of the points that carry state
    (CPML psi, UPML d, ADE q/p).  H half symmetric.
    """
    from gmes_gb300.scene import naux_of
    es = 4 if precision == "fp32" else 8
    out = []
    for side in (0, 1):
        b = 0
        for comp in scene.active:
            c = comp.index
            npts = int(np.prod(scene.shape(c)))
            if (c < 3) == (side == 0):
                b += 2 * es * npts + npts
                counts = engine.class_counts(c) if engine is not None else scene.counts(c)
                for cid, cnt in counts.items():
                    b += 2 * naux_of(scene.classes[c][cid]) * es * cnt
            else:
                b += es * npts
        out.append(b)
    return out


# ---------------------------------------------------------------------------
# our engine
# ---------------------------------------------------------------------------
def timed_loop(sim, steps, warmup, rank_sync):
    import torch
    with torch.cuda.stream(sim.engine.torch_stream):
        return _timed_loop(sim, steps, warmup, rank_sync)


def _timed_loop(sim, steps, warmup, rank_sync, split_steps=50):
    """Time ``steps`` FDTD steps as the engine runs them: chunks of up to
    src_chunk steps, each replayed as one CUDA graph of its launches, with
    the next chunk's source values staged (host evaluation + pinned copy on
    the same stream) while the previous chunk runs.  Returns (device ms of
    the timed region, E half ms, H half ms, wall s).

    The E / H split the roofline needs comes from a second timed pass of
    ``split_steps`` steps launched half-step by half-step with CUDA events
    between them; each half there includes its ghost-copy and source
    kernels and the launch gaps, so the kernel times (and the roofline
    fraction) it gives are upper (lower) bounds.
    """
    import torch
    eng = sim.engine
    chunk = eng.src_chunk
    sizes = {min(chunk, steps - s) for s in range(0, steps, chunk)}
    # warm-up (untimed): the same chunked graph replay
    done = 0
    while done < warmup:
        k = min(chunk, warmup - done)
        eng.stage_sources(float(done), k)
        eng.launch_raw(k)
        done += k
    for k in sizes:  # capture every chunk length the timed region replays
        eng._graph(k)
    torch.cuda.synchronize()
    base = float(warmup)
    # stage the first chunk of source values before the clock starts
    eng.stage_sources(base, min(chunk, steps))
    torch.cuda.synchronize()
    rank_sync()
    torch.cuda.synchronize()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    t_start.record()
    s = 0
    while s < steps:
        k = min(chunk, steps - s)
        if s > 0:
            eng.stage_sources(base + s, k)
        eng.launch_raw(k)
        s += k
    t_end.record()
    torch.cuda.synchronize()
    rank_sync()
    wall = time.perf_counter() - t0
    total_ms = t_start.elapsed_time(t_end)
    # E / H split, half-step by half-step
    n = max(1, min(split_steps, chunk))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    eng.stage_sources(base + steps, n)
    torch.cuda.synchronize()
    for q in range(n):
        a, b, c = ev[q]
        a.record()
        eng.half_step(0, q)
        b.record()
        eng.half_step(1, q)
        c.record()
    torch.cuda.synchronize()
    e_ms = sum(a.elapsed_time(b) for a, b, _ in ev) / n
    h_ms = sum(b.elapsed_time(c) for _, b, c in ev) / n
    return total_ms, e_ms, h_ms, wall


def e2e_loop(sim, steps):
    """Same metric through the public API: sim.step() per step (host source
    evaluation + pinned H2D copy of the step's source values) and a D2H read
    of the probe value at the source point each step.  Each step's value is
    copied to pinned memory right after the step and read on the host one
    step later (two pinned buffers, an event each), so the host never waits
    for a step it has not yet launched past."""
    import torch
    scene = sim.scene
    src = scene.sources[0] if scene.sources else None
    c = src.comp.index if src else scene.active[0].index
    idx = src.idx if src else (0, 0, 0)
    field = sim.engine.fields[c]
    probes = [torch.empty((1,) + tuple(field.shape[3:]), dtype=field.dtype).pin_memory()
              for _ in range(2)]
    events = [torch.cuda.Event(), torch.cuda.Event()]
    # a view of the probed point, made once: each step copies its current value
    point = field[idx].reshape(probes[0].shape)
    for _ in range(3):
        sim.step()
    torch.cuda.synchronize()
    values = []
    t0 = time.perf_counter()
    for s in range(steps):
        sim.step()
        cur = torch.cuda.current_stream()
        probes[s % 2].copy_(point, non_blocking=True)
        events[s % 2].record(cur)
        if s > 0:
            events[(s - 1) % 2].synchronize()
            values.append(float(probes[(s - 1) % 2].reshape(-1)[0]))
    events[(steps - 1) % 2].synchronize()
    values.append(float(probes[(steps - 1) % 2].reshape(-1)[0]))
    wall = time.perf_counter() - t0
    assert len(values) == steps
    h2d = 2 * len(scene.sources) * 8
    d2h = probes[0].numel() * probes[0].element_size()
    return wall, h2d, d2h


def cpu_baseline(sim, seconds, threads=None):
    """Time the CPU oracle on a bounded number of steps of the same scene."""
    from oracle.oracle import Oracle
    t0 = time.perf_counter()
    orc = Oracle(sim.scene)
    setup = time.perf_counter() - t0
    t1 = time.perf_counter()
    orc.step(1)
    one = time.perf_counter() - t1
    nsteps = max(1, min(200, int(seconds / max(one, 1e-6))))
    t2 = time.perf_counter()
    orc.step(nsteps)
    dt = time.perf_counter() - t2
    cells = sim.scene.cells
    return {"value": cells * nsteps / dt / 1e9, "unit": UNIT, "cores": Oracle.threads(),
            "kind": "port",
            "sample": (f"{nsteps} FDTD steps of the same scene after 1 warm-up step "
                       f"(point-list setup {setup:.1f}s excluded), C oracle with OpenMP "
                       f"static loops, {Oracle.threads()} threads")}, nsteps, dt


def replica_throughput(total_ms, cells, steps, dist=None, device="cpu"):
    """(job time in ms, whole-job Gcell-updates/s) of N independent replicas.

    Every rank advanced its own ``cells``-cell grid ``steps`` steps in
    ``total_ms``; the job takes as long as the slowest rank (max over ranks)
    and its throughput counts the cell-updates of all ranks.
    """
    world = 1
    if dist is not None:
        import torch
        world = dist.get_world_size()
        t = torch.tensor([float(total_ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, cells * steps * world / (total_ms / 1e3) / 1e9


def run_ours(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def rank_sync():
        if dist is not None:
            dist.barrier()

    sim, cfg = build_sim(args, args.precision)
    sim.init()
    scene = sim.scene
    cells = scene.cells
    clk = ClockSampler(local)
    clk.start()
    total_ms, e_ms, h_ms, wall = timed_loop(sim, args.steps, args.warmup, rank_sync)
    clocks = clk.stop()
    total_ms, value = replica_throughput(total_ms, cells, args.steps, dist, "cuda")
    eb, hb = half_bytes(scene, args.precision, sim.engine)
    dom = ("E half-step", eb, e_ms) if e_ms >= h_ms else ("H half-step", hb, h_ms)
    peak, peak_src = measured_peak()
    achieved = dom[1] / (dom[2] / 1e3) / 1e9
    step_bytes = eb + hb
    side = dom[0][0]
    traffic = ncu_traffic(cfg["workload"], args.precision, side)
    result = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp64_strict": "f64", "fp32": "f32",
                  "df64": "df64 (f32 pair)"}[args.precision],
        "data": "synthetic (seeded scene, no dataset)",
        "config": arm_config(cfg, scene, args.precision, world),
        "hbm_gbs_alg": round(step_bytes / (total_ms / args.steps / 1e3) / 1e9, 1),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "kernel": dom[0], "alg_bytes_per_launch": dom[1],
                     "launch_ms": round(dom[2], 5), "peak_source": peak_src,
                     "pipe": ncu_pipe(cfg["workload"], args.precision, side)},
        "half_ms": {"E": round(e_ms, 5), "H": round(h_ms, 5)},
        "timing": (f"{args.steps} steps replayed as CUDA graphs of up to {sim.engine.src_chunk} "
                   "steps (the engine's own path), source values staged per chunk on the same "
                   "stream; half_ms and roofline.launch_ms from 50 further steps launched half "
                   "by half with CUDA events between (each half with its ghost-copy and source "
                   "kernels)"),
        "fp64_pipe": fp64_pipe_ceiling(cfg["workload"], args.precision, value, clocks),
        "gpu_launches": args.steps * (6 if scene.sources else 4),
        "clocks": clocks,
    }
    if rank == 0 and not args.quiet_extras:
        if not args.no_variants and args.precision == "fp64" and world == 1:
            result["variants"] = {}
            del sim
            torch.cuda.empty_cache()
            for prec in ("df64", "fp32"):
                vs, _ = build_sim(args, prec)
                vs.init()
                vk = min(args.steps, 100)
                t_ms, ve, vh, _ = timed_loop(vs, vk, 5, lambda: None)
                veb, vhb = half_bytes(vs.scene, prec, vs.engine)
                vdom = (veb, ve) if ve >= vh else (vhb, vh)
                result["variants"][prec] = {
                    "value": round(cells * vk / (t_ms / 1e3) / 1e9, 4),
                    "ms_per_step": round(t_ms / vk, 5),
                    "roofline_frac": round(vdom[0] / (vdom[1] / 1e3) / 1e9 / peak, 4)}
                del vs
                torch.cuda.empty_cache()
            sim, _ = build_sim(args, args.precision)
            sim.init()
        if not args.no_e2e:
            k = max(1, min(args.steps, 200))
            wall_e2e, h2d, d2h = e2e_loop(sim, k)
            result["e2e"] = {"value": round(cells * k * world / wall_e2e / 1e9, 4), "unit": UNIT,
                             "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                             "api": "FDTD.step() + probe read, host source values (each "
                                    "step's probe read on the host one step later)"}
        if not args.no_cpu_baseline and world == 1:
            cb, _, _ = cpu_baseline(sim, args.cpu_seconds)
            result["cpu_baseline"] = cb
        if not args.no_serving and world == 1 and args.workload == "cube":
            # the metric's third clause: a bounded sample of the config-4
            # serving stream (full-size grids and step counts, fewer jobs)
            del sim
            torch.cuda.empty_cache()
            result["serving"] = serving_compare(args.serving_jobs, 0.0, 5000, 1.0,
                                                args.precision)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(result), flush=True)


def arm_config(cfg, scene, precision, world):
    """The ``config`` object of both arms (ours and --impl reference): the
    workload, precision, replica count, cells and the L2 note."""
    es = {"fp32": 4}.get(precision, 8)
    fields = sum(int(np.prod(scene.shape(c.index))) for c in scene.active) * es
    return dict(cfg, precision=precision, parallelism=f"replicas x{world}", cells=scene.cells,
                l2=f"inputs larger than L2 (fields alone {fields / 1e6:.0f} MB)")


def run_reference(args):
    """CPU reference arm: the oracle port on all host cores, same scene and metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    sim, cfg = build_sim(args, args.precision)
    scene = sim.compile()
    from oracle.oracle import Oracle
    t0 = time.perf_counter()
    orc = Oracle(scene)
    setup = time.perf_counter() - t0
    w = max(0, args.warmup)
    tw = time.perf_counter()
    orc.step(max(1, w))
    per_step = (time.perf_counter() - tw) / max(1, w)
    # the median of R repeats of k steps (benchmarks/field_updates.py:122-156),
    # the whole timed sample bounded to about a minute
    repeats = 5
    k = max(1, min(args.steps, int(60.0 / repeats / max(per_step, 1e-6))))
    times = []
    for _ in range(repeats):
        t1 = time.perf_counter()
        orc.step(k)
        times.append(time.perf_counter() - t1)
    dt = statistics.median(times)
    value = scene.cells * k / dt / 1e9
    result = {
        "metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / k * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp64_strict": "f64", "fp32": "f32",
                  "df64": "df64 (f32 pair)"}[args.precision],
        "data": "synthetic (seeded scene, no dataset)", "impl": "reference",
        "config": arm_config(cfg, scene, args.precision, world),
        "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": Oracle.threads(),
                         "kind": "port",
                         "sample": (f"median of {repeats} repeats of {k} FP64 steps of the "
                                    f"same scene (the requested {args.steps} steps bounded to "
                                    f"~60 s), after {max(1, w)} warm-up steps; point-list setup "
                                    f"{setup:.1f}s excluded; C oracle, OpenMP static loops")},
        "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(result), flush=True)


def serving_compare(njobs, rate, max_steps, size_scale, precision, bound=True, tuner=True):
    """Batched serving of a seeded config-4 job stream against the same jobs
    one at a time with the plain single-grid kernels, plus the measured
    batching bound (``serving.batching_bound``).  Returns a dict."""
    from gmes_gb300 import workloads as W
    from gmes_gb300.autotune import Tuner
    from gmes_gb300.serving import Job, Server, batching_bound, run_one_at_a_time
    min_steps = min(500, max_steps)
    stream = W.serving_jobs(njobs, seed=0, rate=rate or None, max_steps=max_steps,
                            min_steps=min_steps, size_scale=size_scale, precision=precision)

    def jobs():
        return [Job(arrival=t, jid=i, build=b, nsteps=n) for i, (t, b, n) in enumerate(stream)]

    tn = Tuner() if tuner else None
    server = Server(precision=precision, chunk=64, max_slots=64, tuner=tn)
    rep = server.run(jobs(), realtime=bool(rate))
    base = run_one_at_a_time(jobs(), precision=precision, realtime=bool(rate))
    out = {
        "jobs": njobs, "seed": 0, "rate_per_s": rate,
        "arrivals": f"Poisson, {rate} jobs/s" if rate else "all at t = 0 (saturating)",
        "grids": "2-D TMz 128^2-1024^2 and 3-D 64^3-160^3 (x size_scale "
                 f"{size_scale}), CPML 8-16, dielectric/Drude/Lorentz sphere",
        "job_steps": f"{min_steps}-{max_steps}", "precision": precision, "chunk": 64,
        "batched_gcells": round(rep["gcells_per_s"], 4),
        "latency_p50_s": round(rep["latency_p50_s"], 4),
        "latency_p99_s": round(rep["latency_p99_s"], 4),
        "wall_s": round(rep["wall_s"], 3), "failed": rep["failed"],
        "failed_errors": sorted({(j.error or "")[:60] for j in server.failed})[:4],
        "one_at_a_time_gcells": round(base["gcells_per_s"], 4),
        "one_at_a_time_latency_p50_s": round(base["latency_p50_s"], 4),
        "one_at_a_time_latency_p99_s": round(base["latency_p99_s"], 4),
        "one_at_a_time_wall_s": round(base["wall_s"], 3),
        "speedup": round(rep["gcells_per_s"] / base["gcells_per_s"], 3),
        "cell_updates": rep["cell_updates"], "chunks": rep["chunks"],
        "gpu_launches": rep["launches"],
    }
    if tn is not None:
        out["autotune"] = tn.summary()
    if bound:
        b = batching_bound(jobs(), base["job_s"], precision=precision)
        out["bound"] = round(b["bound"], 3)
        out["bound_detail"] = {
            "one_at_a_time_s": round(b["one_at_a_time_s"], 3),
            "saturated_s": round(b["saturated_s"], 3),
            "definition": "sum of the jobs' one-at-a-time wall times over the sum of their "
                          "steps x saturated step time (copies of the grid filling the GPU "
                          "through the batch: the multi-grid kernel below 2^17 cells, each "
                          "copy's own kernels above; CUDA events)"}
        out["speedup_over_bound"] = round(out["speedup"] / b["bound"], 3)
    return out


def run_serving(args):
    """Batched serving of a seeded job stream vs the same jobs one at a time."""
    clk = ClockSampler(0)
    clk.start()
    cmp = serving_compare(args.jobs, args.rate, args.max_job_steps, args.size_scale,
                          args.precision, bound=not args.no_bound)
    clocks = clk.stop()
    result = {
        "metric": METRIC, "value": cmp["batched_gcells"], "unit": UNIT, "n_gpus": 1,
        "steps": cmp["chunks"], "warmup": 0, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"fp64": "f64", "fp32": "f32", "df64": "df64 (f32 pair)",
                                       "fp64_strict": "f64"}[args.precision],
        "data": "synthetic (seeded job stream)",
        "config": {"workload": "batched_serving", "jobs": args.jobs, "rate_per_s": args.rate,
                   "grids": cmp["grids"], "job_steps": cmp["job_steps"],
                   "precision": args.precision, "chunk": 64, "max_slots": 64},
        "serving": cmp, "clocks": clocks, "gpu_launches": cmp["gpu_launches"],
    }
    print(json.dumps(result), flush=True)


def run_design(args):
    """Gradient of the monitor objective for a batch of TMz designs (512^2, 2000 steps).

    One benchmark step = one forward (J of every design, keeping what the
    backward needs) plus one backward (dJ/deps of every design).  The
    problem records every step's design increments in the forward when they
    fit in memory (the default here: 2.1 GB in FP32), so the backward is the
    adjoint sweep alone; with √N checkpoints (``--segment``) the backward
    also recomputes the forward.  value = cell-updates per second counting
    every forward, recomputed and adjoint step run (2 or 3 x cells x steps x
    designs per benchmark step).
    """
    import torch
    from gmes_gb300 import workloads as W
    from gmes_gb300.adjoint import TMzAdjoint
    precision = args.precision if args.precision != "fp64_strict" else "fp64"
    n = args.n or 512
    space, geom, src, design, monitor, eps, nsteps = W.design2d(n=n, batch=args.batch)
    prob = TMzAdjoint(space, geom, src, design, monitor, nsteps, batch=args.batch,
                      precision=precision, block_steps=args.block_steps,
                      segment=args.segment or None)
    cells = n * n
    x = torch.tensor(eps, dtype=torch.float64, device="cuda")
    for _ in range(max(1, args.warmup)):
        prob.forward(x)
        prob.backward()
    torch.cuda.synchronize()
    st = prob.grid.torch_stream
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    t_fwd, t_bwd = [], []
    clk = ClockSampler(0)
    clk.start()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ev[0].record(st)
        prob.forward(x)
        ev[1].record(st)
        g = prob.backward()
        ev[2].record(st)
        torch.cuda.synchronize()
        t_fwd.append(ev[0].elapsed_time(ev[1]) / 1e3)
        t_bwd.append(ev[1].elapsed_time(ev[2]) / 1e3)
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    tf, tb = statistics.median(t_fwd), statistics.median(t_bwd)
    per = tf + tb
    passes = 2 if prob.keep_history else 3
    upd = passes * cells * nsteps * args.batch
    es = 4 if precision == "fp32" else 8
    # algorithmic bytes per cell-step: E half reads Ez, Hx, Hy and writes Ez;
    # H half reads Ez, Hx, Hy and writes Hx, Hy (the adjoint halves the same
    # on the adjoint fields): 9 values.  CPML psi and the class maps (shared
    # by the batch, L2-resident) are not counted.
    fwd_gbs = 9 * es * cells * nsteps * args.batch / tf / 1e9
    bwd_gbs = (passes - 1) * 9 * es * cells * nsteps * args.batch / tb / 1e9
    peak = measured_peak()
    spl = (args.block_steps or 4) if precision == "fp32" else 1  # steps per forward launch
    fwd_kernel = (f"forward, k_tmz_tb_fwd ({spl} steps per launch)" if spl > 1
                  else "forward, k_tmz_fe + k_tmz_fh")
    result = {
        "metric": METRIC, "value": round(upd / per / 1e9, 4), "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": max(1, args.warmup), "ms_per_step": round(per * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp32": "f32", "df64": "df64 (f32 pair)"}[precision],
        "data": "synthetic (seeded designs)",
        "config": {"workload": f"design2d_tmz_{n}x{n}_adjoint", "grid": [n, n, 1],
                   "design_points": [64, 64], "monitor_points": [8, 8], "time_steps": nsteps,
                   "batch": args.batch,
                   "history": ("forward records every step's design increments "
                               f"({prob.sizes[3] / 1e9:.2f} GB), no backward recompute"
                               if prob.keep_history else
                               f"checkpoints every {prob.segment} steps, backward recompute"),
                   "checkpoint_segment": None if prob.keep_history else prob.segment,
                   "checkpoints": (0 if prob.keep_history
                                   else (nsteps + prob.segment - 1) // prob.segment),
                   "precision": precision, "block_steps": args.block_steps,
                   "l2": "state 7 x batch x n^2 x elem > L2 for batch 64 (inputs larger than L2)"},
        "gradients_per_s": round(args.batch / per, 3),
        "forward_s": round(tf, 6), "backward_s": round(tb, 6),
        "forward_alg_GBps": round(fwd_gbs, 1), "backward_alg_GBps": round(bwd_gbs, 1),
        "hbm_peak_GBps": peak[0] if peak else None,
        # the forward pass against HBM: algorithmic bytes of a one-step
        # kernel (9 values per cell-step) per second; traffic = measured DRAM
        # bytes of one forward launch (ncu), which temporal blocking keeps
        # well below the algorithmic bytes of the steps it advances
        "roofline": {"bound": "hbm", "achieved": round(fwd_gbs, 1), "peak": peak[0],
                     "unit": "GB/s", "frac": round(fwd_gbs / peak[0], 4),
                     "traffic": ncu_traffic(f"design2d_tmz_{n}x{n}_batch{args.batch}_{spl}steps",
                                            precision),
                     "alg_bytes_per_launch": 9 * es * cells * args.batch * spl,
                     "kernel": fwd_kernel, "peak_source": peak[1]},
        "wall_s": round(wall, 3), "grad_finite": bool(torch.isfinite(g).all()),
        "clocks": clocks,
        "gpu_launches": args.steps * (design_launches(prob, precision, args.block_steps) + 2),
    }
    if not args.no_cpu_baseline:
        result["cpu_baseline"] = design_cpu_baseline(space, geom, src, design, monitor, eps,
                                                     prob, n)
    print(json.dumps(result), flush=True)


def design_launches(prob, precision, block_steps, max_block_steps=4):
    """Kernel launches of one forward + backward.

    One step per launch: E, E sources, H, H sources per step of every pass.
    FP32 temporally blocked (block_steps 0 = the library's most, 4): the
    forward takes one launch per block of up to that many steps of each
    call; the adjoint the fewest launches of at most that many steps whose
    count has the parity of the call's steps (the library's adj_launches).
    Passes: forward and adjoint over all steps when the forward records the
    history; forward, recompute and adjoint per checkpoint segment otherwise.
    """
    nsteps, seg = prob.nsteps, prob.segment
    calls = [nsteps] if prob.keep_history else [min(seg, nsteps - s0)
                                                 for s0 in range(0, nsteps, seg)]
    passes = 2 if prob.keep_history else 3
    per = (block_steps or max_block_steps) if precision == "fp32" else 1
    if per == 1:
        return 4 * passes * nsteps

    def adj(k):
        n = (k + per - 1) // per
        if n % 2 != k % 2:
            n += 1
        return min(n, k)
    fwd = sum((k + per - 1) // per for k in calls)
    return fwd * (passes - 1) + sum(adj(k) for k in calls)


def design_cpu_baseline(space, geom, src, design, monitor, eps, prob, n, steps=100):
    """The oracle's FP64 CPU adjoint (serial) on one design, first ``steps`` steps."""
    from oracle.oracle import Oracle
    (d0, dn), (m0, mn) = prob.design_box, prob.monitor_box
    dpts = [(2, (d0[0] + a, d0[1] + b, 0)) for a in range(dn[0]) for b in range(dn[1])]
    mpts = [(2, (m0[0] + a, m0[1] + b, 0)) for a in range(mn[0]) for b in range(mn[1])]
    o = Oracle(prob.scene)
    o.set_eps(2, [p for _, p in dpts], eps[0].reshape(-1))
    t0 = time.perf_counter()
    o.adjoint(steps, mpts, dpts)
    dt = time.perf_counter() - t0
    return {"value": round(2 * n * n * steps / dt / 1e9, 5), "unit": UNIT, "cores": 1,
            "kind": "port",
            "sample": f"oracle FP64 forward + adjoint sweep of 1 design, {steps} steps of "
                      f"{n}x{n} (counts forward + adjoint steps)"}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serving":
        run_serving(args)
    elif args.workload == "design2d":
        run_design(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

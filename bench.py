#!/usr/bin/env python
"""Throughput benchmark of the checkerboard Cellular Potts sweep on GB300.

Metric: copy attempts per second (one attempt per lattice site per MCS).
Default workload: the 4096x4096 2D tissue (Voronoi tiling at 100 sites per
cell, 3 types, symmetric random J, area + perimeter constraints, T=20); one
step is one 500-MCS run of it, continuing from the previous step's state.

  value      device-resident throughput: the lattice and tables live in HBM;
             each step is timed with CUDA events on the launching stream and
             L2 is flushed (512 MB write) between steps, outside the events.
  e2e        the same metric through the public API with host buffers: every
             step pushes the pinned host lattice (H2D + table recount), runs
             500 MCS and pulls the lattice back (D2H).
  roofline   algorithmic bytes = 8 B per attempt (one int32 read and write of
             every site per MCS) / mean sweep-launch time, against the
             measured HBM copy bandwidth.
  cpu_baseline  the C++ oracle (the same deterministic sweep) on the host
             cores, on a bounded sample of the same lattice.

--impl reference times the CPU oracle (the reference has no CPU sweep of its
own; its CUDA build is timed separately) on all host threads, one MCS of the
same lattice per step.

Under torchrun (N>1) every rank runs its own independent replica of the
workload (replicas only: the path has no data exchange between lattices);
time is the max over ranks and value the attempts of all ranks / that time.
"""
import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

ROOT = pathlib.Path(__file__).resolve().parent
PKG = ROOT / "gpu-cpm_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "copy-attempts/s"
UNIT = "attempts/s"
BYTES_PER_ATTEMPT = 8
REFERENCE_RELAX_MCS = 100  # reference arm: MCS run before its timed steps (20 s at most)
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--workload", default="tissue_2d",
                   choices=["tissue_2d", "tissue_2d_8192", "tissue_3d", "sorting_2d",
                            "sorting_2d_256", "ensemble", "sorting_batch", "gradient", "gradient_check"])
    p.add_argument("--replicas", type=int, default=None,
                   help="replicas of --workload ensemble (256) / gradient (512)")
    p.add_argument("--mcs", type=int, default=None, help="MCS per step")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-loop", action="store_true",
                   help="batches: skip timing the per-replica launch loop")
    p.add_argument("--variant", type=int, default=None,
                   help="tile variant instead of the autotuner's choice (profiling runs: "
                        "timing under a profiler can change the tuner's pick)")
    p.add_argument("--fill", choices=["parity", "vector", "tma", "cluster"], default=None,
                   help="single 2D lattices: how tiles are staged instead of the engine's "
                        "default (see cpm_set_fill)")
    p.add_argument("--dispatch", choices=["grid", "replica", "hybrid"], default=None,
                   help="batches: dispatch instead of the autotuner's choice")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-reference-gpu", action="store_true",
                   help="skip timing the reference's own CUDA sweep on this GPU")
    p.add_argument("--no-secondary", action="store_true",
                   help="default workload: skip the compact results of the 256^3 tissue, "
                        "the ragged ensemble and the gradient ensemble")
    p.add_argument("--no-fd", action="store_true",
                   help="gradient workloads: time only (no finite-difference comparison)")
    p.add_argument("--fd-params", default=None,
                   help="gradient workloads: comma-separated parameters to difference "
                        "(default: all of J_ll,J_dd,J_ld,J_lm,J_dm,lambda_area,T)")
    return p.parse_args()


def build_workload(name):
    from gpucpm import workloads as W
    if name == "tissue_2d":
        return W.tissue_2d()
    if name == "tissue_2d_8192":
        return W.tissue_2d(n=8192, mcs=100)
    if name == "tissue_3d":
        return W.tissue_3d()
    if name == "sorting_2d":
        return W.sorting_2d()
    if name == "sorting_2d_256":
        # the same recipe at the reference's own sorting size (a power of two,
        # which its neighbour wrap needs): 655 5x5 cells, the density of 400
        # cells on 200^2
        return W.sorting_2d(n=256, ncells=655)
    raise ValueError(name)


def describe(w, mcs):
    shape = "x".join(str(s) for s in w.lattice.shape[::-1])
    return {"workload": f"{w.name} {shape}", "sites": w.nsites, "cells": w.ncells,
            "types": int(w.J.shape[0]) - 1, "temperature": w.temperature,
            "mcs_per_step": mcs, "neighbourhood": "moore8" if w.ndim == 2 else "moore26",
            "l2": "flushed between steps (512 MB write, outside the timed events)",
            "seed": 0}


def data_of(w):
    if w.name.startswith("tissue"):
        return "synthetic (seeded Voronoi tissue)"
    return "synthetic (seeded 5x5 squares, two-type sorting)"


def measured_peak_hbm():
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100", "-i", str(self.gpu_id)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def gpu_index_for(torch, dev):
    """nvidia-smi id of a torch device (its UUID when torch exposes it)."""
    try:
        u = str(torch.cuda.get_device_properties(dev).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        return vis.split(",")[dev] if vis else dev


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return world, rank, local


def dist_max(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64,
                     device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_baseline(w, target_s=10.0, max_mcs=20):
    """The C++ oracle on every host thread, on a bounded sample of `w`."""
    import oracle
    threads = os.cpu_count() or 1
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=0)
    t0 = time.perf_counter()
    sim.run(1, nthreads=threads)
    first = time.perf_counter() - t0
    extra = max(0, min(max_mcs - 1, int(target_s / max(first, 1e-3)) - 1))
    t1 = time.perf_counter()
    if extra:
        sim.run(extra, nthreads=threads)
    total = first + (time.perf_counter() - t1)
    mcs = 1 + extra
    # one more MCS on one thread: the per-core rate beside the all-core one
    t2 = time.perf_counter()
    sim.run(1, nthreads=1)
    one = time.perf_counter() - t2
    return {"value": w.nsites * mcs / total, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{mcs} MCS of the {'x'.join(map(str, w.lattice.shape[::-1]))} "
                      f"{w.name} lattice from its seeded initial state ({total:.1f} s)",
            "single_thread": {"value": w.nsites / one, "unit": UNIT, "cores": 1,
                              "sample": f"the next MCS on one thread ({one:.2f} s)"}}


# The reference's synchronisation modes (its run() knobs, src/kernels2d.cu:
# 179-195, src/kernels3d.cu:140-156):
#   grid_each     grid sync before every attempt (its examples' setting)
#   grid_region   grid sync after every ppc^2 attempts, each thread finishing
#                 its ppc x ppc sub-square first (updates_per_barrier =
#                 updates_per_checkerboard_switch = ppc^2)
#   block_each    block sync only (its notebook's setting at 2048^2 and above):
#                 blocks drift apart within an MCS, racy
#   none          no sync inside an MCS (its notebook's final run), racy
# Racy modes launch once per MCS (inner_iterations = 1, as the notebook
# does), so that blocks meet at every MCS boundary.  A grid-synced mode is
# race-free only where each thread's ppt x ppt region holds at least two
# sub-squares per axis (ppt / ppc >= 2, src/kernels2d.cu:89-90,179-181):
# then the sub-squares all threads work at once are separated by one of
# another colour.  With ppt = ppc every thread works its whole region at
# once and neighbouring threads' sites touch.
REF_MODES = (
    ("grid_each", dict(global_sync=1, block_sync=0), False, False),
    ("grid_region", dict(global_sync=1, block_sync=0), True, False),
    ("block_each", dict(global_sync=0, block_sync=1), False, True),
    ("block_region", dict(global_sync=0, block_sync=1), True, True),
    ("none", dict(global_sync=0, block_sync=0), False, True),
)


def reference_gpu_baseline(w, timed_mcs=100, probe_mcs=10, top=6):
    """The reference's own CUDA sweep (oracle/_ref, its src/kernels.cu built
    for sm_103a) on the same lattice and GPU, at its best launch geometry and
    synchronisation mode.

    Geometry: every threads_per_block / positions_per_thread /
    positions_per_checkerboard / shared combination the reference accepts
    for this side (D divisible by tpb * ppt, ppc dividing ppt, grid
    co-resident for its cooperative launch), first with one attempt per grid
    sync as in its examples; the `top` fastest geometries are then timed in
    every other mode of REF_MODES.  The partial_dispatch kernel variant; J
    and T rounded to integers as the reference stores them.  Reports the best
    race-free mode and the best of all modes (racy ones marked).  Returns
    None when the reference build is absent.

    3D runs the non-shared variant only: the shared one asks for 128 KB of
    dynamic shared memory without the opt-in above 48 KB and cannot launch
    (the opt-in is commented out at src/cpm.cu:450).  Its blocks have tpb^3 threads
    and each thread makes ppt^3 attempts per MCS, one grid sync each, so
    ppt stops at 16 and the 26-neighbour sweep gets fewer MCS per probe.
    """
    try:
        from oracle import ref_gpu
    except Exception:
        return None
    if not ref_gpu.available() or w.ndim not in (2, 3):
        return None
    import torch
    n = w.lattice.shape[0]
    if n & (n - 1):
        # it would run, but on another model: the source pick wraps with a mask
        return {"unavailable": f"side {n} is not a power of two: the reference wraps its "
                               "neighbour pick as (x + dx) & (D - 1) (src/random.cu:25)"}
    r = ref_gpu.RefGpu(n, w.ndim, w.ncells, w.temperature, device=torch.cuda.current_device())
    r.apply(w)
    if w.ndim == 3:
        timed_mcs, probe_mcs = max(1, timed_mcs // 2), max(1, probe_mcs // 2)

    def knobs(mode, geo):
        name, sync, region, racy = mode
        ppc = geo["positions_per_checkerboard"]
        per = ppc ** w.ndim if region else 1
        return dict(geo, updates_per_barrier=per, updates_per_checkerboard_switch=per, **sync)

    def timed(mode, geo, mcs, seed):
        k = knobs(mode, geo)
        r.push(w.lattice)
        t0 = time.perf_counter()
        r.run(mcs, seed=seed, inner_iterations=1 if mode[3] else mcs, **k)  # an error ends the leg
        r.synchronize()
        return time.perf_counter() - t0

    geos = []
    for shared in ((0, 1) if w.ndim == 2 else (0,)):
        for tpb in ((4, 8, 16, 32) if w.ndim == 2 else (4, 8)):
            cap = r.max_coop_blocks(tpb, shared)
            for ppt in ((2, 4, 8, 16, 32, 64) if w.ndim == 2 else (2, 4, 8, 16)):
                if n % (tpb * ppt):
                    continue
                blocks = n // (tpb * ppt)
                if blocks ** w.ndim > cap:
                    continue
                for ppc in (1, 2, 4, 8):
                    if ppc > ppt or ppt % ppc or (shared and ppt % (2 * ppc)):
                        continue
                    # The reference's shared-memory branch bounds-checks
                    # against a fixed 64x64 tile (sharedDim = 64) but loads
                    # only a (2 ppc tpb)^2 square (src/kernels2d.cu:137-175,
                    # 368-379): any smaller square leaves shared memory it
                    # reads as cell ids uninitialised.  Only exact 64-site
                    # tiles are valid.
                    if shared and tpb * 2 * ppc != 64:
                        continue
                    geos.append(dict(threads_per_block=tpb, positions_per_thread=ppt,
                                     positions_per_checkerboard=ppc, shared=shared))
    if not geos:
        return None
    probes = sorted((timed(REF_MODES[0], g, probe_mcs, 7), i) for i, g in enumerate(geos))
    tried = [(dt, REF_MODES[0], geos[i]) for dt, i in probes]
    for mode in REF_MODES[1:]:
        for _, i in probes[:top]:
            g = geos[i]
            if g["shared"] and mode[0] != "grid_each":
                continue  # the shared branch is only validated with a grid sync per attempt
            tried.append((timed(mode, g, probe_mcs, 7), mode, g))

    def racy(mode, geo):
        return bool(mode[3]) or (not geo["shared"] and
                                 geo["positions_per_thread"] // geo["positions_per_checkerboard"] < 2)

    def final(entry):
        _, mode, geo = entry
        timed(mode, geo, probe_mcs, 11)  # warm-up
        dt = timed(mode, geo, timed_mcs, 13)
        return {"value": w.nsites * timed_mcs / dt, "unit": UNIT, "mcs_per_s": timed_mcs / dt,
                "mcs": timed_mcs, "mode": mode[0], "racy": racy(mode, geo),
                "run_knobs": knobs(mode, geo)}

    free = [t for t in tried if not racy(t[1], t[2])]
    best_free = final(min(free, key=lambda t: t[0])) if free else None
    best_any_entry = min(tried, key=lambda t: t[0])
    best_any = final(best_any_entry)
    if best_free is not None and best_any["value"] < best_free["value"]:
        best_any = best_free
    per_mode = {}
    for dt, mode, geo in tried:
        rate = w.nsites * probe_mcs / dt
        key = mode[0] + (" (racy geometry)" if racy(mode, geo) and not mode[3] else "")
        if key not in per_mode or rate > per_mode[key]["probe_value"]:
            per_mode[key] = {"probe_value": rate, "run_knobs": knobs(mode, geo),
                             "racy": racy(mode, geo)}
    return {"value": best_any["value"], "unit": UNIT, "mcs_per_s": best_any["mcs_per_s"],
            "mcs": timed_mcs, "mode": best_any["mode"], "racy": best_any["racy"],
            "run_knobs": best_any["run_knobs"],
            "best_race_free": best_free, "per_mode_probe": per_mode,
            "geometries_tried": len(geos), "probes": len(tried),
            "build": "reference src/kernels.cu, its nvcc flags, sm_103a (oracle/ref_gpu)",
            "timing": "host wall clock around run + synchronize (the reference's own "
                      "workflow), default stream",
            "notes": "partial_dispatch variant, J and T rounded to integers; value is the "
                     "best of all modes and geometries (racy ones included), best_race_free "
                     "the best with a grid sync and ppt / ppc >= 2"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    import oracle
    w = build_workload(args.workload)
    threads = os.cpu_count() or 1
    sim = oracle.OracleSim(w.lattice, w.ncells, **w.oracle_kwargs(), seed=0)
    # The GPU arm times a relaxed tissue (after its warm-up runs); relax this
    # one too, within a bounded time, so that both time comparable states.
    relax, t_relax = 0, time.perf_counter()
    while relax < REFERENCE_RELAX_MCS and time.perf_counter() - t_relax < 20.0:
        sim.run(5, nthreads=threads)
        relax += 5
    for _ in range(args.warmup):
        sim.run(1, nthreads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sim.run(1, nthreads=threads)
    dt = time.perf_counter() - t0
    value = w.nsites * args.steps / dt
    cfg = describe(w, 1)
    cfg["l2"] = "n/a (host CPU)"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u32+f32",
            "data": data_of(w), "config": cfg,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"1 MCS of the {w.name} lattice per step, after "
                                       f"{relax} MCS of relaxation from the seeded state, "
                                       f"{threads} OpenMP threads; the reference has no "
                                       "CPU implementation, so this is the oracle port"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def traffic_per_attempt(workload):
    """DRAM bytes per attempt of the sweep from the committed ncu summary."""
    f = ROOT / "profiles" / "traffic.json"
    try:
        d = json.loads(f.read_text())
        return float(d[workload]["dram_bytes_per_attempt"])
    except Exception:
        return None


def warp_inst_per_attempt(workload):
    """Warp instructions per attempt of the sweep from the committed ncu summary."""
    f = ROOT / "profiles" / "traffic.json"
    try:
        return float(json.loads(f.read_text())[workload]["warp_inst_per_attempt"])
    except Exception:
        return None


def issue_roofline(workload, attempts_per_s, clocks, torch, local):
    """The bound the sweep actually meets: warp-instruction issue.  Peak =
    4 schedulers x SMs x the SM clock sampled during the timed steps; achieved
    = attempts/s x the warp instructions per attempt that ncu counted."""
    ipa = warp_inst_per_attempt(workload)
    if ipa is None or not clocks or not clocks.get("sm_mhz"):
        return None
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    peak = 4 * sms * clocks["sm_mhz"] * 1e6
    achieved = attempts_per_s * ipa
    return {"bound": "issue", "achieved": achieved, "peak": peak,
            "unit": "warp instructions/s", "frac": achieved / peak,
            "warp_inst_per_attempt": ipa,
            "peak_source": f"4 x {sms} SMs x {clocks['sm_mhz']:.0f} MHz (sampled)"}


def warm_gpu(seconds=0.3):
    """Keep the GPU busy for a moment so that its clocks have left idle
    before the autotuner times anything (an idle GB300 ramps up over the
    first ~100 ms of work)."""
    import torch
    x = torch.randn(4096, 4096, device="cuda", dtype=torch.bfloat16)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        for _ in range(8):
            x = torch.tanh(x @ x)
        torch.cuda.synchronize()


def run_ours(args, world, rank, local, emit=True):
    import numpy as np
    import torch

    import gpucpm

    torch.cuda.set_device(local)
    gpucpm.set_device(local)
    w = build_workload(args.workload)
    mcs = args.mcs or w.mcs
    n = w.lattice.shape[0]
    sim = gpucpm.Cpm(n, w.ndim, w.ncells, w.temperature, False)
    sim.get_state()[...] = w.lattice.view(np.int32)
    w.apply(sim)
    sim.set_seed(0, rank)
    stream = torch.cuda.Stream()
    sim.set_stream(stream.cuda_stream)
    sim.push_to_gpu()
    if args.variant is not None:
        sim.set_variant(args.variant)
    if getattr(args, "fill", None):
        sim.set_fill({"parity": gpucpm.FILL_PARITY, "vector": gpucpm.FILL_VECTOR,
                      "tma": gpucpm.FILL_TMA, "cluster": gpucpm.FILL_CLUSTER}[args.fill])
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    for _ in range(args.warmup):
        sim.run_mcs(mcs)
    sim.synchronize()
    # the engine's own autotuner picks the tile variant from the relaxed
    # state the timed steps start from (the state is restored after it)
    if args.variant is None:
        warm_gpu()
        variant, tuned_ms = sim.autotune(probe_mcs=8)
        if getattr(args, "fill", None):  # a pinned fill stays pinned
            sim.set_fill({"parity": gpucpm.FILL_PARITY, "vector": gpucpm.FILL_VECTOR,
                          "tma": gpucpm.FILL_TMA, "cluster": gpucpm.FILL_CLUSTER}[args.fill])
    else:
        variant, tuned_ms = args.variant, None
    sim.synchronize()
    torch.cuda.synchronize()

    sampler = ClockSampler(gpu_index_for(torch, local)) if rank == 0 else None
    if sampler:
        sampler.start()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = sim.kernel_launches()
    dist_barrier(world)
    torch.cuda.synchronize()
    wall0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            starts[i].record(stream)
            sim.run_mcs(mcs)
            ends[i].record(stream)
    sim.synchronize()
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    dist_barrier(world)
    launches = sim.kernel_launches() - launches0
    clocks = sampler.stop() if sampler else None
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    dev_s = sum(step_ms) / 1e3
    dev_s_max = dist_max(world, dev_s)
    attempts_total = w.nsites * mcs * args.steps * world
    value = attempts_total / dev_s_max
    ms_per_step = dev_s_max / args.steps * 1e3

    # End to end through the public API with host buffers.
    e2e = None
    if not args.no_e2e:
        e2e_steps = max(1, min(args.steps, 5))
        sim.set_stream(None)
        sim.push_to_gpu()
        sim.run_mcs(mcs)
        sim.synchronize()
        sim.pull_from_gpu()
        dist_barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            sim.push_to_gpu()
            sim.run_mcs(mcs)
            sim.synchronize()
            sim.pull_from_gpu()
        e2e_s = dist_max(world, time.perf_counter() - t0)
        e2e = {"value": w.nsites * mcs * e2e_steps * world / e2e_s, "unit": UNIT,
               "h2d_bytes_per_step": 4 * w.nsites, "d2h_bytes_per_step": 4 * w.nsites + 4,
               "steps": e2e_steps, "path": "Cpm.push_to_gpu + run + synchronize + pull_from_gpu"}

    if rank != 0:
        return None
    peak, peak_kind = measured_peak_hbm()
    per_launch_s = dev_s / args.steps
    attempts_per_launch = w.nsites * mcs
    achieved = BYTES_PER_ATTEMPT * attempts_per_launch / per_launch_s / 1e9
    tpa = traffic_per_attempt(args.workload)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": f"{peak_kind} HBM copy (burst)",
                "traffic": tpa * attempts_per_launch if tpa is not None else None,
                "algorithmic_bytes_per_launch": BYTES_PER_ATTEMPT * attempts_per_launch,
                "kernel": {"parity": "sweep_kernel (one cooperative launch per step)",
                           "cluster": "sweep2d_kernel, cluster mode (one launch of one "
                                      "thread-block cluster per step)"}.get(
                    sim.sweep_config()["fill"],
                    ("sweep2d_kernel" if w.ndim == 2 else "sweep3d_kernel")
                    + " (one cooperative launch per step)")}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32+f32", "data": data_of(w),
            "config": dict(describe(w, mcs), tile=sim.sweep_config()["tile"],
                           fill=sim.sweep_config()["fill"]),
            "roofline": roofline,
            "issue_roofline": issue_roofline(args.workload, value / world, clocks, torch,
                                             local),
            "e2e": e2e,
            "autotune": {"variant": variant, "probe_ms_per_mcs": tuned_ms,
                         "dispatch": sim.sweep_config()["dispatch"],
                         "fill": sim.sweep_config()["fill"]},
            "gpu_launches": int(launches), "clocks": clocks,
            "mcs_per_s": value / w.nsites / world,
            "wall_s": wall, "step_ms": step_ms}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w)
    if not args.no_reference_gpu:
        try:
            ref = reference_gpu_baseline(w)
        except Exception as exc:  # noqa: BLE001 - reported, not fatal
            ref = {"unavailable": f"{type(exc).__name__}: {exc}"}
        if ref is not None:
            if "value" in ref:
                ref["speedup_of_value"] = value / world / ref["value"]
                if ref.get("best_race_free"):
                    ref["best_race_free"]["speedup_of_value"] = (
                        value / world / ref["best_race_free"]["value"])
            line["reference_gpu"] = ref
    if emit:
        print(json.dumps(line), flush=True)
    return line


def run_ensemble(args, world, rank, local, emit=True):
    """Batches: all replicas in one graph-captured persistent launch
    (batched) against the same replicas as a per-replica launch loop.

      ensemble       256 ragged replicas, side log-uniform in [64, 1024],
                     per-replica parameters (~193 MB of lattice)
      sorting_batch  512 replicas of the 256x256 two-type sorting lattice
                     (2600 cells of area 25; the forward of the gradient
                     workload without scores, 134 MB of lattice)

    Each rank runs its own ensemble (replica stream ids offset by rank).  The
    total lattice exceeds L2, so no flush is needed between steps.
    """
    import numpy as np
    import torch

    import gpucpm
    from gpucpm import workloads as W

    torch.cuda.set_device(local)
    gpucpm.set_device(local)
    sorting = args.workload == "sorting_batch"
    nrep = args.replicas or (512 if sorting else 256)
    ws = ([W.sorting_grid(n=256, ncells=2600, seed=0)] * nrep if sorting
          else W.ensemble_2d(nrep=nrep, seed=3))
    mcs = args.mcs or 500
    sizes = [w.lattice.shape[::-1] for w in ws]
    stream = torch.cuda.Stream()

    b = gpucpm.Batch(2, sizes, [w.ncells for w in ws])
    for r, w in enumerate(ws):
        b.lattice(r)[...] = w.lattice.view(np.int32)
        w.apply(b, replica=r)
    b.set_seed(0, rank * nrep)
    b.set_stream(stream.cuda_stream)
    b.push_to_gpu()
    if args.variant is not None:
        b.set_variant(args.variant)
    if args.dispatch is not None:
        b.set_dispatch({"replica": gpucpm.DISPATCH_REPLICA,
                        "hybrid": gpucpm.DISPATCH_HYBRID}.get(args.dispatch,
                                                              gpucpm.DISPATCH_GRID))
    for _ in range(args.warmup):
        b.run_graph(mcs)
    b.synchronize()
    # tuned from the relaxed state the timed steps start from; one more
    # untimed graph run captures the chosen launch
    if args.variant is None and args.dispatch is None:
        warm_gpu()
        variant, tuned_ms = b.autotune(probe_mcs=8)
        b.run_graph(mcs)
    else:
        variant, tuned_ms = b.sweep_config()["variant"], None
    b.synchronize()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = b.kernel_launches()
    sampler = ClockSampler(gpu_index_for(torch, local)) if rank == 0 else None
    if sampler:
        sampler.start()
    dist_barrier(world)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            starts[i].record(stream)
            b.run_graph(mcs)
            ends[i].record(stream)
    b.synchronize()
    torch.cuda.synchronize()
    clocks = sampler.stop() if sampler else None
    dist_barrier(world)
    launches = b.kernel_launches() - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    dev_s = dist_max(world, sum(step_ms) / 1e3)
    sites = sum(w.nsites for w in ws)
    value = sites * mcs * args.steps * world / dev_s
    batched_ms = dev_s / args.steps * 1e3

    # The same replicas as a per-replica launch loop: one single-lattice
    # engine per replica, each with the tile its own autotuner picks,
    # launched back to back on one stream.
    loop_ms = None
    engines = [] if not args.no_loop else None
    if engines is not None:
        for r, w in enumerate(ws):
            n = w.lattice.shape
            e = gpucpm.create_box(n[1], n[0], 1, 2, w.ncells, w.temperature)
            e.lattice(0)[...] = w.lattice.view(np.int32)
            w.apply(e, replica=0)
            e.set_seed(0, rank * nrep + r)
            e.set_stream(stream.cuda_stream)
            e.push_to_gpu()
            engines.append(e)
        for e in engines:
            e.run_mcs(2)  # warm-up
            e.autotune(probe_mcs=4)
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            t0.record(stream)
            for e in engines:
                e.run_mcs(mcs)
            t1.record(stream)
        for e in engines:
            e.synchronize()
        torch.cuda.synchronize()
        loop_ms = dist_max(world, t0.elapsed_time(t1) / 1e3) * 1e3
        del engines

    if rank != 0:
        return None
    peak, peak_kind = measured_peak_hbm()
    achieved = BYTES_PER_ATTEMPT * sites * mcs / (batched_ms / 1e3) / 1e9
    side = [s[0] for s in sizes]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": batched_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u32+f32",
            "data": "synthetic (seeded sorting grid)" if sorting else
                    "synthetic (seeded Voronoi replicas)",
            "config": {"workload": (f"sorting_batch {nrep} replicas of sorting_grid 256x256, "
                                    "2600 cells of target area 25" if sorting else
                                    f"ensemble_2d {nrep} replicas, side log-uniform "
                                    f"[64,1024] ({min(side)}..{max(side)}), cells = side^2/50, "
                                    "per-replica J~U[2,20], lambda~U[0.5,2], T~U[5,30]"),
                       "sites": sites, "mcs_per_step": mcs, "tile_variant": variant,
                       "dispatch": b.sweep_config()["dispatch"],
                       "l2": "inputs larger than L2 (no flush)", "seed": 0},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "peak_source": f"{peak_kind} HBM copy (burst)", "traffic": None,
                         "algorithmic_bytes_per_launch": BYTES_PER_ATTEMPT * sites * mcs,
                         "kernel": "sweep_kernel (one graph-captured launch per step)"},
            "gpu_launches": int(launches),
            "batched_vs_loop": None if loop_ms is None else {
                "batched_ms": batched_ms, "loop_ms": loop_ms, "speedup": loop_ms / batched_ms,
                "loop": "one single-lattice engine per replica, each with its own "
                        "autotuned tile, launched back to back on one stream"},
            "autotune": {"variant": variant, "probe_ms_per_mcs": tuned_ms,
                         "dispatch": b.sweep_config()["dispatch"]},
            "step_ms": step_ms, "clocks": clocks, "e2e": None}
    if emit:
        print(json.dumps(line), flush=True)
    return line


def run_gradient(args, world, rank, local, emit=True):
    """Differentiated ensemble of two-type sorting lattices, observable O =
    heterotypic fraction at the last MCS, theta = (J_ll, J_dd, J_ld, J_lm,
    J_dm, lambda_area, T).

      gradient        512 replicas of 256x256 (2600 cells of target area 25
                      on the 51x51 grid of 5-strided slots), O at MCS 500
      gradient_check  131072 replicas of 60x60 (143 cells on the 12x12 grid,
                      the same packing), O at MCS 10: the likelihood-ratio
                      error shrinks with replicas and short horizons, not
                      with lattice size, so this is where a 5% comparison
                      with finite differences is resolvable

    Times a forward pass alone (restart + MCS + observation) against the
    differentiated step (the same forward with score accumulation, then the
    backward kernel through torch.autograd), and compares the likelihood-ratio
    gradient of mean_r O with CRN central differences at +-1% of each
    parameter.  Both estimates come with their standard errors over
    replicas.  Each rank runs its own ensemble (stream ids offset by rank).
    """
    import numpy as np
    import torch

    import gpucpm
    from gpucpm import grad as G
    from gpucpm import workloads as W

    torch.cuda.set_device(local)
    gpucpm.set_device(local)
    check = args.workload == "gradient_check"
    side, ncells = (60, 143) if check else (256, 2600)
    nrep = args.replicas or (131072 if check else 512)
    mcs = args.mcs or (10 if check else 500)
    w = W.sorting_grid(n=side, ncells=ncells, seed=0)
    # N > 1: the ranks shard one ensemble of N * nrep replicas; the baseline
    # and the gradient are the global ones (one all-reduce of observable
    # totals before the backward kernel, one of the gradient after it)
    group = None
    if world > 1:
        import torch.distributed as dist
        group = dist.group.WORLD
    ens = G.Ensemble([w] * nrep, seed=0, stream_id=rank * nrep, group=group)
    theta0 = ens.theta0()
    names = ["J_ll", "J_dd", "J_ld", "J_lm", "J_dm", "lambda_area", "T"]

    def fwd():
        return ens.forward(theta0, mcs, [mcs], scores=False)[0]

    def lr_step():
        th = theta0.clone().requires_grad_(True)
        O = G.LikelihoodRatio.apply(th, ens, mcs, [mcs])
        O.mean().backward()
        torch.cuda.synchronize()
        return th.grad

    for _ in range(args.warmup):
        fwd()
        lr_step()
    torch.cuda.synchronize()
    launches0 = ens.batch.kernel_launches()
    dist_barrier(world)
    sampler = ClockSampler(gpu_index_for(torch, local))
    sampler.start()
    t_fwd, t_lr = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        fwd()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        g = lr_step()
        t2 = time.perf_counter()
        t_fwd.append(t1 - t0)
        t_lr.append(t2 - t1)
    clocks = sampler.stop()
    dist_barrier(world)
    launches = ens.batch.kernel_launches() - launches0
    fwd_s = dist_max(world, statistics.median(t_fwd))
    lr_s = dist_max(world, statistics.median(t_lr))

    if args.no_fd:
        if rank != 0:
            return None
        line = {"metric": METRIC, "value": nrep * w.nsites * mcs * world / lr_s, "unit": UNIT,
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": lr_s * 1e3, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "u32+f32",
                "data": "synthetic (seeded sorting grid)",
                "config": {"workload": f"{args.workload}: {nrep} replicas of sorting_grid "
                                       f"{side}x{side}, {ncells} cells of target area 25, "
                                       f"O = heterotypic fraction at MCS {mcs}",
                           "sites": nrep * w.nsites, "mcs_per_step": mcs, "seed": 0},
                "gradient": {"forward_ms": fwd_s * 1e3,
                             "forward_scores_backward_ms": lr_s * 1e3,
                             "cost_ratio": lr_s / fwd_s},
                "gpu_launches": int(launches), "clocks": clocks, "e2e": None}
        if emit:
            print(json.dumps(line), flush=True)
        return line

    # standard error of the LR estimate from its per-replica terms
    O, sc, _ = ens.forward(theta0, mcs, [mcs], scores=True)
    o = O[:, 0].double().cpu().numpy()
    cum = sc[:, :, :ens.nparam].double().sum(dim=1).cpu().numpy()
    b = (o.sum() - o) / (nrep - 1)
    terms = (o - b)[:, None] * cum
    lr_np = terms.mean(axis=0)
    lr_se = terms.std(axis=0, ddof=1) / np.sqrt(nrep)
    fd_params = None
    if args.fd_params:
        fd_params = [names.index(n) for n in args.fd_params.split(",")]
    fd, fd_per = G.crn_finite_difference(ens, theta0, mcs, rel_step=0.01, per_replica=True,
                                         params=fd_params)
    fd = fd.numpy()
    fd_se = fd_per.numpy().std(axis=0, ddof=1) / np.sqrt(nrep)
    lr = g.double().cpu().numpy()

    if rank != 0:
        return None
    sites = nrep * w.nsites
    rel = np.abs(lr - fd) / np.maximum(np.abs(fd), 1e-30)
    z = (lr - fd) / np.sqrt(lr_se ** 2 + fd_se ** 2)
    per_param = {n: {"theta": float(theta0[k]), "lr": float(lr[k]), "lr_se": float(lr_se[k]),
                     "fd": float(fd[k]), "fd_se": float(fd_se[k]), "rel_diff": float(rel[k]),
                     "z": float(z[k])}
                 for k, n in enumerate(names)}
    line = {"metric": METRIC, "value": sites * mcs * world / lr_s, "unit": UNIT,
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": lr_s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32+f32", "data": "synthetic (seeded sorting grid)",
            "config": {"workload": f"{args.workload}: {nrep} replicas of sorting_grid "
                                   f"{side}x{side}, {ncells} cells of target area 25, "
                                   f"O = heterotypic fraction at MCS {mcs}",
                       "sites": sites, "mcs_per_step": mcs,
                       "l2": "inputs larger than L2 (no flush)", "seed": 0},
            "gradient": {"forward_ms": fwd_s * 1e3, "forward_scores_backward_ms": lr_s * 1e3,
                         "cost_ratio": lr_s / fwd_s,
                         "lr_matches_autograd": bool(np.allclose(lr_np, lr, rtol=1e-3,
                                                                 atol=1e-3 * np.abs(lr).max())),
                         "fd_step": "central, +-1% of each parameter, common random numbers",
                         "params": per_param,
                         "max_rel_diff": float(np.nanmax(rel)),
                         "within_5pct": [n for k, n in enumerate(names) if rel[k] <= 0.05],
                         "resolvable": [n for k, n in enumerate(names)
                                        if abs(fd[k]) > 20 * np.hypot(lr_se[k], fd_se[k])]},
            "timing": "wall clock of whole forward / differentiated steps (median), "
                      "each including restart (H2D of the initial lattices) and observation",
            "gpu_launches": int(launches), "clocks": clocks, "e2e": None}
    if emit:
        print(json.dumps(line), flush=True)
    return line


def secondary(args, world, rank, local):
    """Compact results of the other benchmark configurations, measured in the
    same process after the headline: the 256^3 tissue and the 256^2 sorting
    recipe (attempts/s, each with the reference's CUDA build on it), the
    256-replica ragged ensemble (one
    graph-captured launch against a per-replica launch loop) and the
    512 x 256^2 gradient ensemble (forward + scores + backward against the
    forward alone).  Each carries its own clock record."""
    import copy

    def sub(**kw):
        a = copy.copy(args)
        a.no_e2e, a.no_cpu_baseline, a.no_reference_gpu = True, True, True
        a.variant = a.dispatch = a.mcs = a.replicas = a.fill = None
        a.no_loop, a.no_fd, a.no_secondary = False, True, True
        for k, v in kw.items():
            setattr(a, k, v)
        return a

    out = {}
    line = run_ours(sub(workload="tissue_3d", steps=3, warmup=2, no_reference_gpu=False),
                    world, rank, local, emit=False)
    if line is not None:
        ref = line.get("reference_gpu") or {}
        out["tissue_3d_256"] = {
            "value": line["value"], "unit": UNIT, "ms_per_step": line["ms_per_step"],
            "mcs_per_step": line["config"]["mcs_per_step"],
            "roofline_frac": line["roofline"]["frac"], "tile": line["config"]["tile"],
            "clocks": line["clocks"],
            "reference_gpu": {k: ref.get(k) for k in ("value", "mode", "racy", "run_knobs",
                                                      "speedup_of_value")}
            if "value" in ref else ref or None,
            "reference_gpu_race_free": {k: (ref.get("best_race_free") or {}).get(k)
                                        for k in ("value", "mode", "run_knobs",
                                                  "speedup_of_value")}
            if "value" in ref else None}
    line = run_ours(sub(workload="sorting_2d_256", steps=3, warmup=3, no_reference_gpu=False),
                    world, rank, local, emit=False)
    if line is not None:
        ref = line.get("reference_gpu") or {}
        out["sorting_256"] = {
            "value": line["value"], "unit": UNIT, "ms_per_step": line["ms_per_step"],
            "mcs_per_step": line["config"]["mcs_per_step"], "tile": line["config"]["tile"],
            "fill": line["config"]["fill"], "clocks": line["clocks"],
            "reference_gpu": {k: ref.get(k) for k in ("value", "mode", "racy", "run_knobs",
                                                      "speedup_of_value")}
            if "value" in ref else ref or None,
            "reference_gpu_race_free": {k: (ref.get("best_race_free") or {}).get(k)
                                        for k in ("value", "mode", "run_knobs",
                                                  "speedup_of_value")}
            if "value" in ref else None}
    line = run_ensemble(sub(workload="ensemble", steps=2, warmup=2), world, rank, local,
                        emit=False)
    if line is not None:
        out["ensemble_256"] = {"value": line["value"], "unit": UNIT,
                               "sites": line["config"]["sites"], "mcs_per_step": 500,
                               "dispatch": line["config"]["dispatch"],
                               "batched_vs_loop": line["batched_vs_loop"],
                               "clocks": line["clocks"]}
    line = run_gradient(sub(workload="gradient", steps=2, warmup=1), world, rank, local,
                        emit=False)
    if line is not None:
        out["gradient_512x256"] = dict(line["gradient"], clocks=line["clocks"],
                                       workload=line["config"]["workload"])
    return out


def main():
    args = parse_args()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload in ("ensemble", "sorting_batch"):
        run_ensemble(args, world, rank, local)
    elif args.workload in ("gradient", "gradient_check"):
        run_gradient(args, world, rank, local)
    else:
        secondary_keys = args.workload == "tissue_2d" and not args.no_secondary
        line = run_ours(args, world, rank, local, emit=not secondary_keys)
        if secondary_keys:
            extra = secondary(args, world, rank, local)
            if line is not None:
                line["secondary"] = extra
                print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

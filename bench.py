#!/usr/bin/env python3
"""Throughput bench of the GB300 FMM gravity step (body-steps/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl fmm|reference]

A bench step is one full solve of the workload: the scene is reset from a
device-resident pristine copy (upload + leaf sort + deposit) and advanced
`fmm_steps` leapfrog steps.  The default workload is the reference's default
preset, a 1,048,576-body Plummer sphere (a = 0.1, centred in the unit box,
truncated at r = 0.5, G = 1, eps = 1e-3, dt = 5e-4) run for 60 steps.

Timing: W untimed warm-up steps, then exactly K timed steps, each bracketed by
CUDA events on the solver's stream; L2 is flushed (512 MiB write) between
timed steps, outside the events.  Barrier + synchronize on both sides, max
over ranks.  N GPUs run N independent replicas (one process per GPU; the
plain solve does not shard), so `value` is the sum of all replicas' work over
the slowest replica's time.

The JSON line adds: `e2e` (the same metric through the C ABI from pinned host
buffers, host<->device copies inside the timed region), `roofline` for the
dominant kernel (integrate), `cpu_baseline` (the CPU oracle on the host cores,
rank 0 only), `clocks` sampled during the timed region, `gpu_launches`, and
per-kernel times.

`--impl reference` times the reference algorithm's CPU implementation (the
oracle port: the reference's Rust/WGSL harness needs a Vulkan adapter and a
Rust toolchain, neither of which exists here) on the host cores, one FMM step
of the same workload per bench step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "fmm-rainbow_gb300")
for _p in (REPO, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

from rfmm import workloads  # noqa: E402  (numpy only; the solver library loads later)

PEAKS_FILE = os.path.join(REPO, "MEASURED_PEAKS.json")
TRAFFIC_FILE = os.path.join(REPO, "profiles", "ncu_traffic.json")
FALLBACK_HBM_GBS = 6800.0
P2P_MAX_BODIES = 1 << 18


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="plummer_1m", choices=sorted(workloads.WORKLOADS))
    ap.add_argument("--impl", default="fmm", choices=["fmm", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--requests", type=int, default=0, help="served: requests per rate point")
    ap.add_argument("--rates", type=float, nargs="*", default=None, help="served: arrival rates /s")
    ap.add_argument("--near", default="reference", choices=["reference", "p2p"],
                    help="near field: the reference's cell monopoles, or exact pair sums")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_scene(w):
    from rfmm import workloads
    return workloads.scene(w)


def batch_scenes(w):
    from rfmm import workloads
    return workloads.batch_scenes(w)


def roofline_bytes_integrate(n, cells, depth):
    from rfmm import workloads
    return workloads.roofline_bytes_integrate(n, cells, depth)


def clocks_sampler(gpu_index):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        return subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + q,
                                 "--format=csv,noheader,nounits", "-lms", "100"],
                                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
    except OSError:
        return None


def clocks_summary(proc):
    if proc is None:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    proc.terminate()
    try:
        out, _ = proc.communicate(timeout=5)
    except subprocess.TimeoutExpired:
        proc.kill()
        out, _ = proc.communicate()
    sm, smax, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in out.strip().splitlines():
        f = [x.strip() for x in line.split(",")]
        if len(f) < 9:
            continue
        try:
            sm.append(float(f[1]))
            smax.append(float(f[2]))
        except ValueError:
            continue
        for name, v in zip(names, f[5:9]):
            if v.lower() == "active":
                reasons.add(name)
    return {"sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    try:
        with open(PEAKS_FILE) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def traffic_for(workload):
    try:
        with open(TRAFFIC_FILE) as f:
            t = json.load(f)
        entry = t.get("k_integrate", {}).get(workload)
        return None if entry is None else float(entry["dram_bytes_per_launch"])
    except (OSError, ValueError, KeyError):
        return None


def cpu_baseline(w, seconds, near="reference"):
    """The CPU oracle (the reference algorithm restated in C, OpenMP) on this
    host: all host threads, then one thread on a shorter sample."""
    from oracle import oracle as O
    scene = make_scene(w)

    def sample(threads, budget):
        cores = O.set_threads(threads)
        st = O.OracleState(scene, O.make_params(w["n"], gravity=w["G"], softening=w["eps"], dt=w["dt"],
                                                near_mode=1 if near == "p2p" else 0))
        done, t0 = 0, time.perf_counter()
        while True:
            st.step(1)
            done += 1
            el = time.perf_counter() - t0
            if el >= budget or done >= w["fmm_steps"]:
                break
        return w["n"] * done / el, cores, done, el

    value, cores, done, el = sample(os.cpu_count() or 1, seconds)
    v1, _, d1, e1 = sample(1, seconds / 3.0)
    O.set_threads(os.cpu_count() or 1)
    return {"value": value, "unit": "body-steps/s", "cores": cores, "kind": "port",
            "sample": "%d FMM step(s) of the same workload (%d bodies, %s near field) on %d host "
                      "threads, %.1f s" % (done, w["n"], near, cores, el),
            "single_thread": {"value": v1, "sample": "%d step(s), %.1f s" % (d1, e1)}}


def run_reference(args, w):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    cores = O.set_threads(os.cpu_count() or 1)
    if w["kind"] == "batched":
        ps = batch_scenes(w)
        states = [O.OracleState(p, O.make_params(len(p), gravity=w["G"], softening=w["eps"],
                                                 dt=w["dt"])) for p in ps]
        bodies = sum(len(p) for p in ps)
    else:
        states = [O.OracleState(make_scene(w), O.make_params(w["n"], gravity=w["G"],
                                                             softening=w["eps"], dt=w["dt"]))]
        bodies = w["n"]
    for _ in range(args.warmup):
        for st in states:
            st.step(1)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for st in states:
            st.step(1)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    value = bodies * args.steps / total
    line = {
        "impl": "reference", "metric": "body-steps/s", "value": value, "unit": "body-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded): " + w["desc"],
        "config": {"workload": args.workload, "bodies": bodies, "fmm_steps_per_bench_step": 1,
                   "implementation": "CPU oracle port of the reference compute passes "
                                     "(reference wgpu/Vulkan harness unavailable on this box)"},
        "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": cores, "kind": "port",
                         "sample": "one FMM step of %d bodies per bench step, %d host threads"
                                   % (bodies, cores)},
        "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, w):
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from rfmm import build as pkg_build
    pkg_build.build()
    import rfmm

    n, fmm_steps = w["n"], w["fmm_steps"]
    if args.near == "p2p" and n > P2P_MAX_BODIES:
        raise SystemExit("--near p2p: at most %d bodies (the depth-6 cap leaves Plummer cores with "
                         "thousands of bodies per leaf, ~1e5 pairs per body)" % P2P_MAX_BODIES)
    scene = make_scene(w)
    params = rfmm.default_params(gravity=w["G"], softening=w["eps"], dt=w["dt"])
    # A real (non-default) stream shared by torch's events/flush and the solver.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    solver = rfmm.Solver(n, params)
    solver.set_stream(stream.cuda_stream)
    if args.near == "p2p":
        solver.set_near_mode(rfmm.NEAR_P2P)
    pristine = torch.from_numpy(scene.view(np.uint8).copy()).cuda()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")

    def bench_step():
        solver.upload_device(pristine.data_ptr(), pristine.numel())
        solver.step(fmm_steps)

    tuning = solver.tuning()
    if not args.no_autotune:  # project autotuner: launch shapes timed on this scene
        solver.upload_device(pristine.data_ptr(), pristine.numel())
        tuning = solver.autotune(20)
    for _ in range(args.warmup):
        bench_step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clk = clocks_sampler(local)
    time.sleep(0.3)
    barrier()
    l0 = solver.launch_count()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        bench_step()
        ends[k].record(stream)
    barrier()
    launches = solver.launch_count() - l0
    clocks = clocks_summary(clk)
    local_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    from rfmm import replicas
    value, _, slowest_s = replicas.reduce_throughput(n * fmm_steps * args.steps, local_ms * 1e-3)
    total_ms = slowest_s * 1e3
    solver.sync()

    # Per-kernel device times over the same workload (event pair around every launch).
    solver.upload_device(pristine.data_ptr(), pristine.numel())
    prof = solver.profile_steps(fmm_steps)
    integ_ms, integ_n = prof["integrate"]
    alg_bytes = roofline_bytes_integrate(n, solver.cells, solver.depth)
    peak, peak_kind = hbm_peak()
    achieved = alg_bytes / (integ_ms / integ_n * 1e-3) / 1e9
    roofline = {"kernel": "k_integrate", "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": alg_bytes,
                "avg_launch_ms": integ_ms / integ_n, "traffic": traffic_for(args.workload)}
    kernel_ms = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in prof.items()}

    # End to end through the C ABI with host buffers: pinned input upload
    # (H2D + leaf sort), the solve, pinned download of the result (D2H).
    pin_in = torch.from_numpy(scene.view(np.uint8).copy()).pin_memory()
    pin_out = torch.empty(n * 32, dtype=torch.uint8).pin_memory()
    e2e_times = []
    for k in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        solver.upload_host_ptr(pin_in.data_ptr(), pin_in.numel())
        solver.step(fmm_steps)
        solver.download_host_ptr(rfmm.BUF_PARTICLES, pin_out.data_ptr(), pin_out.numel())
        if k > 0:
            e2e_times.append(time.perf_counter() - t0)
    e2e = None
    if e2e_times:
        e2e_s = statistics.median(e2e_times)  # host wall clock: the median resists scheduler jitter
        e2e = {"value": world * n * fmm_steps / e2e_s, "unit": "body-steps/s",
               "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": n * 32,
               "ms_per_step": 1e3 * e2e_s, "timer": "host wall clock"}

    # Accuracy of the state the bench ends on (outside every timed region):
    # FP64 direct-sum force error on a seeded target sample, FP64 energy.
    rms, mx = solver.force_error(4096, 1)
    diag = solver.diagnostics()
    accuracy = {"near_field": args.near, "force_rms_rel": rms, "force_max_rel": mx,
                "targets": min(4096, n),
                "reference": "FP64 softened direct sum on the GPU (all N sources)",
                "energy_total": diag["total"], "kinetic": diag["kinetic"],
                "potential": diag["potential"]}
    if args.near == "reference":  # the same final state with exact near-field pair sums
        solver.set_near_mode(rfmm.NEAR_P2P)
        prms, pmx = solver.force_error(4096, 1)
        accuracy["p2p_mode"] = {"force_rms_rel": prms, "force_max_rel": pmx}
        solver.set_near_mode(rfmm.NEAR_REFERENCE)

    # Headless display pass of the final state (1920 x 1080 canvas), outside
    # every timed region: splat, two blur passes and the resolve on the GPU.
    render = None
    if args.near == "reference":
        rp = rfmm.default_render_params(width=1920, height=1080)
        img = torch.empty(1080 * 1920 * 4, dtype=torch.uint8, device="cuda")
        r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        solver.render_device(rp, img.data_ptr(), img.numel())  # warm (allocates the textures)
        frames = 5
        r0.record(stream)
        for _ in range(frames):
            solver.render_device(rp, img.data_ptr(), img.numel())
        r1.record(stream)
        torch.cuda.synchronize()
        render = {"canvas": [1920, 1080], "points": n, "frame_ms": r0.elapsed_time(r1) / frames,
                  "kernels_per_frame": 5, "note": "includes the host round trip of each call"}

    line = {
        "metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, numpy PCG64): " + w["desc"],
        "config": {"workload": args.workload, "form": "plain single-scene solve",
                   "near_field": args.near,
                   "bodies": n, "fmm_steps_per_bench_step": fmm_steps, "depth": solver.depth,
                   "cells": solver.cells, "fixed_point_scale": solver.scale,
                   "l2": "flushed between timed steps (512 MiB write outside the events)",
                   "parallelism": "replicas x%d" % world},
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
        "kernel_avg_ms": kernel_ms, "tuning": tuning.as_dict(), "accuracy": accuracy,
        "render": render,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_seconds, args.near)
    if rank == 0:
        print(json.dumps(line), flush=True)
    solver.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_gpu_batched(args, w):
    """Batched form vs the same scenes solved back to back through plain handles."""
    import numpy as np
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from rfmm import build as pkg_build
    pkg_build.build()
    import rfmm
    from rfmm import replicas

    all_scenes = batch_scenes(w)
    mine = replicas.shard_scenes([len(p) for p in all_scenes], world)[rank]
    ps = [all_scenes[i] for i in mine]
    sizes = [len(p) for p in ps]
    bodies = sum(sizes)
    fmm_steps = w["fmm_steps"]
    params = rfmm.default_params(gravity=w["G"], softening=w["eps"], dt=w["dt"])
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    dev = [torch.from_numpy(p.view(np.uint8).copy()).cuda() for p in ps]
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    batch = rfmm.Batch(sizes, [params] * len(ps))
    batch.set_stream(stream.cuda_stream)

    dev_ptrs = [d.data_ptr() for d in dev]

    def batched_step():
        batch.upload_device_all(dev_ptrs)  # one copy launch for all scenes
        batch.commit()
        batch.step(fmm_steps)

    def timed(fn, k):
        st = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
        for j in range(k):
            flush.zero_()
            st[j].record(stream)
            fn()
            en[j].record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in zip(st, en))

    batched_step()
    tuning = batch.tuning()
    if not args.no_autotune:
        tuning = batch.autotune(5)
    for _ in range(args.warmup):
        batched_step()
    torch.cuda.synchronize()
    clk = clocks_sampler(local)
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    l0 = batch.launch_count()
    local_ms = timed(batched_step, args.steps)
    if world > 1:
        torch.distributed.barrier()
    launches = batch.launch_count() - l0
    clocks = clocks_summary(clk)
    value, _, slowest_s = replicas.reduce_throughput(bodies * fmm_steps * args.steps, local_ms * 1e-3)

    # The same scenes back to back through plain handles (one handle per scene).
    solvers = []
    for p in ps:
        s = rfmm.Solver(len(p), params)
        s.set_stream(stream.cuda_stream)
        solvers.append(s)

    def plain_step():
        for s, d in zip(solvers, dev):
            s.upload_device(d.data_ptr(), d.numel())
            s.step(fmm_steps)

    plain_step()
    torch.cuda.synchronize()
    plain_k = max(1, min(args.steps, 3))
    plain_ms = timed(plain_step, plain_k)
    plain_value = bodies * fmm_steps * plain_k / (plain_ms * 1e-3)
    for s in solvers:
        s.close()

    prof = batch.profile_steps(fmm_steps)
    kernel_ms = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in prof.items()}
    integ_ms, integ_n = prof["integrate"]
    alg = sum(64 * n for n in sizes) + sum(64 * pl[1] + 16 * 8 ** pl[0] for pl in batch.plans)
    peak, peak_kind = hbm_peak()
    achieved = alg / (integ_ms / integ_n * 1e-3) / 1e9
    roofline = {"kernel": "k_integrate", "bound": "hbm", "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": alg, "avg_launch_ms": integ_ms / integ_n,
                "traffic": traffic_for(args.workload)}

    # End to end: pinned host scenes in, every scene's particles out.
    pin = [torch.from_numpy(p.view(np.uint8).copy()).pin_memory() for p in ps]
    outs = [torch.empty(len(p) * 32, dtype=torch.uint8).pin_memory() for p in ps]
    out_ptrs = [t.data_ptr() for t in outs]
    e2e_times = []
    for k in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i, t in enumerate(pin):
            rfmm._check(rfmm.lib().rfmm_batch_upload(batch._h, i, t.data_ptr(), t.numel()), "upload")
        batch.commit()
        batch.step(fmm_steps)
        batch.download_all_into(rfmm.BUF_PARTICLES, out_ptrs)  # one synchronisation
        if k > 0:
            e2e_times.append(time.perf_counter() - t0)
    e2e = None
    if e2e_times:
        e2e_s = statistics.mean(e2e_times)
        e2e = {"value": world * bodies * fmm_steps / e2e_s, "unit": "body-steps/s",
               "h2d_bytes_per_step": bodies * 32, "d2h_bytes_per_step": bodies * 32,
               "ms_per_step": 1e3 * e2e_s, "timer": "host wall clock"}
    line = {
        "metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": slowest_s * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, numpy PCG64): " + w["desc"],
        "config": {"workload": args.workload, "form": "batched (all scenes per launch)",
                   "scenes": len(ps), "bodies": bodies, "fmm_steps_per_bench_step": fmm_steps,
                   "plain_back_to_back_body_steps_per_s": plain_value,
                   "batched_over_plain": value / world / plain_value,
                   "l2": "flushed between timed steps (512 MiB write outside the events)",
                   "parallelism": "scenes sharded over %d rank(s)" % world},
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
        "kernel_avg_ms": kernel_ms, "tuning": tuning.as_dict(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    batch.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def served_requests(w, count):
    """Seeded request pool: (particles, steps)."""
    import numpy as np
    from rfmm import scenes
    rng = np.random.default_rng(w["seed"])
    out = []
    for i in range(count):
        n = int(np.exp(rng.uniform(np.log(w["n_min"]), np.log(w["n_max"]))))
        steps = int(rng.integers(1, w["steps_max"] + 1))
        kind = ("uniform", "plummer", "clusters4")[i % 3]
        out.append((scenes.make(kind, n, 2000 + i), steps))
    return out


def run_gpu_served(args, w):
    """Throughput and p50/p99 latency of the continuous-batching server."""
    import threading
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    from rfmm import build as pkg_build
    pkg_build.build()
    import rfmm

    import numpy as np
    count = max(4, args.requests or w["requests"])
    pool = served_requests(w, count)
    params = rfmm.default_params(gravity=w["G"], softening=w["eps"], dt=w["dt"])
    rates = args.rates or w["rates"]
    sweep = []
    clk = None
    launches = 0
    # Warm-up: module load and first graph captures on a small server.
    warm = rfmm.Server(max_bodies=w["n_max"], memory_budget_bytes=w["budget"], max_slots=4,
                       max_chunk_steps=4)
    for p, steps in pool[: min(3, len(pool))]:
        rid = warm.submit(p, steps, params)
        warm.wait(rid, 600000)
        warm.result(rid)
    warm.close()
    for ri, rate in enumerate(rates):
        srv = rfmm.Server(max_bodies=w["n_max"], memory_budget_bytes=w["budget"],
                          max_slots=w["slots"], max_chunk_steps=4)
        arrivals = np.cumsum(np.random.default_rng(w["seed"] + ri).exponential(1.0 / rate, count))
        ids = [None] * count
        if ri == len(rates) - 1:
            clk = clocks_sampler(local)
        t0 = time.perf_counter()

        def producer():
            for i, (p, steps) in enumerate(pool):
                delay = t0 + arrivals[i] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                ids[i] = srv.submit(p, steps, params)

        th = threading.Thread(target=producer)
        th.start()
        th.join()
        for rid in ids:
            srv.wait(rid, 3600000)
            srv.result(rid)
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        sweep.append({"rate_per_s": rate, "requests": count, "p50_ms": st["p50_ms"],
                      "p99_ms": st["p99_ms"], "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
                      "body_steps_per_s": st["body_steps_per_s"], "wall_s": wall,
                      "slots": st["slots"]})
    clocks = clocks_summary(clk)
    top = sweep[-1]
    body_steps = sum(len(p) * s for p, s in pool)
    line = {
        "metric": "body-steps/s", "value": top["body_steps_per_s"], "unit": "body-steps/s",
        "n_gpus": world, "steps": count, "warmup": 3, "ms_per_step": top["wall_s"] * 1e3 / count,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, numpy PCG64): " + w["desc"],
        "config": {"workload": args.workload, "form": "served (continuous batching)",
                   "requests_per_rate": count, "body_steps_per_rate": body_steps,
                   "memory_budget_bytes": w["budget"], "slot_capacity": w["n_max"],
                   "p50_ms": top["p50_ms"], "p99_ms": top["p99_ms"], "sweep": sweep,
                   "timer": "host wall clock, submit to result on host",
                   "parallelism": "1 GPU"},
        "clocks": clocks,
        "e2e": {"value": top["body_steps_per_s"], "unit": "body-steps/s",
                "h2d_bytes_per_step": body_steps and int(sum(len(p) for p, _ in pool) * 32 / count),
                "d2h_bytes_per_step": int(sum(len(p) for p, _ in pool) * 32 / count),
                "note": "a step is one request; the served path is end to end by construction"},
        "gpu_launches": None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    w = workloads.WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    if w["kind"] == "batched":
        return run_gpu_batched(args, w)
    if w["kind"] == "served":
        return run_gpu_served(args, w)
    return run_gpu(args, w)


if __name__ == "__main__":
    sys.exit(main())

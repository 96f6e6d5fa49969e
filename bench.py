#!/usr/bin/env python3
"""Throughput bench of the GB300 FMM gravity step (body-steps/s).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl fmm|reference]

A bench step is one full solve of the workload: the scene is reset from a
device-resident pristine copy (upload + leaf sort + deposit) and advanced
`fmm_steps` leapfrog steps.  The default workload is the reference's default
preset, a 1,048,576-body Plummer sphere (a = 0.1, centred in the unit box,
truncated at r = 0.5, G = 1, eps = 1e-3, dt = 5e-4) run for 60 steps; its line
also carries the batched form (256 scenes, one set of launches per step)
measured against the same scenes solved back to back through plain handles.

Timing: W untimed warm-up steps, then exactly K timed steps, each bracketed by
CUDA events on the solver's stream; L2 is flushed (512 MiB write) between
timed steps, outside the events.  Barrier + synchronize on both sides, max
over ranks.  N GPUs run N independent replicas (one process per GPU; the
plain solve does not shard), so `value` is the sum of all replicas' work over
the slowest replica's time.

Per-phase times come from a second timed pass with the in-graph timeline on
(rfmm_set_timeline): every step kernel stamps, with %globaltimer, its first
CTA's begin (after its dependency wait) and its last CTA's end inside the
same CUDA graphs and programmatic dependent launches that produce `value`.
Each phase's algorithmic bytes (flops for M2L) are counted exactly from the
tree the run ends on (rfmm/roofline.py).

The JSON line adds: `e2e` (the same metric through the C ABI from pinned host
buffers, host<->device copies inside the timed region), `roofline` for the
dominant kernel (integrate) with `phases` for every step kernel,
`cpu_baseline` (the CPU oracle on the host cores, rank 0 only), `clocks`
sampled during the timed region and `gpu_launches`.

`--impl reference` times the reference algorithm's CPU implementation (the
oracle port: the reference's Rust/WGSL harness needs a Vulkan adapter and a
Rust toolchain, neither of which exists here) on all host cores, with the
same protocol as `cpu_baseline`: each bench step resets the scene and runs
the workload's FMM steps.  Both CPU legs also report `reference_shader`: the
reference's own WGSL compute passes, translated to C++, on the same cores
(slower than the port, which therefore stays the conservative baseline).
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
REFERENCE_BUDGET_S = 150.0  # the reference arm's whole run


def parse_args():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="plummer_1m", choices=sorted(workloads.WORKLOADS))
    ap.add_argument("--impl", default="fmm", choices=["fmm", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=8)
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-baseline-only", action="store_true",
                    help="print the CPU baseline object of the workload and exit (no GPU use)")
    ap.add_argument("--no-batched", action="store_true", help="plain workload only")
    ap.add_argument("--no-served", action="store_true",
                    help="default line: skip the short served measurement")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    ap.add_argument("--no-extras", action="store_true",
                    help="timed steps only (no timeline, fast-variant, accuracy or render pass): "
                         "the command profilers capture")
    ap.add_argument("--requests", type=int, default=0, help="served: requests per rate point")
    ap.add_argument("--rates", type=float, nargs="*", default=None, help="served: arrival rates /s")
    ap.add_argument("--served-timeline", action="store_true",
                    help="served: record the step kernels' in-graph timeline per rate point")
    ap.add_argument("--no-plain", action="store_true",
                    help="served: skip the back-to-back plain solves of the request list")
    ap.add_argument("--near", default="reference", choices=["reference", "p2p"],
                    help="near field: the reference's cell monopoles, or exact pair sums")
    ap.add_argument("--float", default="exact", choices=["exact", "fast"],
                    help="float variant of the headline run (exact: the oracle's contract)")
    ap.add_argument("--fmm-steps", type=int, default=0,
                    help="FMM steps per bench step (0: the workload's own count)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def host_cpu():
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"nproc": os.cpu_count(), "model": model}


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


# ---------------------------------------------------------------- CPU oracle

class CpuRuns:
    """The CPU oracle (the reference algorithm restated in C, OpenMP) on the
    workload's scenes.  One run = reset every scene to its starting state and
    advance it `steps` FMM steps, the same unit the GPU bench step times."""

    def __init__(self, w, near="reference"):
        from oracle import oracle as O
        self.O = O
        if w["kind"] == "batched":
            self.scenes = workloads.batch_scenes(w)
        else:
            self.scenes = [workloads.scene(w)]
        self.params = [O.make_params(len(p), gravity=w["G"], softening=w["eps"], dt=w["dt"],
                                     near_mode=1 if near == "p2p" else 0) for p in self.scenes]
        self.bodies = sum(len(p) for p in self.scenes)

    def run(self, steps):
        states = [self.O.OracleState(p, prm) for p, prm in zip(self.scenes, self.params)]
        t0 = time.perf_counter()
        for st in states:
            st.step(steps)
        return time.perf_counter() - t0


def cpu_baseline_child(args):
    """cpu_baseline in a fresh interpreter that never touches the GPU, so the
    oracle's host threads do not share the process with CUDA and torch."""
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-baseline-only", "--workload", args.workload,
           "--cpu-seconds", str(args.cpu_seconds), "--near", args.near]
    try:
        out = subprocess.run(cmd, capture_output=True, text=True, check=True, timeout=600).stdout
        return json.loads(out.strip().splitlines()[-1])
    except (subprocess.SubprocessError, ValueError, IndexError) as e:
        return {"value": None, "unavailable": "CPU baseline process failed: %s" % type(e).__name__}


def cpu_baseline(w, seconds, near="reference", warmup=1):
    """All host threads: whole runs of the workload until `seconds` have
    passed (at least one); then one thread on a shorter sample."""
    runs = CpuRuns(w, near)
    O = runs.O
    cores = O.set_threads(os.cpu_count() or 1)
    steps = w["fmm_steps"]
    for _ in range(warmup):
        runs.run(steps)
    el, done = 0.0, 0
    while el < seconds or done == 0:
        el += runs.run(steps)
        done += 1
    value = runs.bodies * steps * done / el
    O.set_threads(1)
    s1 = max(1, min(steps, 8))
    e1 = runs.run(s1)
    O.set_threads(os.cpu_count() or 1)
    return {"value": value, "unit": "body-steps/s", "cores": cores, "kind": "port",
            "sample": "%d run(s) of %d FMM steps of the same workload (%d bodies, %s near field) "
                      "after %d warm-up run(s), %d host threads, %.1f s"
                      % (done, steps, runs.bodies, near, warmup, cores, el),
            "single_thread": {"value": runs.bodies * s1 / e1,
                              "sample": "%d FMM step(s) from the starting state, %.1f s" % (s1, e1)},
            "host": host_cpu()}


def reference_shader_rate(w, seconds=5.0, near="reference"):
    """The reference's own WGSL compute passes (translated to C++ into
    oracle/_ref/ by oracle/wgsl_transpile.py, run in the native harness's
    dispatch order) on all host threads: FMM frames of the workload's first
    scene from its starting state until `seconds` have passed.  Reported
    beside the oracle port, which stays the baseline value: the port is the
    faster of the two, so ratios against it are the conservative ones."""
    if near != "reference":
        return {"unavailable": "the reference shader has no P2P near field"}
    try:
        import numpy as np
        from oracle import oracle as O, wgsl_ref as W
        if not W.available():
            return {"unavailable": "no translation of the reference shader on this machine "
                                   "(oracle/_ref/ is generated where the reference checkout is)"}
        W.build()
        cores = W.set_threads(0)
        p = workloads.batch_scenes(w)[0] if w["kind"] == "batched" else workloads.scene(w)
        n = len(p)
        depth, cells, scale = O.plan(n)
        cfg = W.config(n, depth, cells, scale, gravity=w["G"], softening=w["eps"], dt=w["dt"])
        st = W.RefState(p.view(np.float32).ravel(), cfg)
        st.frames(1)  # warm-up
        frames, t0 = 0, time.perf_counter()
        while frames == 0 or time.perf_counter() - t0 < seconds:
            st.frames(1)
            frames += 1
        el = time.perf_counter() - t0
        return {"value": n * frames / el, "unit": "body-steps/s", "cores": cores,
                "kind": "reference",
                "sample": "%d FMM frame(s) of a %d-body scene of the workload after 1 warm-up "
                          "frame, %d host threads, %.1f s" % (frames, n, cores, el),
                "code": "src/rainbow_fmm.wgsl compute passes translated to C++ "
                        "(oracle/wgsl_transpile.py), native/main.rs dispatch order"}
    except Exception as e:  # a failed build or run never fails the bench line
        return {"unavailable": "reference shader timing failed: %s" % type(e).__name__}


def run_reference(args, w):
    """The reference arm: the CPU oracle on the same config, same protocol
    as cpu_baseline (each bench step resets the scene and runs the workload's
    FMM steps); a bounded sample of those steps when the whole run would
    exceed REFERENCE_BUDGET_S."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    if w["kind"] == "served":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no request server "
                          "(its only loop is native/main.rs:522-534); the served workload has no "
                          "CPU counterpart"}), flush=True)
        return 0
    runs = CpuRuns(w, args.near)
    O = runs.O
    cores = O.set_threads(os.cpu_count() or 1)
    steps = w["fmm_steps"]
    probe = runs.run(1)  # one FMM step: sizes the sample
    est = probe * steps * (args.warmup + args.steps)
    if est > REFERENCE_BUDGET_S:
        steps = max(1, int(steps * REFERENCE_BUDGET_S / est))
    for _ in range(args.warmup):
        runs.run(steps)
    times = [runs.run(steps) for _ in range(args.steps)]
    total = sum(times)
    value = runs.bodies * steps * args.steps / total
    line = {
        "impl": "reference", "metric": "body-steps/s", "value": value, "unit": "body-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded): " + w["desc"],
        "config": {"workload": args.workload, "bodies": runs.bodies,
                   "fmm_steps_per_bench_step": steps,
                   "implementation": "CPU oracle port of the reference compute passes "
                                     "(reference wgpu/Vulkan harness unavailable on this box)"},
        "cpu_baseline": {"value": value, "unit": "body-steps/s", "cores": cores, "kind": "port",
                         "sample": "%d bench steps of %d FMM steps (scene reset each), %d host "
                                   "threads" % (args.steps, steps, cores),
                         "host": host_cpu()},
        "e2e": {"value": value, "unit": "body-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    line["cpu_baseline"]["reference_shader"] = reference_shader_rate(w, near=args.near)
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU helpers

def timed_events(torch, stream, flush, fn, k):
    """k calls of fn, each bracketed by CUDA events on `stream`, L2 flushed
    before each (outside the events); returns the summed device ms."""
    st = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    en = [torch.cuda.Event(enable_timing=True) for _ in range(k)]
    for j in range(k):
        flush.zero_()
        st[j].record(stream)
        fn()
        en[j].record(stream)
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in zip(st, en))


def timeline_pass(torch, stream, flush, handle, fn, k, fmm_steps, ms_per_step):
    """A second timed pass with the in-graph timeline on; returns its summary."""
    handle.set_timeline(True)
    fn()  # captures the stamped graphs
    torch.cuda.synchronize()
    ms = timed_events(torch, stream, flush, fn, k) / k
    tl = handle.timeline()
    handle.set_timeline(False)
    steps = max(tl["steps"], 1)
    per_step = {kk: {"busy_us": 1e3 * v["busy_ms"] / steps, "gap_us": 1e3 * v["gap_ms"] / steps}
                for kk, v in tl["kinds"].items()}
    return tl, {
        "steps_recorded": tl["steps"],
        "fmm_step_span_us": 1e3 * tl["span_ms"] / steps,
        "per_fmm_step": per_step,
        "busy_sum_us": sum(v["busy_us"] for v in per_step.values()),
        "gap_sum_us": sum(v["gap_us"] for v in per_step.values()),
        "bench_ms_per_step_with_timeline": ms,
        "bench_ms_per_step_without": ms_per_step,
        "fmm_step_us_from_bench": 1e3 * ms_per_step / fmm_steps,
        "timer": "%globaltimer stamps inside the graphs: first CTA begin (after its dependency "
                 "wait) to last CTA end, per launch; each graph's last run",
    }


def dominant_roofline(phases, timeline, work, workload, peak, peak_kind, event_ms):
    k = timeline["kinds"]["integrate"]
    ms = k["busy_ms"] / max(k["launches"], 1)
    alg = work["integrate"]["bytes"]
    achieved = alg / (ms * 1e-3) / 1e9
    return {"kernel": "k_integrate", "bound": "hbm", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": alg, "avg_launch_ms": ms,
            "avg_launch_timer": "in-graph %globaltimer (timeline pass)",
            "event_avg_launch_ms": event_ms,
            "event_timer": "CUDA events around direct (non-graph) launches of the same kernel",
            "traffic": traffic_for(workload), "phases": phases, "phase_work": work}


def float_variant_pass(args, torch, rfmm, stream, flush, handle, fn, body_steps, fmm_steps, peak,
                       peak_kind, fp32, clocks, work_fn):
    """The same bench steps with the fast float variant: value, per-phase
    rates from its own timeline pass, dominant-kernel roofline."""
    from rfmm import replicas, roofline
    handle.set_float_mode(rfmm.FLOAT_FAST)
    for _ in range(max(2, args.warmup)):
        fn()
    torch.cuda.synchronize()
    ms = timed_events(torch, stream, flush, fn, args.steps)
    value, _, slowest_s = replicas.reduce_throughput(body_steps * args.steps, ms * 1e-3)
    ms_per_step = slowest_s * 1e3 / args.steps
    tl, tl_summary = timeline_pass(torch, stream, flush, handle, fn, min(args.steps, 5), fmm_steps,
                                   ms_per_step)
    work = work_fn()
    phases = roofline.phases_roofline(work, tl, peak, fp32, peak_kind)
    k = tl["kinds"]["integrate"]
    ims = k["busy_ms"] / max(k["launches"], 1)
    ach = work["integrate"]["bytes"] / (ims * 1e-3) / 1e9
    return {"value": value, "unit": "body-steps/s", "ms_per_step": ms_per_step,
            "float_mode": "fast (contraction, approximate div/sqrt, hardware rsqrt)",
            "parity": "integer work bit-exact; fields rel rms <= 1e-5, accelerations rel rms "
                      "<= 1e-4 against the oracle (tests/test_gpu_fast_mode.py)",
            "roofline": {"kernel": "k_integrate", "bound": "hbm", "achieved": ach, "peak": peak,
                         "unit": "GB/s", "frac": ach / peak, "avg_launch_ms": ims,
                         "phases": phases},
            "timeline": tl_summary}


def pipelined_e2e(torch, pair, k, upload, solve, download):
    """Wall time of `k` end-to-end bench steps through the public C ABI with
    host buffers, two handles alternating.  `pair` holds two (handle, torch
    stream) pairs; upload(h) enqueues one bench step's host->device input
    copy (and the commit's sort), solve(h) its FMM steps, download(h) reads
    its result into host memory and returns once the bytes are there.  Bench
    step i runs on handle i % 2: while it computes, the next step's input is
    copied in on the other handle's stream, and the next solve waits (an
    event) only for this one's compute, so this step's device->host read
    overlaps the next solve.  Two solves never run at once (each keeps the
    L2 to itself); every step's copies stay inside the timed region."""
    ev = [torch.cuda.Event(), torch.cuda.Event()]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h0, s0 = pair[0]
    upload(h0)
    solve(h0)
    ev[0].record(s0)
    for i in range(k):
        hx, _ = pair[i % 2]
        if i + 1 < k:
            hy, sy = pair[(i + 1) % 2]
            upload(hy)
            sy.wait_event(ev[i % 2])
            solve(hy)
            ev[(i + 1) % 2].record(sy)
        download(hx)
    return time.perf_counter() - t0


def run_gpu_plain(args, w, torch, rfmm, stream, flush, rank, world, local):
    import numpy as np
    from rfmm import replicas, roofline

    n, fmm_steps = w["n"], args.fmm_steps or w["fmm_steps"]
    scene = workloads.scene(w)
    params = rfmm.default_params(gravity=w["G"], softening=w["eps"], dt=w["dt"])
    solver = rfmm.Solver(n, params)
    solver.set_stream(stream.cuda_stream)
    if args.near == "p2p":
        solver.set_near_mode(rfmm.NEAR_P2P)
    if args.float == "fast":
        solver.set_float_mode(rfmm.FLOAT_FAST)
    pristine = torch.from_numpy(scene.view(np.uint8).copy()).cuda()

    def bench_step():
        solver.upload_device(pristine.data_ptr(), pristine.numel())
        solver.step(fmm_steps)

    tuning = solver.tuning()
    # Project autotuner: launch shapes timed on this scene.  Not in the P2P
    # mode, whose step is the pair kernel (its trials of 64 steps would take
    # minutes and the tree-pass shapes do not matter there).
    if not args.no_autotune and args.near == "reference":
        solver.upload_device(pristine.data_ptr(), pristine.numel())
        tuning = solver.autotune(20)
    for _ in range(args.warmup):
        bench_step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clk = clocks_sampler(local)
    time.sleep(0.3)
    barrier()
    l0 = solver.launch_count()
    local_ms = timed_events(torch, stream, flush, bench_step, args.steps)
    barrier()
    launches = solver.launch_count() - l0
    clocks = clocks_summary(clk)
    value, _, slowest_s = replicas.reduce_throughput(n * fmm_steps * args.steps, local_ms * 1e-3)
    ms_per_step = slowest_s * 1e3 / args.steps
    solver.sync()
    if args.no_extras:
        solver.close()
        return {"metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "config": {"workload": args.workload, "bodies": n,
                           "fmm_steps_per_bench_step": fmm_steps, "extras": "skipped"},
                "clocks": clocks, "gpu_launches": launches}

    # Per-phase times inside the graphs, and the work of the tree the run ends on.
    tl, tl_summary = timeline_pass(torch, stream, flush, solver, bench_step, min(args.steps, 5),
                                   fmm_steps, ms_per_step)
    mom = solver.moments()
    tw = roofline.tree_work(mom, solver.depth)
    work = roofline.phase_work(n, tw)
    if args.near == "p2p":
        tw["p2p_pairs"] = roofline.p2p_pairs(mom, solver.depth)
        work["near_p2p"] = {"bytes": 32 * n, "flops": 20 * tw["p2p_pairs"]}
    peak, peak_kind = hbm_peak()
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    fp32 = roofline.fp32_peak_tflops(torch.cuda.get_device_properties(local).multi_processor_count,
                                     sm_mhz)
    phases = roofline.phases_roofline(work, tl, peak, fp32, peak_kind)
    # The same kernels launched directly between CUDA events (no graph, no PDL).
    solver.upload_device(pristine.data_ptr(), pristine.numel())
    prof = solver.profile_steps(fmm_steps)
    event_ms = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in prof.items()}
    roof = dominant_roofline(phases, tl, work, args.workload, peak, peak_kind, event_ms["integrate"])
    roof["tree"] = tw

    # The fast float variant on the same workload, same protocol.
    fast = None
    if args.near == "reference" and args.float == "exact":
        fast = float_variant_pass(args, torch, rfmm, stream, flush, solver, bench_step,
                                  n * fmm_steps, fmm_steps, peak, peak_kind, fp32, clocks,
                                  lambda: roofline.phase_work(
                                      n, roofline.tree_work(solver.moments(), solver.depth)))
        fast["force_rms_rel"], fast["force_max_rel"] = solver.force_error(4096, 1)
        solver.set_float_mode(rfmm.FLOAT_EXACT)

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
        serial = {"value": world * n * fmm_steps / e2e_s, "ms_per_step": 1e3 * e2e_s,
                  "timer": "host wall clock (median of %d), one handle: upload, solve and "
                           "download one after another" % len(e2e_times)}
        # The same calls on two handles, pipelined (copies of one bench step
        # overlap the neighbouring steps' compute).
        other = rfmm.Solver(n, params)
        other_stream = torch.cuda.Stream()
        other.set_stream(other_stream.cuda_stream)
        other.set_tuning(tuning)
        if args.near == "p2p":
            other.set_near_mode(rfmm.NEAR_P2P)
        if args.float == "fast":
            other.set_float_mode(rfmm.FLOAT_FAST)
        pair = [(solver, stream), (other, other_stream)]
        up = lambda h: h.upload_host_ptr(pin_in.data_ptr(), pin_in.numel())
        sol = lambda h: h.step(fmm_steps)
        down = lambda h: h.download_host_ptr(rfmm.BUF_PARTICLES, pin_out.data_ptr(), pin_out.numel())
        pipelined_e2e(torch, pair, 2, up, sol, down)  # warm-up: the second handle's graphs
        kp = max(2, args.e2e_steps)
        el = pipelined_e2e(torch, pair, kp, up, sol, down)
        other.close()
        e2e = {"value": world * n * fmm_steps * kp / el, "unit": "body-steps/s",
               "h2d_bytes_per_step": n * 32, "d2h_bytes_per_step": n * 32,
               "ms_per_step": 1e3 * el / kp,
               "timer": "host wall clock over %d bench steps through two handles on two streams "
                        "(one step's host copies overlap its neighbours' compute; the solves run "
                        "one at a time)" % kp,
               "serial": serial}

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
    solver.close()

    return {
        "metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, numpy PCG64): " + w["desc"],
        "config": {"workload": args.workload, "form": "plain single-scene solve",
                   "near_field": args.near, "float_mode": args.float,
                   "bodies": n, "fmm_steps_per_bench_step": fmm_steps, "depth": tw["depth"],
                   "cells": tw["cells"], "fixed_point_scale": rfmm.plan_unclamped(n)[2],
                   "l2": "flushed between timed steps (512 MiB write outside the events)",
                   "parallelism": "replicas x%d" % world},
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roof,
        "timeline": tl_summary, "kernel_event_avg_ms": event_ms, "tuning": tuning.as_dict(),
        "accuracy": accuracy, "render": render, "fast_float": fast,
    }


def run_gpu_batched(args, w, torch, rfmm, stream, flush, rank, world, local):
    """Batched form vs the same scenes back to back through plain handles."""
    import numpy as np
    from rfmm import replicas, roofline

    all_scenes = workloads.batch_scenes(w)
    mine = replicas.shard_scenes([len(p) for p in all_scenes], world)[rank]
    ps = [all_scenes[i] for i in mine]
    sizes = [len(p) for p in ps]
    bodies = sum(sizes)
    fmm_steps = w["fmm_steps"]
    params = rfmm.default_params(gravity=w["G"], softening=w["eps"], dt=w["dt"])
    dev = [torch.from_numpy(p.view(np.uint8).copy()).cuda() for p in ps]
    batch = rfmm.Batch(sizes, [params] * len(ps))
    batch.set_stream(stream.cuda_stream)
    dev_ptrs = [d.data_ptr() for d in dev]

    def batched_step():
        batch.upload_device_all(dev_ptrs)  # one copy launch for all scenes
        batch.commit()
        batch.step(fmm_steps)

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
    local_ms = timed_events(torch, stream, flush, batched_step, args.steps)
    if world > 1:
        torch.distributed.barrier()
    launches = batch.launch_count() - l0
    clocks = clocks_summary(clk)
    value, _, slowest_s = replicas.reduce_throughput(bodies * fmm_steps * args.steps, local_ms * 1e-3)
    ms_per_step = slowest_s * 1e3 / args.steps
    if args.no_extras and args.workload == "batched_256":
        batch.close()
        return {"metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
                "config": {"workload": "batched_256", "scenes": len(ps), "bodies": bodies,
                           "fmm_steps_per_bench_step": fmm_steps, "extras": "skipped"},
                "clocks": clocks, "gpu_launches": launches}

    tl, tl_summary = timeline_pass(torch, stream, flush, batch, batched_step, min(args.steps, 3),
                                   fmm_steps, ms_per_step)
    moms = [np.empty(pl[1], rfmm.MOMENT_DTYPE) for pl in batch.plans]
    batch.download_all_into(rfmm.BUF_MOMENTS, [a.ctypes.data for a in moms])
    work = None
    for m, pl, nb in zip(moms, batch.plans, sizes):
        work = roofline.add_work(work, roofline.phase_work(nb, roofline.tree_work(m, pl[0])))
    peak, peak_kind = hbm_peak()
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    fp32 = roofline.fp32_peak_tflops(torch.cuda.get_device_properties(local).multi_processor_count,
                                     sm_mhz)
    phases = roofline.phases_roofline(work, tl, peak, fp32, peak_kind)
    prof = batch.profile_steps(fmm_steps)
    event_ms = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in prof.items()}
    roof = dominant_roofline(phases, tl, work, "batched_256", peak, peak_kind, event_ms["integrate"])

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
    plain_ms = timed_events(torch, stream, flush, plain_step, plain_k)
    plain_value = bodies * fmm_steps * plain_k / (plain_ms * 1e-3)
    for s in solvers:
        s.close()

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
        e2e_s = statistics.median(e2e_times)
        serial = {"value": world * bodies * fmm_steps / e2e_s, "ms_per_step": 1e3 * e2e_s,
                  "timer": "host wall clock (median of %d), one batch handle: upload, solve and "
                           "download one after another" % len(e2e_times)}
        other = rfmm.Batch(sizes, [params] * len(ps))
        other_stream = torch.cuda.Stream()
        other.set_stream(other_stream.cuda_stream)
        other.set_tuning(batch.tuning())
        pair = [(batch, stream), (other, other_stream)]

        def up(b):
            for i, t in enumerate(pin):
                rfmm._check(rfmm.lib().rfmm_batch_upload(b._h, i, t.data_ptr(), t.numel()), "upload")
            b.commit()

        sol = lambda b: b.step(fmm_steps)
        down = lambda b: b.download_all_into(rfmm.BUF_PARTICLES, out_ptrs)
        pipelined_e2e(torch, pair, 2, up, sol, down)  # warm-up: the second handle's graphs
        kp = max(2, args.e2e_steps)
        el = pipelined_e2e(torch, pair, kp, up, sol, down)
        other.close()
        e2e = {"value": world * bodies * fmm_steps * kp / el, "unit": "body-steps/s",
               "h2d_bytes_per_step": bodies * 32, "d2h_bytes_per_step": bodies * 32,
               "ms_per_step": 1e3 * el / kp,
               "timer": "host wall clock over %d bench steps through two batch handles on two "
                        "streams (one step's host copies overlap its neighbours' compute; the "
                        "solves run one at a time)" % kp,
               "serial": serial}
    batch.close()
    return {
        "metric": "body-steps/s", "value": value, "unit": "body-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, numpy PCG64): " + w["desc"],
        "config": {"workload": "batched_256", "form": "batched (all scenes per launch)",
                   "scenes": len(ps), "bodies": bodies, "fmm_steps_per_bench_step": fmm_steps,
                   "l2": "flushed between timed steps (512 MiB write outside the events)",
                   "parallelism": "scenes sharded over %d rank(s)" % world},
        "plain_back_to_back": {"value": plain_value, "unit": "body-steps/s",
                               "timed_steps": plain_k,
                               "form": "one plain handle per scene, solved one after another"},
        "batched_over_plain": value / world / plain_value,
        "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roof,
        "timeline": tl_summary, "kernel_event_avg_ms": event_ms, "tuning": tuning.as_dict(),
    }


def gpu_setup(world, local):
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from rfmm import build as pkg_build
    pkg_build.build()
    import rfmm
    # A real (non-default) stream shared by torch's events/flush and the solver.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device="cuda")
    return torch, rfmm, stream, flush


def run_gpu(args, w):
    rank, world, local = dist_env()
    torch, rfmm, stream, flush = gpu_setup(world, local)
    if w["kind"] == "batched":
        line = run_gpu_batched(args, w, torch, rfmm, stream, flush, rank, world, local)
    else:
        line = run_gpu_plain(args, w, torch, rfmm, stream, flush, rank, world, local)
        if args.workload == "plummer_1m" and not args.no_batched and args.near == "reference":
            b = run_gpu_batched(args, workloads.WORKLOADS["batched_256"], torch, rfmm, stream,
                                flush, rank, world, local)
            line["batched"] = {k: b[k] for k in ("value", "unit", "ms_per_step", "data", "config",
                                                 "plain_back_to_back", "batched_over_plain",
                                                 "clocks", "e2e", "gpu_launches", "roofline",
                                                 "timeline", "tuning")}
        if (args.workload == "plummer_1m" and not args.no_served and args.near == "reference"
                and world == 1):
            line["served"] = served_summary(args, torch, rfmm, local)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_child(args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ------------------------------------------------------------------ serving

def served_summary(args, torch, rfmm, local):
    """A short served measurement for the default line: 4,000 requests of the
    served workload's distribution, one rate below saturation (latency) and
    one above it (throughput), and the same list back to back through plain
    handles.  A short run's throughput includes the fill and drain of the
    slots, so it reads below the full sweep's (--workload served)."""
    w = workloads.WORKLOADS["served"]
    count, rates = 4000, [1000.0, 3000.0]
    sweep, plain_value, clocks, pool = served_sweep(args, w, torch, rfmm, local, count, rates, True)
    top = max(sweep, key=lambda r: r["body_steps_per_s"])
    return {"value": top["body_steps_per_s"], "unit": "body-steps/s",
            "requests_per_rate": count, "body_steps_per_rate": pool.body_steps(),
            "rates": [{k: r[k] for k in ("offered_rate_per_s", "achieved_rate_per_s", "p50_ms",
                                          "p99_ms", "body_steps_per_s", "wall_s", "worker")}
                      for r in sweep],
            "plain_back_to_back": plain_value,
            "served_over_plain": top["body_steps_per_s"] / plain_value if plain_value else None,
            "clocks": clocks,
            "data": "synthetic (seeded, numpy PCG64): " + w["desc"],
            "note": "short form of --workload served (10,000 requests per rate, 50-2,000 req/s); "
                    "the fill and drain of the slots weigh more in a short run"}


def served_sweep(args, w, torch, rfmm, local, count, rates, with_plain, timeline=False):
    """Continuous-batching server under Poisson arrivals (open loop), against
    the same request list solved back to back through plain handles.

    Producer threads submit each request at its scheduled arrival time and
    pass that time to the server (rfmm_server_submit_at), so latency runs from
    the scheduled arrival whether or not a submission starts late; a
    collector thread takes the results as they finish.  The achieved
    submission rate and the producers' lag behind the schedule are reported
    beside the offered rate.  Returns (sweep, plain body-steps/s or None,
    clocks, pool).
    """
    import threading
    import numpy as np

    pool = workloads.served_pool(w, count)
    params = rfmm.default_params(gravity=w["G"], softening=w["eps"], dt=w["dt"])
    producers, collectors = 8, 4
    staging = 24 << 30  # pinned host staging of the server (inputs 18 GiB, results 6 GiB)
    body_steps = pool.body_steps()
    fmode = rfmm.FLOAT_FAST if args.float == "fast" else rfmm.FLOAT_EXACT

    # Warm-up: module load and graph captures on a small server.
    warm = rfmm.Server(max_bodies=w["n_max"], memory_budget_bytes=2 << 30, max_slots=2,
                       max_chunk_steps=4, float_mode=fmode)
    for i in range(min(3, count)):
        rid = warm.submit(pool.bodies(i), int(pool.steps[i]), params)
        warm.wait(rid, 600000)
        warm.result(rid)
    warm.close()

    sweep = []
    clk = None
    for ri, rate in enumerate(rates):
        srv = rfmm.Server(max_bodies=w["n_max"], memory_budget_bytes=w["budget"],
                          max_chunk_steps=4, staging_bytes=staging, float_mode=fmode,
                          timeline=timeline)
        arrivals = np.cumsum(np.random.default_rng(w["seed"] + ri).exponential(1.0 / rate, count))
        ids = [None] * count
        actual = np.zeros(count)
        errors = []
        if ri == len(rates) - 1:
            clk = clocks_sampler(local)
        offset = srv.clock() - time.perf_counter()  # server clock minus this clock
        t0 = time.perf_counter() + 0.05

        def producer(k):
            try:
                for i in range(k, count, producers):
                    d = t0 + arrivals[i] - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                    actual[i] = time.perf_counter()
                    ids[i] = srv.submit_at(pool.bodies(i), int(pool.steps[i]), params,
                                           t0 + arrivals[i] + offset)
            except Exception as e:  # surfaced after the run
                errors.append(e)

        def collector(k):
            try:
                for i in range(k, count, collectors):
                    while ids[i] is None and not errors:
                        time.sleep(0.0002)
                    if errors:
                        return
                    srv.wait(ids[i], 3600000)
                    srv.result(ids[i])
            except Exception as e:
                errors.append(e)

        ths = [threading.Thread(target=producer, args=(k,)) for k in range(producers)]
        ths += [threading.Thread(target=collector, args=(k,)) for k in range(collectors)]
        for th in ths:
            th.start()
        for th in ths:
            th.join()
        if errors:
            raise errors[0]
        wall = time.perf_counter() - t0
        st = srv.stats()
        tl = srv.timeline() if timeline else None
        srv.close()
        lag = (actual - (t0 + arrivals)) * 1e3
        sweep.append({"offered_rate_per_s": rate,
                      "achieved_rate_per_s": (count - 1) / (actual.max() - actual.min()),
                      "submit_lag_ms": {"p50": float(np.percentile(lag, 50)),
                                        "p99": float(np.percentile(lag, 99)),
                                        "max": float(lag.max())},
                      "requests": count, "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
                      "mean_ms": st["mean_ms"], "max_ms": st["max_ms"],
                      "body_steps_per_s": st["body_steps_per_s"], "wall_s": wall,
                      "slots": st["slots"], "device_bytes": st["device_bytes"],
                      "worker": {k: st[k] for k in ("chunks", "mean_active_slots",
                                                    "pageable_inputs", "worker_gpu_wait_ms",
                                                    "worker_admit_ms", "worker_lists_ms",
                                                    "worker_step_ms", "worker_retire_ms",
                                                    "gpu_step_ms", "gpu_between_ms")}})
        if tl is not None:
            sweep[-1]["timeline"] = {
                "note": "most recent run of each captured step graph",
                "steps": tl["steps"], "span_ms_per_step": tl["span_ms"] / max(tl["steps"], 1),
                "busy_ms_per_launch": {k: v["busy_ms"] / v["launches"]
                                       for k, v in tl["kinds"].items() if v["launches"]}}
    clocks = clocks_summary(clk)

    # The same request list back to back through plain handles: each request
    # gets its own handle (created and destroyed outside the timer), then its
    # upload, steps and download are timed on the host clock.
    plain_s = 0.0
    for i in range(count if with_plain else 0):
        s = rfmm.Solver(int(pool.n[i]), params)
        s.set_float_mode(fmode)
        torch.cuda.synchronize()
        t = time.perf_counter()
        s.upload(pool.bodies(i))
        s.step(int(pool.steps[i]))
        s.particles()
        plain_s += time.perf_counter() - t
        s.close()
    plain_value = body_steps / plain_s if plain_s > 0 else None
    return sweep, plain_value, clocks, pool


def run_gpu_served(args, w):
    import numpy as np

    rank, world, local = dist_env()
    torch, rfmm, stream, flush = gpu_setup(world, local)
    count = args.requests or w["requests"]
    rates = args.rates or w["rates"]
    sweep, plain_value, clocks, pool = served_sweep(args, w, torch, rfmm, local, count, rates,
                                                    not args.no_plain, args.served_timeline)
    body_steps = pool.body_steps()
    producers, collectors = 8, 4
    staging = 24 << 30
    top = max(sweep, key=lambda r: r["body_steps_per_s"])
    line = {
        "metric": "body-steps/s", "value": top["body_steps_per_s"], "unit": "body-steps/s",
        "n_gpus": world, "steps": count, "warmup": 3, "ms_per_step": top["wall_s"] * 1e3 / count,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded, numpy PCG64): " + w["desc"],
        "config": {"workload": args.workload, "form": "served (continuous batching)",
                   "float_mode": args.float,
                   "requests_per_rate": count, "body_steps_per_rate": body_steps,
                   "memory_budget_bytes": w["budget"], "slot_capacity": w["n_max"],
                   "producer_threads": producers, "collector_threads": collectors,
                   "staging_bytes": staging, "sweep": sweep,
                   "timer": "host monotonic clock, scheduled arrival to result in host memory",
                   "parallelism": "1 GPU"},
        "plain_back_to_back": {"value": plain_value, "unit": "body-steps/s",
                               "requests": count,
                               "timer": "host clock around upload + steps + download per request "
                                        "(handle creation outside)"},
        "served_over_plain": top["body_steps_per_s"] / plain_value if plain_value else None,
        "clocks": clocks,
        "e2e": {"value": top["body_steps_per_s"], "unit": "body-steps/s",
                "h2d_bytes_per_step": int(np.sum(pool.n) * 32 / count),
                "d2h_bytes_per_step": int(np.sum(pool.n) * 32 / count),
                "note": "a step is one request; the served path is end to end by construction"},
        "gpu_launches": None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse_args()
    w = workloads.WORKLOADS[args.workload]
    if args.cpu_baseline_only:
        line = cpu_baseline(w, args.cpu_seconds, args.near)
        line["reference_shader"] = reference_shader_rate(w, near=args.near)
        print(json.dumps(line), flush=True)
        return 0
    if args.impl == "reference":
        return run_reference(args, w)
    if w["kind"] == "served":
        return run_gpu_served(args, w)
    return run_gpu(args, w)


if __name__ == "__main__":
    sys.exit(main())

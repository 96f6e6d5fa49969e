"""Regenerates tests/golden/reference_wgsl_digests.json from the reference's own shader code.

Each case runs the reference's WGSL compute passes (src/rainbow_fmm.wgsl),
translated to C++ by oracle/wgsl_transpile.py and driven in the native
harness's dispatch order (oracle/wgsl_ref_harness.cpp, after
native/main.rs:362-451), and records FNV-1a digests (the harness's digest,
native/main.rs:152-163) of:
  * the seeded galaxy (`initialize`) for galaxy cases;
  * moments and fields after one field solve (the harness's digest block);
  * particles, moments and fields after `frames` full frames.
The benchmarked workloads (uniform_64k, plummer_1m, clusters_5m and the 256
scenes of batched_256) are among the cases.  The CPU tests check the oracle
against these digests, the GPU tests the CUDA path.

Needs the reference checkout (RFMM_REFERENCE_DIR, default /root/reference);
takes a few minutes on 8 cores:

    python tests/golden/make_reference_golden.py
"""
import json
import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "fmm-rainbow_gb300"))
OUT = os.path.join(HERE, "reference_wgsl_digests.json")

HARNESS = dict(gravity=0.34, softening=0.012, dt=0.0009)   # native/main.rs:57-59
BENCH = dict(gravity=1.0, softening=1e-3, dt=5e-4)
CONTROL = dict(control_point=(0.1, -0.05, 0.02, 1.0), control_strength=2.0, control_radius=0.2)

CASES = [
    # The harness's own scene and parameters (native/main.rs:165-454).
    dict(name="galaxy_16384", input=["galaxy", 16384], params=HARNESS, frames=3),
    dict(name="galaxy_65536", input=["galaxy", 65536], params=HARNESS, frames=2),
    dict(name="galaxy_300000", input=["galaxy", 300000], params=HARNESS, frames=2),
    # The control field's three modes (wgsl:659-689).
    dict(name="galaxy_control_pull", input=["galaxy", 16384], frames=3,
         params=dict(HARNESS, control_axis_mode=(0.3, 0.8, -0.2, 1.0), **CONTROL)),
    dict(name="galaxy_control_push", input=["galaxy", 16384], frames=3,
         params=dict(HARNESS, control_axis_mode=(0.3, 0.8, -0.2, 2.0), **CONTROL)),
    dict(name="galaxy_control_vortex", input=["galaxy", 16384], frames=3,
         params=dict(HARNESS, control_axis_mode=(0.3, 0.8, -0.2, 3.0), **CONTROL)),
    # The benchmarked workloads, at full size.
    dict(name="uniform_64k", input=["workload", "uniform_64k"], frames=1,
         params=dict(gravity=1.0, softening=1e-3, dt=1e-3)),
    dict(name="plummer_1m", input=["workload", "plummer_1m"], params=BENCH, frames=60),
    dict(name="clusters_5m", input=["workload", "clusters_5m"], frames=5,
         params=dict(gravity=1.0, softening=5e-4, dt=5e-4)),
    # Smaller scenes and edge cases.
    dict(name="plummer_20000", input=["scene", "plummer", 20000, 5], params=BENCH, frames=3),
    dict(name="clusters_40000", input=["scene", "clusters", 40000, 9], params=BENCH, frames=2),
    dict(name="outside_box_5000", input=["outside", 5000, 2], params=BENCH, frames=3),
    dict(name="one_leaf_3000", input=["one_leaf", 3000, 4], params=BENCH, frames=3),
    dict(name="tiny_1", input=["scene", "plummer", 1, 1], params=BENCH, frames=3),
    dict(name="tiny_17", input=["scene", "plummer", 17, 1], params=BENCH, frames=3),
    dict(name="fast_speed_8000", input=["scene", "plummer", 8000, 8], frames=2,
         params=dict(gravity=1.0, softening=1e-3, dt=4e-3, speed=2.5)),
    # Plan overrides (rfmm_params depth / fixed_point_scale), which the shader
    # takes through its uniform block like the planner's values.
    dict(name="plummer_20000_depth6", input=["scene", "plummer", 20000, 5], frames=2,
         params=dict(BENCH, depth=6)),
    dict(name="clusters_40000_depth4", input=["scene", "clusters", 40000, 9], frames=2,
         params=dict(BENCH, depth=4)),
    dict(name="uniform_30000_scale128", input=["scene", "uniform", 30000, 7], frames=2,
         params=dict(BENCH, scale=128.0)),
]
BATCH = dict(name="batched_256", workload="batched_256", frames=4, params=BENCH)


def make_input(spec):
    """Input particles of a case (None for galaxy cases: seeded by `initialize`)."""
    import numpy as np
    from rfmm import scenes, workloads
    kind = spec[0]
    if kind == "galaxy":
        return None
    if kind == "workload":
        return workloads.scene(workloads.WORKLOADS[spec[1]])
    if kind == "scene":
        return scenes.make(spec[1], spec[2], spec[3])
    if kind == "outside":  # far outside the world box: soft wall and clamp paths (wgsl:736-752)
        p = scenes.make("uniform", spec[1], spec[2]).copy()
        p["pos"] *= np.float32(3.5)
        p["vel"] = np.float32(0.7)
        return p
    if kind == "one_leaf":  # every body in one leaf cell
        p = scenes.make("uniform", spec[1], spec[2]).copy()
        p["pos"] = p["pos"] * np.float32(1e-3) + np.float32(0.3)
        return p
    raise ValueError(kind)


def n_of(spec):
    from rfmm import workloads
    if spec[0] in ("galaxy", "outside", "one_leaf"):
        return spec[1]
    if spec[0] == "workload":
        return workloads.WORKLOADS[spec[1]]["n"]
    return spec[2]


def ref_config(n, params):
    """The uniform values of a case: the planner's depth and scale unless the
    case overrides them (keys `depth`, `scale`)."""
    from oracle import oracle as O, wgsl_ref as W
    depth, _, scale = O.plan(n)
    kw = dict(params)
    depth = kw.pop("depth", depth)
    scale = kw.pop("scale", scale)
    return W.config(n, depth, O.lib().oracle_total_cells(depth), scale, **kw)


def run_case(case):
    import numpy as np
    from oracle import oracle as O, wgsl_ref as W
    W.set_threads(1)  # one process per case
    n = n_of(case["input"])
    cfg = ref_config(n, case["params"])
    p = make_input(case["input"])
    entry = {"input": case["input"], "n": n, "params": case["params"], "frames": case["frames"],
             "depth": cfg.depth, "cells": cfg.cells, "scale": cfg.scale}
    if p is None:
        raw = W.seed(cfg)
        entry["seed_particles"] = O.fnv1a(raw)
    else:
        raw = p.view(np.float32).ravel().copy()
        entry["input_particles"] = O.fnv1a(p)
    st = W.RefState(raw, cfg)
    st.solve_fields()
    entry["solve_moments"] = O.fnv1a(st.moments)
    entry["solve_fields"] = O.fnv1a(st.fields)
    st = W.RefState(raw, cfg)
    st.frames(case["frames"])
    entry["frame_particles"] = O.fnv1a(st.particles)
    entry["frame_moments"] = O.fnv1a(st.moments)
    entry["frame_fields"] = O.fnv1a(st.fields)
    return case["name"], entry


def run_batch_scene(args):
    import numpy as np
    from oracle import oracle as O, wgsl_ref as W
    from rfmm import workloads
    W.set_threads(1)
    i, frames, params = args
    p = workloads.batch_scenes(workloads.WORKLOADS[BATCH["workload"]])[i]
    cfg = ref_config(len(p), params)
    st = W.RefState(p.view(np.float32).ravel().copy(), cfg)
    st.frames(frames)
    return i, [O.fnv1a(p), len(p), O.fnv1a(st.particles), O.fnv1a(st.moments), O.fnv1a(st.fields)]


def main():
    from oracle import wgsl_ref as W
    W.build()
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(8, os.cpu_count() or 1)) as pool:
        cases = dict(pool.map(run_case, sorted(CASES, key=lambda c: -n_of(c["input"]) * c["frames"])))
        nscenes = 256
        scenes_out = dict(pool.map(run_batch_scene,
                                   [(i, BATCH["frames"], BATCH["params"]) for i in range(nscenes)]))
    data = {
        "generator": "tests/golden/make_reference_golden.py",
        "source": "src/rainbow_fmm.wgsl compute passes, translated by oracle/wgsl_transpile.py, "
                  "dispatched in the order of native/main.rs",
        "digest": "FNV-1a 32 over the buffer bytes (native/main.rs:152-163)",
        "cases": {c["name"]: cases[c["name"]] for c in CASES},
        "batched_256": {"frames": BATCH["frames"], "params": BATCH["params"],
                        "scenes": [scenes_out[i] for i in range(nscenes)],
                        "columns": ["input_particles", "n", "frame_particles", "frame_moments",
                                    "frame_fields"]},
    }
    with open(OUT, "w") as fh:
        json.dump(data, fh, indent=1)
        fh.write("\n")
    print("wrote", OUT)


if __name__ == "__main__":
    main()

"""The CUDA path against the reference's own shader code (GPU).

Each case of tests/golden/reference_wgsl_digests.json -- digests that the
reference's WGSL compute passes (src/rainbow_fmm.wgsl) produced when
translated by oracle/wgsl_transpile.py and dispatched in the native
harness's order (native/main.rs:362-451) -- is run through the C ABI and its
FNV-1a digests (native/main.rs:152-163) compared: the GPU-seeded galaxy, one
field solve, and multi-frame runs, including the benchmarked workloads at
full size (plummer_1m over all 60 frames at the default resort interval,
clusters_5m, uniform_64k) and all 256 scenes of the batched workload in one
batch.  No oracle runs here: the reference's digests are the expected values.
"""
import json
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "reference_wgsl_digests.json")))
CASES = GOLDEN["cases"]


def _params(R, prm):
    kw = dict(prm)
    if "scale" in kw:  # a plan override: rfmm_params.fixed_point_scale
        kw["fixed_point_scale"] = kw.pop("scale")
    return R.default_params(**kw)


@pytest.mark.parametrize("name", list(CASES))
def test_gpu_matches_reference_shader(rfmm_mod, oracle_mod, name):
    import make_reference_golden as G
    R, O = rfmm_mod, oracle_mod
    g = CASES[name]
    p = G.make_input(g["input"])
    if p is not None and O.fnv1a(p) != g["input_particles"]:
        pytest.skip("%s: this platform's scene generator gives other input bits" % name)
    with R.Solver(g["n"], _params(R, g["params"])) as s:
        assert (s.depth, s.cells, s.scale) == (g["depth"], g["cells"], g["scale"])
        if p is None:
            s.seed_galaxy()
            assert s.digest(R.BUF_PARTICLES) == g["seed_particles"], "galaxy seed"
            p = s.particles()
        else:
            s.upload(p)
        s.solve_fields()
        assert s.digest(R.BUF_MOMENTS) == g["solve_moments"], "moments of one solve"
        assert s.digest(R.BUF_FIELDS) == g["solve_fields"], "fields of one solve"
        s.upload(p)
        s.step(g["frames"])
        assert s.digest(R.BUF_PARTICLES) == g["frame_particles"], "particles after the frames"
        assert s.digest(R.BUF_MOMENTS) == g["frame_moments"], "moments after the frames"
        assert s.digest(R.BUF_FIELDS) == g["frame_fields"], "fields after the frames"


def test_gpu_batch_matches_reference_shader(rfmm_mod, oracle_mod):
    import torch
    R, O = rfmm_mod, oracle_mod
    from rfmm import workloads
    B = GOLDEN["batched_256"]
    ps = workloads.batch_scenes(workloads.WORKLOADS["batched_256"])
    for i, (p, row) in enumerate(zip(ps, B["scenes"])):
        if O.fnv1a(p) != row[0]:
            pytest.skip("scene %d: this platform's scene generator gives other input bits" % i)
    prm = _params(R, B["params"])
    with R.Batch([len(p) for p in ps], [prm] * len(ps)) as b:
        dev = [torch.from_numpy(p.view(np.uint8).copy()).cuda() for p in ps]
        b.upload_device_all([d.data_ptr() for d in dev])
        b.commit()
        b.step(B["frames"])
        for i, row in enumerate(B["scenes"]):
            got = (b.digest(i, R.BUF_PARTICLES), b.digest(i, R.BUF_MOMENTS), b.digest(i, R.BUF_FIELDS))
            assert got == tuple(row[2:]), "scene %d after %d frames" % (i, B["frames"])


# Cases submitted together to one server: the 60-frame plummer_1m request
# runs through chunking and several periodic re-sorts while the others are
# admitted and retired around it; per-request parameters include the
# control field, speed and dt overrides.
SERVED = ["plummer_1m", "galaxy_control_vortex", "galaxy_control_pull", "clusters_40000",
          "fast_speed_8000", "plummer_20000", "outside_box_5000", "one_leaf_3000", "tiny_17",
          "uniform_64k", "galaxy_65536"]


def test_served_requests_match_reference_shader(rfmm_mod, oracle_mod):
    import threading
    import time
    import make_reference_golden as G
    R, O = rfmm_mod, oracle_mod
    reqs = []
    for name in SERVED:
        g = CASES[name]
        p = G.make_input(g["input"])
        if p is None:  # galaxy: seeded on the GPU, checked against the seed digest
            with R.Solver(g["n"], _params(R, g["params"])) as s:
                s.seed_galaxy()
                p = s.particles()
            assert O.fnv1a(p) == g["seed_particles"], name
        elif O.fnv1a(p) != g["input_particles"]:
            pytest.skip("%s: this platform's scene generator gives other input bits" % name)
        reqs.append((name, p, g))
    ids = []
    with R.Server(max_bodies=1 << 20, memory_budget_bytes=8 << 30, max_slots=4,
                  max_chunk_steps=4) as srv:
        def client(chunk):
            for name, p, g in chunk:
                ids.append((srv.submit(p, g["frames"], _params(R, g["params"])), name))
                time.sleep(0.003)  # arrivals while earlier requests run

        threads = [threading.Thread(target=client, args=(reqs[k::2],)) for k in range(2)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        results = {}
        for rid, name in ids:
            srv.wait(rid, 300000)
            results[name] = srv.result(rid)
        assert srv.stats()["completed"] == len(reqs)
    for name, got in results.items():
        assert O.fnv1a(got) == CASES[name]["frame_particles"], \
            "%s: served result differs from the reference shader's" % name


def test_noalloc_solve_matches_reference_shader(rfmm_mod, oracle_mod):
    """rfmm_solve_fields_noalloc (caller buffers, fixed scratch) against the
    reference's one-solve digests, for every planner-sized case it takes."""
    import torch
    import make_reference_golden as G
    R, O = rfmm_mod, oracle_mod
    checked = 0
    for name, g in CASES.items():
        n = g["n"]
        if n > (1 << 17) or "depth" in g["params"] or "scale" in g["params"]:
            continue
        p = G.make_input(g["input"])
        if p is None:
            with R.Solver(n, _params(R, g["params"])) as s:
                s.seed_galaxy()
                p = s.particles()
        elif O.fnv1a(p) != g["input_particles"]:
            continue
        dev = torch.from_numpy(p.view(np.uint8).copy()).cuda()
        mom = torch.zeros(g["cells"] * 16, dtype=torch.uint8, device="cuda")
        fld = torch.zeros(g["cells"] * 48, dtype=torch.uint8, device="cuda")
        stream = torch.cuda.current_stream()
        R.solve_fields_noalloc(dev.data_ptr(), n, _params(R, g["params"]), mom.data_ptr(),
                               fld.data_ptr(), stream.cuda_stream)
        assert R.noalloc_device_error(stream.cuda_stream) == (R.RFMM_OK, 0, 0)
        torch.cuda.synchronize()
        assert O.fnv1a(mom.cpu().numpy()) == g["solve_moments"], name
        assert O.fnv1a(fld.cpu().numpy()) == g["solve_fields"], name
        checked += 1
    assert checked >= 8

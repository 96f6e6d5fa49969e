"""Served form: requests admitted while others run, each result bit-identical
to the same scene solved alone through a plain handle."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _requests():
    from rfmm import scenes
    rng = np.random.default_rng(31)
    out = []
    for i in range(24):
        n = int(np.exp(rng.uniform(np.log(17), np.log(120000))))
        kind = ["uniform", "plummer", "clusters4"][i % 3]
        steps = int(rng.integers(1, 13))
        out.append((scenes.make(kind, n, 500 + i), steps, 0.5 + 0.1 * (i % 5)))
    return out


def test_served_results_match_plain_alone(rfmm_mod):
    R = rfmm_mod
    reqs = _requests()
    results = {}
    with R.Server(max_bodies=131072, memory_budget_bytes=2 << 30, max_slots=6,
                  max_chunk_steps=3) as srv:
        ids = []

        def client(chunk):
            for p, steps, g in chunk:
                ids.append((srv.submit(p, steps, R.default_params(gravity=g, softening=1e-3,
                                                                  dt=5e-4)), p, steps, g))
                time.sleep(0.002)  # arrivals while earlier requests are on the GPU

        threads = [threading.Thread(target=client, args=(reqs[k::3],)) for k in range(3)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        for rid, p, steps, g in ids:
            srv.wait(rid, 120000)
            results[rid] = (srv.result(rid), p, steps, g)
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["slots"] == 6
        assert st["p99_ms"] >= st["p50_ms"] > 0
    for rid, (got, p, steps, g) in results.items():
        with R.Solver(len(p), R.default_params(gravity=g, softening=1e-3, dt=5e-4)) as s:
            s.upload(p)
            s.step(steps)
            ref = s.particles()
        assert np.array_equal(_bits(got), _bits(ref)), (rid, len(p), steps)


def test_server_rejects_oversize_request(rfmm_mod):
    R = rfmm_mod
    from rfmm import scenes
    with R.Server(max_bodies=4096, memory_budget_bytes=1 << 28, max_slots=2) as srv:
        with pytest.raises(R.RFMMError):
            srv.submit(scenes.uniform(5000, seed=1), 2)
        rid = srv.submit(scenes.uniform(4096, seed=1), 2)
        srv.wait(rid)
        assert srv.result(rid).shape == (4096,)


def test_served_resorts_keep_results(rfmm_mod):
    """Requests long enough that the engine re-sorts its active slots (every
    16 steps) while they run, and requests staged before a re-sort flips the
    particle buffers but admitted after it: each result still equals the
    plain solve alone."""
    R = rfmm_mod
    from rfmm import scenes
    rng = np.random.default_rng(77)
    reqs = []
    for i in range(16):
        n = int(np.exp(rng.uniform(np.log(2000), np.log(90000))))
        reqs.append((scenes.make(["plummer", "clusters4", "uniform"][i % 3], n, 800 + i),
                     int(rng.integers(17, 46))))
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Server(max_bodies=131072, memory_budget_bytes=2 << 30, max_slots=4,
                  max_chunk_steps=5) as srv:
        ids = []
        for p, steps in reqs:
            ids.append(srv.submit(p, steps, prm))
            time.sleep(0.001)
        got = []
        for rid in ids:
            srv.wait(rid, 120000)
            got.append(srv.result(rid))
    for (p, steps), g in zip(reqs, got):
        with R.Solver(len(p), prm) as s:
            s.upload(p)
            s.step(steps)
            assert np.array_equal(_bits(g), _bits(s.particles())), (len(p), steps)


def test_server_fast_float_mode_and_timeline(rfmm_mod):
    """A server created with the fast float variant gives each request the
    plain fast solve's result bit for bit, and its timeline records the step
    kernels."""
    R = rfmm_mod
    from rfmm import scenes
    reqs = [(scenes.make(k, n, 860 + i), st) for i, (k, n, st) in
            enumerate([("plummer", 40000, 9), ("uniform", 20000, 20), ("clusters4", 60000, 5)])]
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Server(max_bodies=65536, memory_budget_bytes=1 << 30, max_slots=3, max_chunk_steps=4,
                  float_mode=R.FLOAT_FAST, timeline=True) as srv:
        ids = [srv.submit(p, steps, prm) for p, steps in reqs]
        got = []
        for rid in ids:
            srv.wait(rid, 120000)
            got.append(srv.result(rid))
        tl = srv.timeline()
    assert tl["steps"] > 0
    for kind in ("upward", "m2l", "l2l_near", "integrate"):
        assert tl["kinds"][kind]["launches"] > 0 and tl["kinds"][kind]["busy_ms"] > 0.0, kind
    for (p, steps), g in zip(reqs, got):
        with R.Solver(len(p), prm) as s:
            s.set_float_mode(R.FLOAT_FAST)
            s.upload(p)
            s.step(steps)
            assert np.array_equal(_bits(g), _bits(s.particles())), (len(p), steps)

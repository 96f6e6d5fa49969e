"""In-graph timeline of the step kernels (rfmm_set_timeline / rfmm_get_timeline).

The stamps must not change results, and the records must describe the graph
runs consistently: one record per kernel kind and step, busy and gap times
that add up to no more than each run's span.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_timeline_keeps_results_and_is_consistent(rfmm_mod):
    R = rfmm_mod
    from rfmm import scenes
    n = 200000
    p = scenes.plummer(n, seed=8)
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    out = []
    for on in (False, True):
        with R.Solver(n, prm) as s:
            s.set_timeline(on)
            s.upload(p)
            s.step(40)  # chunks of 16 + resort, 16 + resort, 8
            out.append((s.particles(), s.fields(), s.timeline()))
    assert np.array_equal(_bits(out[0][0]), _bits(out[1][0]))
    assert np.array_equal(_bits(out[0][1]), _bits(out[1][1]))
    assert out[0][2]["steps"] == 0  # nothing recorded without the timeline
    t = out[1][2]
    assert t["steps"] == 40
    k = t["kinds"]
    for kind in ("upward", "m2l", "l2l_near", "integrate"):
        assert k[kind]["launches"] == 40, kind
        assert k[kind]["busy_ms"] > 0.0, kind
    assert k["resort"]["launches"] == 2
    busy = sum(v["busy_ms"] for v in k.values())
    gaps = sum(v["gap_ms"] for v in k.values())
    assert busy + gaps <= t["span_ms"] * 1.0001 + 1e-6
    assert busy >= 0.3 * t["span_ms"]


def test_batch_timeline_records_every_kind(rfmm_mod):
    R = rfmm_mod
    from rfmm import scenes
    ps = [scenes.plummer(30000, seed=1), scenes.uniform(9000, seed=2), scenes.clusters(70000, seed=3)]
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Batch([len(q) for q in ps], [prm] * 3) as b:
        b.set_timeline(True)
        for i, q in enumerate(ps):
            b.upload(i, q)
        b.commit()
        b.step(20)
        t = b.timeline()
    assert t["steps"] == 20
    for kind in ("upward", "m2l", "l2l_near", "integrate"):
        assert t["kinds"][kind]["launches"] == 20, kind
    assert t["kinds"]["resort"]["launches"] == 1

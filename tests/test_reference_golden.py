"""The oracle against the reference's own shader code (CPU).

tests/golden/reference_wgsl_digests.json holds digests produced by the
reference's WGSL compute passes (src/rainbow_fmm.wgsl), translated to C++ by
oracle/wgsl_transpile.py and dispatched in the native harness's order
(native/main.rs:362-451); tests/golden/make_reference_golden.py wrote it.
These tests pin the oracle to those digests: the galaxy seed, one field
solve and multi-frame runs of the harness's scene, the three control-field
modes, the benchmarked workloads at full size (uniform_64k, plummer_1m 60
frames, clusters_5m, all 256 batched scenes) and edge cases.

Where the reference checkout is present, the translation also runs live:
full buffers against the oracle, and a planted mistake in a copy of the
shader text must be caught.
"""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "reference_wgsl_digests.json")))
CASES = GOLDEN["cases"]


def _params(O, n, prm):
    kw = dict(prm)
    for k in ("control_point", "control_axis_mode"):
        if k in kw:
            kw[k] = tuple(kw[k])
    return O.make_params(n, **kw)


@pytest.mark.parametrize("name", list(CASES))
def test_oracle_matches_reference_shader(oracle_mod, name):
    import make_reference_golden as G
    O = oracle_mod
    g = CASES[name]
    n = g["n"]
    params = _params(O, n, g["params"])
    assert (params.depth, params.scale) == (g["depth"], g["scale"])
    p = G.make_input(g["input"])
    if p is None:
        p = O.initialize(n, params)
        assert O.fnv1a(p) == g["seed_particles"], "galaxy seed"
    else:
        assert O.fnv1a(p) == g["input_particles"], "input scene differs from the fixture's"
    st = O.OracleState(p, params)
    st.solve_fields()
    assert O.fnv1a(st.moments) == g["solve_moments"], "moments of one solve"
    assert O.fnv1a(st.fields) == g["solve_fields"], "fields of one solve"
    st = O.OracleState(p, params)
    st.step(g["frames"])
    assert O.fnv1a(st.particles) == g["frame_particles"], "particles after %d frames" % g["frames"]
    assert O.fnv1a(st.moments) == g["frame_moments"], "moments after %d frames" % g["frames"]
    assert O.fnv1a(st.fields) == g["frame_fields"], "fields after %d frames" % g["frames"]


def test_oracle_matches_reference_shader_batched_256(oracle_mod):
    from rfmm import workloads
    O = oracle_mod
    B = GOLDEN["batched_256"]
    scenes = workloads.batch_scenes(workloads.WORKLOADS["batched_256"])
    assert len(scenes) == len(B["scenes"]) == 256
    for i, (p, row) in enumerate(zip(scenes, B["scenes"])):
        d_in, n, d_p, d_m, d_f = row
        assert (len(p), O.fnv1a(p)) == (n, d_in), "scene %d input" % i
        st = O.OracleState(p, _params(O, n, B["params"]))
        st.step(B["frames"])
        assert (O.fnv1a(st.particles), O.fnv1a(st.moments), O.fnv1a(st.fields)) == (d_p, d_m, d_f), \
            "scene %d after %d frames" % (i, B["frames"])


def _ref_module():
    from oracle import wgsl_ref as W
    if not W.shader_available():
        pytest.skip("reference checkout absent: the committed digests above stand in for it")
    return W


LIVE = [("galaxy", 16384, 2, {}),
        ("plummer", 20000, 3, dict(gravity=1.0, softening=1e-3, dt=5e-4)),
        ("clusters", 40000, 2, dict(gravity=1.0, softening=5e-4, dt=5e-4))]


@pytest.mark.parametrize("kind,n,frames,prm", LIVE)
def test_translated_reference_matches_oracle_full_buffers(oracle_mod, kind, n, frames, prm):
    W = _ref_module()
    O = oracle_mod
    from rfmm import scenes
    params = O.make_params(n, **prm)
    cfg = W.config(n, params.depth, O.lib().oracle_total_cells(params.depth), params.scale, **prm)
    p = O.initialize(n, params) if kind == "galaxy" else scenes.make(kind, n, 7)
    if kind == "galaxy":
        assert np.array_equal(W.seed(cfg).view(np.uint32), p.view(np.uint32).ravel())
    ref = W.RefState(p.view(np.float32).ravel(), cfg)
    st = O.OracleState(p, params)
    ref.solve_fields()
    st.solve_fields()
    assert np.array_equal(ref.moments, st.moments.view(np.uint32).ravel())
    assert np.array_equal(ref.fields.view(np.uint32), st.fields.view(np.uint32).ravel())
    ref.frames(frames)
    st.step(frames)
    for a, b, what in ((ref.particles, st.particles, "particles"), (ref.moments, st.moments, "moments"),
                       (ref.fields, st.fields, "fields")):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32).ravel()), what


# Edits of the shader text, each a one-token change the comparison must see:
# the M2L softening constant, the near-field stencil's self-skip, and the
# integrate's soft-wall damping.
PLANTED = [("0.06 * WORLD_HALF_EXTENT", "0.0601 * WORLD_HALF_EXTENT", "fields"),
           ("if (dx == 0 && dy == 0 && dz == 0) {", "if (dx == 0 && dy == 0 && dz == 2) {", "fields"),
           ("velocity[axis] *= 1.0 - absorb * 0.16;", "velocity[axis] *= 1.0 - absorb * 0.161;",
            "particles")]


@pytest.mark.parametrize("old,new,where", PLANTED)
def test_planted_shader_mistake_is_caught(oracle_mod, old, new, where):
    W = _ref_module()
    O = oracle_mod
    import make_reference_golden as G
    with open(W.SHADER) as fh:
        text = fh.read()
    assert text.count(old) == 1
    lib = W.build_variant(text.replace(old, new), "planted%d" % [x[0] for x in PLANTED].index(old))
    if where == "particles":
        p = G.make_input(["outside", 5000, 2])  # bodies in the wall band
        prm = dict(gravity=1.0, softening=1e-3, dt=5e-4)
    else:
        p = O.initialize(16384)
        prm = {}
    params = O.make_params(len(p), **prm)
    cfg = W.config(len(p), params.depth, O.lib().oracle_total_cells(params.depth), params.scale, **prm)
    ref = W.RefState(p.view(np.float32).ravel(), cfg, library=lib)
    st = O.OracleState(p, params)
    ref.frames(1)
    st.step(1)
    same_f = np.array_equal(ref.fields.view(np.uint32), st.fields.view(np.uint32).ravel())
    same_p = np.array_equal(ref.particles.view(np.uint32), st.particles.view(np.uint32).ravel())
    assert not (same_f and same_p), "the planted change went unnoticed"
    assert not (same_f if where == "fields" else same_p)


def test_missing_entry_point_is_reported(oracle_mod):
    """A shader whose pass the harness dispatches is gone fails loudly."""
    W = _ref_module()
    O = oracle_mod
    with open(W.SHADER) as fh:
        text = fh.read()
    assert text.count("fn near_all(") == 1
    lib = W.build_variant(text.replace("fn near_all(", "fn near_all_renamed("), "renamed")
    p = O.initialize(4096)
    params = O.make_params(4096)
    cfg = W.config(4096, params.depth, O.lib().oracle_total_cells(params.depth), params.scale)
    with pytest.raises(RuntimeError):
        W.RefState(p.view(np.float32).ravel(), cfg, library=lib).solve_fields()

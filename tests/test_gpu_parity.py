"""GPU parity: the CUDA path against the CPU oracle on the same inputs.

The solver is called through its C ABI (include/rfmm.h, via ctypes).  The
bar is bit-exact for the integer tree (moments, occupancy) and, because the
kernels follow the oracle's floating-point contract (binary32,
round-to-nearest, no contraction, IEEE div/sqrt, reference loop order, the
contract's own sin/cos/exp/pow/atan2), also bit-exact for fields and
particles, the galaxy seed and the control field.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(kind, n, seed=7):
    from rfmm import scenes
    return scenes.make(kind, n, seed)


def _oracle_params(O, n, gravity=1.0, softening=1e-3, dt=5e-4, **kw):
    return O.make_params(n, gravity=gravity, softening=softening, dt=dt, **kw)


def _solver(rfmm, n, gravity=1.0, softening=1e-3, dt=5e-4, **kw):
    return rfmm.Solver(n, rfmm.default_params(gravity=gravity, softening=softening, dt=dt, **kw))


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _assert_same(gpu, ref, what):
    g, r = _bits(gpu), _bits(ref)
    bad = np.nonzero(g != r)[0]
    assert len(bad) == 0, "%s differs in %d of %d words; first at %d: %r vs %r" % (
        what, len(bad), len(g), bad[0], g[bad[0]], r[bad[0]])


CASES = [
    ("uniform", 65536),    # the reference's CPU-runnable size, depth 5
    ("plummer", 16384),    # depth 4, dense adaptive core
    ("clusters", 40000),   # depth 5, eight clusters, ragged N
    ("uniform", 4096),     # below the exported planner clamp (unclamped plan)
    ("plummer", 262147),   # depth 6, N not a multiple of the body tile
]


@pytest.mark.parametrize("kind,n", CASES)
def test_solve_fields_bit_exact(rfmm_mod, oracle_mod, kind, n):
    O, R = oracle_mod, rfmm_mod
    p = _scene(kind, n)
    st = O.OracleState(p, _oracle_params(O, n))
    st.solve_fields()
    with _solver(R, n) as s:
        s.upload(p)
        s.solve_fields()
        _assert_same(s.moments(), st.moments, "moments")
        _assert_same(s.fields(), st.fields, "fields")
        assert s.digest(R.BUF_MOMENTS) == O.fnv1a(st.moments)
        assert s.digest(R.BUF_FIELDS) == O.fnv1a(st.fields)
        _assert_same(s.particles(), p, "particles (order restored)")


@pytest.mark.parametrize("kind,n", CASES[:3])
def test_steps_bit_exact(rfmm_mod, oracle_mod, kind, n):
    O, R = oracle_mod, rfmm_mod
    p = _scene(kind, n)
    st = O.OracleState(p, _oracle_params(O, n))
    st.step(5)
    with _solver(R, n) as s:
        s.set_resort_interval(2)  # exercise the resident-order refresh mid-run
        s.upload(p)
        s.step(5)
        _assert_same(s.particles(), st.particles, "particles after 5 steps")
        _assert_same(s.moments(), st.moments, "moments of the last step")
        _assert_same(s.fields(), st.fields, "fields of the last step")


def test_galaxy_seed_digest_solve(rfmm_mod, oracle_mod):
    """The reference harness's own scene (native/main.rs:423-454): the seed,
    the field solve and two steps, bit for bit (the seed's sin/cos/pow/atan2
    are the contract's own functions on both sides)."""
    O, R = oracle_mod, rfmm_mod
    n = 65536
    with R.Solver(n) as s:  # harness defaults: dt 0.0009, G 0.34, eps 0.012
        s.seed_galaxy()
        gp = s.particles()
        ref = O.initialize(n)
        _assert_same(gp, ref, "seeded particles")
        st = O.OracleState(ref, O.make_params(n))
        st.solve_fields()
        s.solve_fields()
        _assert_same(s.moments(), st.moments, "moments")
        _assert_same(s.fields(), st.fields, "fields")
        assert s.digest(R.BUF_FIELDS) == O.fnv1a(st.fields)
        st = O.OracleState(ref, O.make_params(n))
        st.step(2)
        s.seed_galaxy()
        s.step(2)
        _assert_same(s.particles(), st.particles, "particles after 2 steps")


def _edge_scene(name):
    from rfmm import scenes
    rng = np.random.default_rng(17)
    if name == "outliers":  # dense cluster + a few bodies in far, sparse subtrees
        p = scenes.plummer(20000, seed=4)
        p["pos"][:12] = rng.uniform(-1.55, 1.55, (12, 3)).astype(np.float32)
        return p
    if name == "outside_world":  # bodies beyond the +-1.6 world clamp to edge cells
        p = scenes.uniform(5000, seed=5)
        p["pos"][:50] = rng.uniform(-3.0, 3.0, (50, 3)).astype(np.float32)
        return p
    if name == "one_point":  # every body in one leaf
        p = scenes.uniform(3000, seed=6)
        p["pos"][:] = np.float32(0.25)
        return p
    if name == "tiny":
        return scenes.uniform(17, seed=7)
    if name == "single":
        return scenes.uniform(1, seed=8)
    if name == "fixed_point_ties":  # positions exactly on i32 rounding ties and cell faces
        p = scenes.uniform(4096, seed=9)
        k = rng.integers(-200000, 200000, (4096, 3))
        p["pos"] = ((k + 0.5) / 262144.0).astype(np.float32)
        p["pos"][:64, 0] = np.float32(0.0)
        return p
    raise ValueError(name)


@pytest.mark.parametrize("name", ["outliers", "outside_world", "one_point", "tiny", "single",
                                  "fixed_point_ties"])
def test_edge_cases_bit_exact(rfmm_mod, oracle_mod, name):
    O, R = oracle_mod, rfmm_mod
    p = _edge_scene(name)
    n = len(p)
    st = O.OracleState(p, _oracle_params(O, n))
    st.step(3)
    with _solver(R, n) as s:
        s.upload(p)
        s.step(3)
        _assert_same(s.particles(), st.particles, "particles")
        _assert_same(s.moments(), st.moments, "moments")
        _assert_same(s.fields(), st.fields, "fields")


def test_params_speed_depth_override_bit_exact(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 30000
    p = scenes.plummer(n, seed=12)
    st = O.OracleState(p, O.make_params(n, gravity=0.7, softening=2e-3, dt=7e-4, speed=1.5, depth=6))
    st.step(2)
    prm = R.default_params(gravity=0.7, softening=2e-3, dt=7e-4, speed=1.5, depth=6)
    with R.Solver(n, prm) as s:
        assert s.depth == 6
        s.upload(p)
        s.step(2)
        _assert_same(s.particles(), st.particles, "particles")
        _assert_same(s.fields(), st.fields, "fields")


@pytest.mark.parametrize("mode", [1.0, 2.0, 3.0])
def test_control_field_bit_exact(rfmm_mod, oracle_mod, mode):
    """Pull, push and vortex shepherd fields (wgsl:659-689), bit for bit."""
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 20000
    p = scenes.make("plummer", n, 13)
    cp, ax = (0.5, 0.55, 0.5, 1.0), (0.0, 1.0, 0.3, mode)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4, control_point=cp,
                                        control_axis_mode=ax, control_strength=2.0, control_radius=0.2))
    st.step(2)
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4, control_point=cp,
                           control_axis_mode=ax, control_strength=2.0, control_radius=0.2)
    with R.Solver(n, prm) as s:
        s.upload(p)
        s.step(2)
        _assert_same(s.particles(), st.particles, "particles")
        _assert_same(s.fields(), st.fields, "fields")


def test_golden_digests_on_gpu(rfmm_mod, oracle_mod):
    """The GPU reproduces the oracle's frozen digests (tests/golden/oracle_digests.json)."""
    import json, os, sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import make_golden
    R, O = rfmm_mod, oracle_mod
    gold = json.load(open(os.path.join(here, "golden", "oracle_digests.json")))
    checked, galaxies, skipped = 0, 0, []
    for name, g in sorted(gold.items()):
        galaxy = g["kind"] == "galaxy"
        galaxies += galaxy
        p = None if galaxy else make_golden.scene(g["kind"], g["n"], g["seed"])
        if not galaxy and O.fnv1a(p) != g["input_particles"]:
            # This platform's numpy scene generator differs in the last bits:
            # the frozen digests do not apply to these inputs (the live
            # oracle comparisons in this file still cover them).
            skipped.append(name)
            continue
        prm = R.default_params(gravity=g["gravity"], softening=g["softening"], dt=g["dt"])
        with R.Solver(g["n"], prm) as s:
            if galaxy:  # seeded on the GPU
                s.seed_galaxy()
                assert s.digest(R.BUF_PARTICLES) == g["input_particles"], name
                p = s.particles()
            else:
                s.upload(p)
            s.solve_fields()
            assert s.digest(R.BUF_MOMENTS) == g["solve_moments"], name
            assert s.digest(R.BUF_FIELDS) == g["solve_fields"], name
            s.upload(p)
            s.step(g["steps"])
            assert s.digest(R.BUF_PARTICLES) == g["step_particles"], name
            assert s.digest(R.BUF_MOMENTS) == g["step_moments"], name
            assert s.digest(R.BUF_FIELDS) == g["step_fields"], name
        checked += 1
    if skipped:
        import warnings
        warnings.warn("golden entries with platform-dependent inputs not checked: %s" % skipped)
    # The GPU-seeded galaxies do not depend on the host's numpy: always checked.
    assert galaxies >= 1 and checked >= galaxies, (checked, galaxies, skipped)


def test_tuning_never_changes_results(rfmm_mod, oracle_mod):
    """Launch shapes, schedules, PDL and graph length change speed, not bits."""
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 60000
    p = scenes.plummer(n, seed=21)
    st = O.OracleState(p, _oracle_params(O, n))
    st.step(6)
    variants = [dict(), dict(integrate_dynamic=1, graph_steps=4, pdl=0, m2l_compact=1),
                dict(upward_ctas_per_sm=2, m2l_ctas_per_sm=1, l2l_ctas_per_sm=1,
                     integrate_ctas_per_sm=1, resort_interval=3, graph_steps=1),
                dict(m2l_lanes=1, l2l_lanes=1, upward_warps=1),
                dict(m2l_lanes=0, l2l_lanes=0, upward_warps=0),
                dict(m2l_lanes=2, l2l_lanes=2, upward_warps=1),
                dict(m2l_lanes=1, l2l_lanes=1, m2l_ctas_per_sm=1, l2l_ctas_per_sm=1, pdl=0)]
    for v in variants:
        with _solver(R, n) as s:
            t = s.tuning()
            for k, val in v.items():
                setattr(t, k, val)
            s.set_tuning(t)
            s.upload(p)
            s.step(6)
            _assert_same(s.particles(), st.particles, "particles %r" % v)
            _assert_same(s.fields(), st.fields, "fields %r" % v)
    with _solver(R, n) as s:
        s.upload(p)
        best = s.autotune(4)
        assert 1 <= best.integrate_ctas_per_sm
        s.upload(p)
        s.step(6)
        _assert_same(s.particles(), st.particles, "particles after autotune")

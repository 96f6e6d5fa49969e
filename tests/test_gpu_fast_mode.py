"""The fast float variant (rfmm_set_float_mode(RFMM_FLOAT_FAST)) against the
oracle, within stated tolerances.

Fast mode keeps every integer result of a field solve (moments, occupancy,
parent and target lists) bit-exact on the same input; its floating-point
results follow WGSL's latitude (contraction, hardware reciprocal square root
for inverseSqrt, approximate division) and are held to:

  * per-cell moments: bit-exact (max relative error 0 <= 1e-5);
  * fields of the solve: relative rms <= 1e-5 over all cells and components;
  * per-body accelerations: relative rms <= 1e-4 (sqrt(sum |da|^2 / sum |a|^2));
  * 60 leapfrog steps of a Plummer sphere: position rms difference <= 1e-5
    (box half-extent 1.6) and fewer than 0.1% of bodies apart by more than 1e-4.

Fast mode is itself deterministic: the batched form reproduces the plain
form's fast results bit for bit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELD_RMS_TOL = 1e-5
ACCEL_RMS_TOL = 1e-4


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _rel_rms(got, ref):
    g = np.asarray(got, np.float64)
    r = np.asarray(ref, np.float64)
    return float(np.sqrt(np.sum((g - r) ** 2) / max(np.sum(r ** 2), 1e-300)))


@pytest.mark.parametrize("kind,n", [("plummer", 262147), ("uniform", 65536), ("clusters", 40000)])
def test_fast_solve_within_tolerance(rfmm_mod, oracle_mod, kind, n):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    p = scenes.make(kind, n, 7)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4))
    st.solve_fields()
    acc_ref = st.accelerations()
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.set_float_mode(R.FLOAT_FAST)
        s.upload(p)
        s.solve_fields()
        assert np.array_equal(_bits(s.moments()), _bits(st.moments)), "moments must be bit-exact"
        f = s.fields()
        fr = _rel_rms(f.view(np.float32), st.fields.view(np.float32))
        acc = s.accelerations()[:, :3]
    ar = _rel_rms(acc, acc_ref)
    print("fast %s n=%d: fields rel rms %.3g, accelerations rel rms %.3g" % (kind, n, fr, ar))
    assert fr <= FIELD_RMS_TOL, fr
    assert ar <= ACCEL_RMS_TOL, ar


def test_fast_run_tracks_exact(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 262144
    p = scenes.plummer(n, seed=3)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4))
    st.step(60)
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.set_float_mode(R.FLOAT_FAST)
        s.upload(p)
        s.step(60)
        got = s.particles()
        mom = s.moments()
    assert np.isfinite(got["pos"]).all() and np.isfinite(got["vel"]).all()
    assert int(mom["count"][0]) == n  # every body deposited once
    d = np.linalg.norm(got["pos"].astype(np.float64) - st.particles["pos"].astype(np.float64), axis=1)
    rms = float(np.sqrt(np.mean(d ** 2)))
    far = float(np.mean(d > 1e-4))
    print("fast 60 steps: position rms diff %.3g, fraction > 1e-4: %.3g, max %.3g" % (rms, far, d.max()))
    assert rms <= 1e-5, rms
    assert far < 1e-3, far


def test_fast_mode_batch_equals_plain(rfmm_mod):
    R = rfmm_mod
    from rfmm import scenes
    ps = [scenes.plummer(50000, seed=1), scenes.uniform(9000, seed=2), scenes.clusters(120000, seed=3)]
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Batch([len(q) for q in ps], [prm] * 3) as b:
        b.set_float_mode(R.FLOAT_FAST)
        for i, q in enumerate(ps):
            b.upload(i, q)
        b.commit()
        b.step(20)
        got = [b.download(i) for i in range(3)]
    for i, q in enumerate(ps):
        with R.Solver(len(q), prm) as s:
            s.set_float_mode(R.FLOAT_FAST)
            s.upload(q)
            s.step(20)
            assert np.array_equal(_bits(got[i]), _bits(s.particles())), i


def test_switching_back_to_exact_restores_bit_parity(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 30000
    p = scenes.plummer(n, seed=5)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4))
    st.step(3)
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.set_float_mode(R.FLOAT_FAST)
        s.upload(p)
        s.step(3)
        s.set_float_mode(R.FLOAT_EXACT)
        s.upload(p)
        s.step(3)
        assert np.array_equal(_bits(s.particles()), _bits(st.particles))


def test_fast_p2p_accelerations_within_tolerance(rfmm_mod, oracle_mod):
    """Exact near-field mode under the fast variant: the tiled pair sums
    against the oracle's, accelerations relative rms <= 1e-4."""
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 100000
    p = scenes.plummer(n, seed=9)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4, near_mode=1))
    st.solve_fields()
    ref = st.accelerations()
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.set_near_mode(R.NEAR_P2P)
        s.set_float_mode(R.FLOAT_FAST)
        s.upload(p)
        acc = s.accelerations()[:, :3]
        s.step(3)
        assert np.isfinite(s.particles()["pos"]).all()
    ar = _rel_rms(acc, ref)
    print("fast p2p n=%d: accelerations rel rms %.3g" % (n, ar))
    assert ar <= ACCEL_RMS_TOL, ar

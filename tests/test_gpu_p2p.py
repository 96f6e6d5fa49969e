"""GPU parity of the near-field P2P accuracy mode against the oracle.

Same floating-point contract as the reference mode (binary32, no contraction,
IEEE div/sqrt, fixed summation order): the pair sums visit cells z-, y-,
x-major and bodies by (leaf Morton code, caller index), so the GPU matches
the oracle bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _same(g, r, what):
    g, r = _bits(g).ravel(), _bits(r).ravel()
    bad = np.nonzero(g != r)[0]
    assert len(bad) == 0, "%s differs in %d of %d words; first at %d" % (what, len(bad), len(g), bad[0])


CASES = [("plummer", 16384), ("clusters", 40000), ("uniform", 65536), ("plummer", 262147)]


@pytest.mark.parametrize("kind,n", CASES)
def test_p2p_solve_and_accelerations_bit_exact(rfmm_mod, oracle_mod, kind, n):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    p = scenes.make(kind, n, 41)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4, near_mode=1))
    st.solve_fields()
    ref_acc = st.accelerations()
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.set_near_mode(R.NEAR_P2P)
        s.upload(p)
        s.solve_fields()
        _same(s.moments(), st.moments, "moments")
        _same(s.fields(), st.fields, "fields")
        acc = s.accelerations()
    _same(acc[:, :3].copy(), ref_acc, "accelerations")


@pytest.mark.parametrize("kind,n", CASES[:3])
def test_p2p_steps_bit_exact(rfmm_mod, oracle_mod, kind, n):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    p = scenes.make(kind, n, 42)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4, near_mode=1))
    st.step(4)
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.upload(p)
        s.set_near_mode(R.NEAR_P2P)  # switching after upload re-sorts the bodies
        s.step(4)
        _same(s.particles(), st.particles, "particles")
        _same(s.moments(), st.moments, "moments of the last step")
        _same(s.fields(), st.fields, "fields of the last step")


def _sparse_octant(n):
    """Most bodies in the (+,+,+) octant, a dozen in (-,-,-): those sample a
    level-1 cell whose 3x3x3 block reaches the Morton-last cell."""
    from rfmm import scenes
    p = scenes.uniform(n, seed=46)
    p["pos"][:12] = -np.random.default_rng(3).uniform(0.1, 1.2, (12, 3)).astype(np.float32)
    return p


@pytest.mark.parametrize("n", [3000, 70000])
def test_p2p_sparse_octant_bit_exact(rfmm_mod, oracle_mod, n):
    O, R = oracle_mod, rfmm_mod
    p = _sparse_octant(n)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4, near_mode=1))
    st.step(2)
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.set_near_mode(R.NEAR_P2P)
        s.upload(p)
        s.step(2)
        _same(s.particles(), st.particles, "particles")


def test_switching_back_to_reference_mode(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 30000
    p = scenes.make("plummer", n, 43)
    a = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4, near_mode=1))
    a.step(2)
    b = O.OracleState(a.particles, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4))
    b.step(2)
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.set_near_mode(R.NEAR_P2P)
        s.upload(p)
        s.step(2)
        s.set_near_mode(R.NEAR_REFERENCE)
        s.step(2)
        _same(s.particles(), b.particles, "particles")
        _same(s.fields(), b.fields, "fields")


def test_p2p_batch_per_scene_bit_exact(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    sizes = [5000, 20000, 70000]
    ps = [scenes.make(k, n, 44 + i) for i, (k, n) in enumerate(zip(["uniform", "plummer", "clusters"], sizes))]
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Batch(sizes, [prm] * 3) as b:
        b.set_near_mode(R.NEAR_P2P)
        for i, p in enumerate(ps):
            b.upload(i, p)
        b.commit()
        b.step(3)
        for i, (n, p) in enumerate(zip(sizes, ps)):
            st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4, near_mode=1))
            st.step(3)
            _same(b.download(i, R.BUF_PARTICLES), st.particles, "scene %d particles" % i)
            _same(b.download(i, R.BUF_FIELDS), st.fields, "scene %d fields" % i)


def test_p2p_force_error_is_small(rfmm_mod, oracle_mod):
    R = rfmm_mod
    from rfmm import scenes
    n = 100000
    p = scenes.make("plummer", n, 45)
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.upload(p)
        ref_rms, _ = s.force_error(2048, 3)
        s.set_near_mode(R.NEAR_P2P)
        p2p_rms, _ = s.force_error(2048, 3)
    assert p2p_rms < 0.05 and p2p_rms < 0.25 * ref_rms, (p2p_rms, ref_rms)

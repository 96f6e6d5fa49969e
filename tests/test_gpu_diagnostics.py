"""FP64 accuracy diagnostics on the GPU: per-body FMM accelerations, force
error against a direct sum, and compensated energy / momentum reductions.

Accelerations are the integrate's own (src/rainbow_fmm.wgsl:619-657) and so
bit-exact against the oracle; the FP64 reductions are checked against numpy
to a relative tolerance of 1e-9 (the summation orders differ).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

M64 = (1 << 64) - 1


def _sample(n, nt, seed):
    """The solver's target sample: splitmix64 partial Fisher-Yates."""
    idx = list(range(n))
    x = seed
    for i in range(min(nt, n)):
        x = (x + 0x9E3779B97F4A7C15) & M64
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        z ^= z >> 31
        j = i + z % (n - i)
        idx[i], idx[j] = idx[j], idx[i]
    return np.array(idx[:min(nt, n)], np.uint32)


@pytest.mark.parametrize("kind,n", [("plummer", 16384), ("clusters", 40000)])
def test_accelerations_bit_exact(rfmm_mod, oracle_mod, kind, n):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    p = scenes.make(kind, n, 31)
    st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4))
    st.solve_fields()
    ref = st.accelerations()
    with R.Solver(n, R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)) as s:
        s.upload(p)
        acc = s.accelerations()
    assert np.array_equal(acc[:, :3].view(np.uint32), ref.view(np.uint32))
    assert np.all(np.isfinite(acc[:, 3])) and acc[:, 3].max() < 0.0


def test_force_error_matches_oracle_direct_sum(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n, nt, seed = 50000, 2000, 5
    p = scenes.make("plummer", n, 3)
    # The solver's parameters are binary32: the reference uses the same values.
    G, eps = float(np.float32(0.34)), float(np.float32(0.012))
    with R.Solver(n) as s:  # harness defaults: G 0.34, eps 0.012
        s.upload(p)
        rms, mx = s.force_error(nt, seed)
        acc = s.accelerations()[:, :3].astype(np.float64)
    t = _sample(n, nt, seed)
    ref = O.direct_sum_f64(p, t, G, eps)
    d = acc[t] - ref
    rms_ref = np.sqrt((d ** 2).sum() / (ref ** 2).sum())
    mx_ref = np.sqrt(((d ** 2).sum(1) / (ref ** 2).sum(1))).max()
    assert abs(rms - rms_ref) <= 1e-9 * rms_ref, (rms, rms_ref)
    assert abs(mx - mx_ref) <= 1e-9 * mx_ref, (mx, mx_ref)
    assert 0.0 < rms < 0.4


def test_energy_momentum_reductions(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 8192
    p = scenes.make("plummer", n, 9)
    G, eps = float(np.float32(0.34)), float(np.float32(0.012))
    with R.Solver(n) as s:
        s.upload(p)
        dg = s.diagnostics()
        phi = s.accelerations()[:, 3].astype(np.float64)
    x = p["pos"].astype(np.float64)
    v = p["vel"].astype(np.float64)
    m = 1.0 / n
    ke = 0.5 * m * (v ** 2).sum()
    pe = 0.5 * m * phi.sum()
    mom = m * v.sum(0)
    am = m * np.cross(x, v).sum(0)
    assert abs(dg["kinetic"] - ke) <= 1e-9 * abs(ke)
    assert abs(dg["potential"] - pe) <= 1e-9 * abs(pe)
    assert abs(dg["total"] - (ke + pe)) <= 1e-9 * (abs(ke) + abs(pe))
    assert np.allclose(dg["momentum"], mom, rtol=0, atol=1e-12)
    assert np.allclose(dg["angular_momentum"], am, rtol=0, atol=1e-12)
    # The expansion's potential against the FP64 pairwise potential energy.
    inv = 0.0
    for a in range(0, n, 512):
        r2 = ((x[a:a + 512, None, :] - x[None, :, :]) ** 2).sum(-1) + eps * eps
        r2[np.arange(len(r2)), np.arange(a, a + len(r2))] = np.inf
        inv += (1.0 / np.sqrt(r2)).sum()
    pe_direct = -0.5 * G * m * m * inv
    assert abs(pe - pe_direct) < 0.1 * abs(pe_direct), (pe, pe_direct)

"""The near-field P2P mode of the oracle (an accuracy mode with no reference
counterpart): the fields carry M2L + L2L only and every body adds the exact
softened pair forces of the bodies in the 3x3x3 cells around its sample cell.

Checked against an independent numpy evaluation of the same decomposition
(FP64, so to a tolerance), and for the accuracy it is for: a lower force error
against the FP64 direct sum than the reference near field."""
import os

import numpy as np
import pytest


def _cells(pos, level):
    """Cell coordinates at `level` (wgsl:144-152 with IEEE division)."""
    half = np.float32(1.6)
    u = np.clip(pos / half, np.float32(-0.99999), np.float32(0.99999)) * np.float32(0.5) + np.float32(0.5)
    return np.minimum(np.floor(u * np.float32(1 << level)).astype(np.int64), (1 << level) - 1)


@pytest.mark.parametrize("kind,n,seed", [("plummer", 6000, 3), ("clusters", 9000, 4)])
def test_p2p_matches_numpy_decomposition(oracle_mod, kind, n, seed):
    O = oracle_mod
    from rfmm import scenes
    p = scenes.make(kind, n, seed)
    G, eps = 1.0, 1e-3
    st = O.OracleState(p, O.make_params(n, gravity=G, softening=eps, dt=5e-4, near_mode=1))
    st.solve_fields()
    acc = st.accelerations().astype(np.float64)
    sample = st.sample_cells()
    off = np.array([O.lib().oracle_level_offset(l) for l in range(8)])
    level = np.searchsorted(off, sample, side="right") - 1
    pos = p["pos"].astype(np.float32)
    f = st.fields.view(np.float32).reshape(-1, 12).astype(np.float64)
    checked = 0
    for i in np.random.default_rng(0).choice(n, 300, replace=False):
        l = int(level[i])
        c = _cells(pos[i:i + 1], l)[0]
        dim = 1 << l
        centre = (c.astype(np.float64) + 0.5) * (3.2 / dim) - 1.6
        r = pos[i].astype(np.float64) - centre
        fa = f[sample[i]]
        jm = np.array([fa[4] * r[0] + fa[5] * r[1] + fa[6] * r[2],
                       fa[5] * r[0] + fa[7] * r[1] + fa[8] * r[2],
                       fa[6] * r[0] + fa[8] * r[1] + fa[9] * r[2]])
        cj = _cells(pos, l)
        near = np.all(np.abs(cj - c) <= 1, axis=1)
        near[i] = False
        d = pos[near].astype(np.float64) - pos[i].astype(np.float64)
        w = (np.sum(d * d, axis=1) + np.float64(np.float32(eps)) ** 2) ** -1.5
        expect = fa[:3] + jm + (G / n) * (d * w[:, None]).sum(0)
        scale = max(np.linalg.norm(expect), 1e-6)
        assert np.linalg.norm(acc[i] - expect) <= 2e-4 * scale, (i, acc[i], expect)
        checked += 1
    assert checked == 300


def test_p2p_lowers_force_error(oracle_mod):
    O = oracle_mod
    from rfmm import scenes
    n, eps = 40000, 1e-3
    p = scenes.make("plummer", n, 7)
    targets = np.random.default_rng(1).choice(n, 1024, replace=False).astype(np.uint32)
    ref = O.direct_sum_f64(p, targets, 1.0, float(np.float32(eps)))
    errs = []
    for mode in (0, 1):
        st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=eps, dt=5e-4, near_mode=mode))
        st.solve_fields()
        a = st.accelerations()[targets].astype(np.float64)
        errs.append(np.sqrt(((a - ref) ** 2).sum() / (ref ** 2).sum()))
    assert errs[1] < 0.5 * errs[0], errs


def test_p2p_step_is_deterministic_and_finite(oracle_mod):
    O = oracle_mod
    from rfmm import scenes
    n = 5000
    p = scenes.make("uniform", n, 2)
    outs = []
    for threads in (1, 4):
        O.set_threads(threads)
        st = O.OracleState(p, O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4, near_mode=1))
        st.step(2)
        outs.append(st.particles.copy())
    O.set_threads(os.cpu_count() or 1)
    assert np.array_equal(outs[0].view(np.uint32), outs[1].view(np.uint32))
    assert np.all(np.isfinite(outs[0]["pos"]))

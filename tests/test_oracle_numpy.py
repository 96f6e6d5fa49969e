"""The C oracle against an independent numpy restatement of the WGSL passes.

Both are written from src/rainbow_fmm.wgsl under the same floating-point
definition, so moments, fields and the integrated particles must agree bit for
bit.  Small scenes (depth 4 and 5) keep the vectorised numpy version fast.
"""
import numpy as np
import pytest

import numpy_reference as NR


def _as_rows(particles):
    return np.ascontiguousarray(particles).view(np.float32).reshape(-1, 8)


@pytest.mark.parametrize("kind,n,seed", [("plummer", 4096, 3), ("uniform", 20000, 4),
                                         ("clusters", 12000, 5)])
def test_oracle_matches_numpy_restatement(oracle_mod, kind, n, seed):
    O = oracle_mod
    from rfmm import scenes
    p = scenes.make(kind, n, seed)
    params = O.make_params(n, gravity=1.0, softening=1e-3, dt=5e-4)
    st = O.OracleState(p, params)
    st.solve_fields()
    rows = _as_rows(p)
    mom, fields = NR.solve_fields(rows[:, 0:3].copy(), n, params.depth, params.scale, 1.0, 1e-3)
    assert np.array_equal(st.moments.view(np.uint32).reshape(-1, 4), mom)
    assert np.array_equal(st.fields.view(np.uint32).reshape(-1, 12), fields.view(np.uint32))
    st.integrate()
    out = NR.integrate(rows, mom, fields, n, params.depth, params.scale, 1.0, 1e-3, 5e-4)
    assert np.array_equal(_as_rows(st.particles).view(np.uint32), out.view(np.uint32))


def test_oracle_matches_numpy_on_the_reference_galaxy(oracle_mod):
    """The reference harness's own scene and defaults (native/main.rs:57-60, 423-449)."""
    O = oracle_mod
    n = 16384
    params = O.make_params(n)  # dt 0.0009, G 0.34, eps 0.012
    p = O.initialize(n, params)
    st = O.OracleState(p, params)
    st.solve_fields()
    rows = _as_rows(p)
    mom, fields = NR.solve_fields(rows[:, 0:3].copy(), n, params.depth, params.scale, 0.34, 0.012)
    assert np.array_equal(st.moments.view(np.uint32).reshape(-1, 4), mom)
    assert np.array_equal(st.fields.view(np.uint32).reshape(-1, 12), fields.view(np.uint32))

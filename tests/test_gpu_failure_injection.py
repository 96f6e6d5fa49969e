"""Failure injection on the host, without a GPU fault: malformed calls return
error codes through the C ABI, and non-finite bodies stay contained -- every
body the oracle keeps finite is bit-identical on the GPU, and the bodies that
turn non-finite are the same ones (NaN payloads may differ between the GPU
and the host, so those are compared as non-finite, not by bits)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_malformed_calls_return_error_codes(rfmm_mod):
    R = rfmm_mod
    from rfmm import scenes
    lib = R.lib()
    h = C.c_void_p()
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    assert lib.rfmm_create(0, C.byref(prm), C.byref(h)) == R.RFMM_ERR_INVALID  # no bodies
    bad_depth = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    bad_depth.depth = 7  # the planner's range is 4..6
    assert lib.rfmm_create(4096, C.byref(bad_depth), C.byref(h)) == R.RFMM_ERR_INVALID
    assert lib.rfmm_create(4096, C.byref(prm), None) == R.RFMM_ERR_INVALID
    p = scenes.uniform(4096, seed=5)
    with R.Solver(len(p), prm) as s:
        assert lib.rfmm_step(s._h, 1) == -4  # RFMM_ERR_STATE: no bodies yet
        a = np.ascontiguousarray(p)
        assert lib.rfmm_upload_particles(s._h, a.ctypes.data, a.nbytes - 32) == R.RFMM_ERR_INVALID
        assert lib.rfmm_upload_particles(s._h, None, a.nbytes) == R.RFMM_ERR_INVALID
        s.upload(p)
        out = np.empty_like(a)
        assert lib.rfmm_download(s._h, R.BUF_PARTICLES, out.ctypes.data, out.nbytes + 32) == R.RFMM_ERR_INVALID
        assert lib.rfmm_download(s._h, 7, out.ctypes.data, out.nbytes) == R.RFMM_ERR_INVALID
        s.step(2)  # the handle is unaffected by the rejected calls
        bad, mx = s.check_finite()
        assert bad == 0 and np.isfinite(mx)


def test_non_finite_bodies_are_contained(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    p = scenes.plummer(20000, seed=11)
    p["pos"][5] = np.nan
    p["pos"][77, 1] = np.inf
    p["vel"][123, 2] = -np.inf
    p["pos"][999, 0] = 1e30  # finite, far outside the world box
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Solver(len(p), prm) as s:
        s.upload(p)
        s.step(3)
        got = s.particles()
        bad_gpu, _ = s.check_finite(len(p))
    st = O.OracleState(p, O.make_params(len(p), gravity=1.0, softening=1e-3, dt=5e-4))
    st.step(3)
    want = st.particles
    g = got.view(np.float32).reshape(-1, 8)
    w = want.view(np.float32).reshape(-1, 8)
    fin_g, fin_w = np.isfinite(g), np.isfinite(w)
    assert np.array_equal(fin_g, fin_w)
    assert np.array_equal(g.view(np.uint32)[fin_g], w.view(np.uint32)[fin_w])
    nonfinite_bodies = int((~fin_g.all(axis=1)).sum())
    assert nonfinite_bodies == 3 and bad_gpu >= 1

"""Failure detection without a GPU fault: the kernels' bounded mbarrier wait,
run on a phase that nothing completes, gives up and reports RFMM_ERR_TIMEOUT
through a status word; the handle stays usable and its results unchanged."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def test_bounded_wait_gives_up_and_handle_stays_usable(rfmm_mod):
    R = rfmm_mod
    from rfmm import scenes
    p = scenes.plummer(20000, seed=7)
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Solver(len(p), prm) as s:
        s.upload(p)
        s.step(1)
        assert s.check_wait_timeout(1024) == R.RFMM_ERR_TIMEOUT
        assert s.check_wait_timeout(1) == R.RFMM_ERR_TIMEOUT
        assert s.check_wait_timeout(0) == R.RFMM_ERR_INVALID
        assert s.device_error() == (0, 0)  # the engine's own error word is untouched
        s.step(2)
        s.sync()
        got = s.particles()
    with R.Solver(len(p), prm) as ref:
        ref.upload(p)
        ref.step(3)
        want = ref.particles()
    assert np.array_equal(_bits(got), _bits(want))

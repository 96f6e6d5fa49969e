"""GPU headless render against the oracle's restatement of the display
passes (wgsl:780-1009): the same image, byte for byte (the contract's own
cos/pow/exp on both sides, exact fixed-point accumulation)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,n,w,h", [("plummer", 65536, 640, 360), ("clusters", 200000, 1280, 720)])
def test_render_matches_oracle(rfmm_mod, oracle_mod, kind, n, w, h):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    p = scenes.make(kind, n, 51)
    with R.Solver(n) as s:
        s.upload(p)
        s.step(2)
        q = s.particles()
        img = s.render(width=w, height=h)
    ref, acc = O.render(q, O.make_params(n), width=w, height=h)
    assert np.array_equal(img, ref), np.abs(img.astype(np.int16) - ref.astype(np.int16)).max()
    assert img[..., :3].max() > 100  # the cloud is visible


def test_render_control_highlight_and_instances(rfmm_mod, oracle_mod):
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    n = 50000
    p = scenes.make("plummer", n, 52)
    cp, ax = (0.5, 0.5, 0.5, 1.0), (0.0, 0.0, 1.0, 2.0)
    prm = R.default_params(control_point=cp, control_axis_mode=ax, control_radius=0.2)
    with R.Solver(n, prm) as s:
        s.upload(p)
        img = s.render(width=480, height=320, instances=n // 2, yaw=0.4, pitch=-0.3, zoom=2.2)
    ref, _ = O.render(p, O.make_params(n, control_point=cp, control_axis_mode=ax, control_radius=0.2),
                      width=480, height=320, instances=n // 2, yaw=0.4, pitch=-0.3, zoom=2.2)
    assert np.array_equal(img, ref)

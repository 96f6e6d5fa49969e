"""Batched form: many scenes of uneven size and depth per launch, each scene
bit-identical to the oracle run on that scene alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _mixed_scenes():
    from rfmm import scenes
    specs = [("uniform", 4096), ("plummer", 40000), ("clusters", 1), ("uniform", 300000),
             ("plummer", 17), ("clusters", 20000), ("plummer", 32768), ("uniform", 32769),
             ("plummer", 5000), ("clusters", 70000)]
    return [scenes.make(kind, n, 100 + i) for i, (kind, n) in enumerate(specs)]


@pytest.mark.parametrize("tree", ["warps", "lanes"])
def test_batch_matches_oracle_per_scene(rfmm_mod, oracle_mod, tree):
    """Both tree-kernel variants (one CTA or one warp per subtree, one warp or
    one lane per target)."""
    O, R = oracle_mod, rfmm_mod
    ps = _mixed_scenes()
    g = [1.0, 0.5, 1.0, 1.0, 2.0, 1.0, 0.8, 1.0, 1.0, 1.2]
    params = [R.default_params(gravity=g[i], softening=1e-3 * (1 + i % 3), dt=5e-4)
              for i in range(len(ps))]
    with R.Batch([len(p) for p in ps], params) as b:
        depths = {pl[0] for pl in b.plans}
        assert depths == {4, 5, 6}
        t = b.tuning()
        t.m2l_lanes = t.l2l_lanes = t.upward_warps = int(tree == "lanes")
        b.set_tuning(t)
        b.set_resort_interval(2)
        for i, p in enumerate(ps):
            b.upload(i, p)
        b.commit()
        b.step(4)
        for i, p in enumerate(ps):
            st = O.OracleState(p, O.make_params(len(p), gravity=g[i], softening=1e-3 * (1 + i % 3),
                                                dt=5e-4))
            st.step(4)
            assert np.array_equal(_bits(b.download(i)), _bits(st.particles)), i
            assert np.array_equal(_bits(b.download(i, R.BUF_MOMENTS)), _bits(st.moments)), i
            assert np.array_equal(_bits(b.download(i, R.BUF_FIELDS)), _bits(st.fields)), i


def test_batch_equals_plain_handles_and_reupload(rfmm_mod):
    R = rfmm_mod
    from rfmm import scenes
    ps = [scenes.plummer(50000, seed=1), scenes.uniform(9000, seed=2), scenes.clusters(120000, seed=3)]
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Batch([len(p) for p in ps], [prm] * 3) as b:
        for i, p in enumerate(ps):
            b.upload(i, p)
        b.commit()
        b.step(3)
        # Replace one scene mid-run: the others continue unchanged.
        b.upload(1, scenes.uniform(9000, seed=22))
        b.commit()
        b.step(2)
        got = [b.download(i) for i in range(3)]
    ref = []
    for i, p in enumerate(ps):
        with R.Solver(len(p), prm) as s:
            if i == 1:
                s.upload(scenes.uniform(9000, seed=22))
                s.step(2)
            else:
                s.upload(p)
                s.step(5)
            ref.append(s.particles())
    for i in range(3):
        assert np.array_equal(_bits(got[i]), _bits(ref[i])), i


def test_bulk_device_upload_equals_per_scene_uploads(rfmm_mod):
    """rfmm_batch_upload_device_all (one copy launch, device buffers) leaves
    exactly the state per-scene uploads leave; a misaligned buffer takes the
    runtime copy."""
    import torch
    R = rfmm_mod
    ps = _mixed_scenes()
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    dev = [torch.from_numpy(p.view(np.uint8).copy()).cuda() for p in ps]
    # Scene 3 from a buffer offset by 4 bytes (not 16-byte aligned).
    odd = torch.empty(dev[3].numel() + 4, dtype=torch.uint8, device="cuda")
    odd[4:].copy_(dev[3])
    ptrs = [d.data_ptr() for d in dev]
    ptrs[3] = odd.data_ptr() + 4
    out = []
    for bulk in (False, True):
        with R.Batch([len(p) for p in ps], [prm] * len(ps)) as b:
            if bulk:
                b.upload_device_all(ptrs)
            else:
                for i, d in enumerate(dev):
                    b.upload_device(i, d.data_ptr(), d.numel())
            b.commit()
            b.step(3)
            out.append([b.download(i) for i in range(len(ps))])
    for i in range(len(ps)):
        assert np.array_equal(_bits(out[0][i]), _bits(out[1][i])), i


def test_bulk_download_equals_per_scene_downloads(rfmm_mod):
    """rfmm_batch_download_all returns, for every buffer kind, exactly what
    per-scene downloads return."""
    R = rfmm_mod
    ps = _mixed_scenes()
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    with R.Batch([len(p) for p in ps], [prm] * len(ps)) as b:
        for i, p in enumerate(ps):
            b.upload(i, p)
        b.commit()
        b.step(3)
        for which, dt in ((R.BUF_PARTICLES, R.PARTICLE_DTYPE), (R.BUF_MOMENTS, R.MOMENT_DTYPE),
                          (R.BUF_FIELDS, R.FIELD_DTYPE)):
            one = [b.download(i, which) for i in range(len(ps))]
            bulk = [np.empty(len(a), dt) for a in one]
            b.download_all_into(which, [a.ctypes.data for a in bulk])
            for i in range(len(ps)):
                assert np.array_equal(_bits(one[i]), _bits(bulk[i])), (which, i)

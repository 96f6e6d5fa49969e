"""The allocation-free field solve (rfmm_solve_fields_noalloc).

Callers that cannot allocate device memory -- a plugin whose device memory
belongs to the host framework, or code running where cudaMalloc would
synchronise the device -- get the field solve through this entry point on
buffers they own; the solver's intermediate data lives in a fixed device
array inside the library.  This checks, through the C ABI, that two calls in
a row each reproduce the allocating handle path (rfmm_solve_fields +
rfmm_download_device) bit for bit, the tolerance every parity test here uses.
The file is named so pytest collects it last.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _handle_solve(R, scene, params):
    import torch
    n = len(scene)
    with R.Solver(n, params) as s:
        s.upload(scene)
        s.solve_fields()
        mom = torch.empty(s.cells * 16, dtype=torch.uint8, device="cuda")
        fld = torch.empty(s.cells * 48, dtype=torch.uint8, device="cuda")
        s.download_device(R.BUF_MOMENTS, mom.data_ptr(), mom.numel())
        s.download_device(R.BUF_FIELDS, fld.data_ptr(), fld.numel())
        torch.cuda.synchronize()
        return mom.cpu().numpy(), fld.cpu().numpy()


@pytest.mark.parametrize("calls", [[("plummer", 20000, 5), ("uniform", 131072, 9)]])
def test_noalloc_matches_handle_two_calls(rfmm_mod, calls):
    import torch
    R = rfmm_mod
    from rfmm import scenes
    params = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    stream = torch.cuda.Stream()
    for kind, n, seed in calls:
        scene = scenes.make(kind, n, seed)
        depth, cells, _ = R.plan_unclamped(n)
        dev_p = torch.from_numpy(scene.view(np.uint8).copy()).cuda()
        # Poison the outputs: the entry point must clear what it writes.
        mom = torch.full((cells * 16,), 0x7F, dtype=torch.uint8, device="cuda")
        fld = torch.full((cells * 48,), 0x7F, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        R.solve_fields_noalloc(dev_p.data_ptr(), n, params, mom.data_ptr(), fld.data_ptr(),
                               stream.cuda_stream)
        # The kernels' status word, read behind the call's work: no error.
        assert R.noalloc_device_error(stream.cuda_stream) == (R.RFMM_OK, 0, 0)
        stream.synchronize()
        ref_mom, ref_fld = _handle_solve(R, scene, params)
        got_mom, got_fld = mom.cpu().numpy(), fld.cpu().numpy()
        assert np.array_equal(got_mom, ref_mom), "moments differ (%s, n=%d)" % (kind, n)
        assert np.array_equal(got_fld, ref_fld), "fields differ (%s, n=%d)" % (kind, n)
        assert ref_mom.view(np.uint32)[0] == n  # the root cell holds every body


def test_noalloc_rejects_oversize(rfmm_mod):
    import torch
    R = rfmm_mod
    buf = torch.empty(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(R.RFMMError):
        R.solve_fields_noalloc(buf.data_ptr(), (1 << 17) + 1, None, buf.data_ptr(), buf.data_ptr())

"""Consecutive jobs through two handles on two streams (GPU).

The pattern a host uses to hide host<->device copies (and the bench's
end-to-end figure): job i runs on handle i % 2; the next job's upload is
enqueued on the other handle's stream while this one computes, its solve
waits on an event for this job's compute only, and this job's download
overlaps the next solve.  Every job must give exactly what a lone handle
gives for the same input.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_two_handle_pipeline_matches_lone_solves(rfmm_mod):
    import torch
    R = rfmm_mod
    from rfmm import scenes
    n, steps = 40000, 7
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    jobs = [scenes.make(kind, n, 100 + i) for i, kind in
            enumerate(["plummer", "uniform", "clusters", "plummer", "uniform"])]
    pin_in = [torch.from_numpy(j.view(np.uint8).copy()).pin_memory() for j in jobs]
    pin_out = [torch.empty(n * 32, dtype=torch.uint8).pin_memory() for _ in jobs]
    streams = [torch.cuda.Stream(), torch.cuda.Stream()]
    ev = [torch.cuda.Event(), torch.cuda.Event()]
    with R.Solver(n, prm) as a, R.Solver(n, prm) as b:
        h = [a, b]
        for k in range(2):
            h[k].set_stream(streams[k].cuda_stream)
        h[0].upload_host_ptr(pin_in[0].data_ptr(), pin_in[0].numel())
        h[0].step(steps)
        ev[0].record(streams[0])
        for i in range(len(jobs)):
            x, y = i % 2, (i + 1) % 2
            if i + 1 < len(jobs):
                h[y].upload_host_ptr(pin_in[i + 1].data_ptr(), pin_in[i + 1].numel())
                streams[y].wait_event(ev[x])
                h[y].step(steps)
                ev[y].record(streams[y])
            h[x].download_host_ptr(R.BUF_PARTICLES, pin_out[i].data_ptr(), pin_out[i].numel())
    for i, j in enumerate(jobs):
        with R.Solver(n, prm) as s:
            s.upload(j)
            s.step(steps)
            ref = s.particles()
        got = pin_out[i].numpy().view(np.uint32)
        assert np.array_equal(got, ref.view(np.uint32).ravel()), "job %d" % i

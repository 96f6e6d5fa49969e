"""GPU parity on the benchmarked configurations themselves, at full size.

Each test runs one measured workload exactly as the bench runs it (same
seeded scene, same plan, default tuning and resort interval, the bench's
reset-from-device-copy between runs) through the C ABI, and compares the
particles, moments and fields after the last step with the CPU oracle bit
for bit.  The integer tree (moments) is bit-exact by construction; fields and
particles are bit-exact because kernels and oracle share one floating-point
contract.  These runs reach what smaller cases cannot: depth 6 at
fixed-point scale 1024 over 60 steps with the resident-order refresh every
16 steps (plummer_1m), scale 128 with 5.2M bodies (clusters_5m), all 256
scenes of the batch, and serving slots reused by requests of other depths.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _assert_same(gpu, ref, what):
    g, r = _bits(gpu), _bits(ref)
    bad = np.nonzero(g != r)[0]
    assert len(bad) == 0, "%s differs in %d of %d words; first at %d: %r vs %r" % (
        what, len(bad), len(g), bad[0], g[bad[0]], r[bad[0]])


def _oracle(O, p, w):
    return O.OracleState(p, O.make_params(len(p), gravity=w["G"], softening=w["eps"], dt=w["dt"]))


def _params(R, w):
    return R.default_params(gravity=w["G"], softening=w["eps"], dt=w["dt"])


@pytest.mark.parametrize("name", ["plummer_1m", "clusters_5m"])
def test_plain_workload_full_run_bit_exact(rfmm_mod, oracle_mod, name):
    """The bench's plain workloads, all 60 steps, twice from the same device copy."""
    import torch
    O, R = oracle_mod, rfmm_mod
    from rfmm import workloads
    w = workloads.WORKLOADS[name]
    p = workloads.scene(w)
    st = _oracle(O, p, w)
    st.step(w["fmm_steps"])
    with R.Solver(w["n"], _params(R, w)) as s:
        if name == "plummer_1m":
            assert (s.depth, s.cells, s.scale) == (6, 299593, 1024.0)
        else:
            assert (s.depth, s.scale) == (6, 128.0)
        assert s.tuning().resort_interval == 16
        pristine = torch.from_numpy(p.view(np.uint8).copy()).cuda()
        for run in range(2):  # the bench resets the scene between its steps
            s.upload_device(pristine.data_ptr(), pristine.numel())
            s.step(w["fmm_steps"])
            _assert_same(s.moments(), st.moments, "%s run %d: moments of step 60" % (name, run))
            _assert_same(s.fields(), st.fields, "%s run %d: fields of step 60" % (name, run))
            _assert_same(s.particles(), st.particles, "%s run %d: particles" % (name, run))
        assert s.digest(R.BUF_PARTICLES) == O.fnv1a(st.particles)


def test_uniform_64k_force_eval_and_step(rfmm_mod, oracle_mod):
    """The reference's CPU-runnable case: one field solve and one step at dt 1e-3."""
    O, R = oracle_mod, rfmm_mod
    from rfmm import workloads
    w = workloads.WORKLOADS["uniform_64k"]
    p = workloads.scene(w)
    st = _oracle(O, p, w)
    st.solve_fields()
    with R.Solver(w["n"], _params(R, w)) as s:
        assert (s.depth, s.cells) == (5, 37449)
        s.upload(p)
        s.solve_fields()
        _assert_same(s.moments(), st.moments, "solve moments")
        _assert_same(s.fields(), st.fields, "solve fields")
        st = _oracle(O, p, w)
        st.step(1)
        s.upload(p)
        s.step(1)
        _assert_same(s.particles(), st.particles, "particles after one step")
        _assert_same(s.fields(), st.fields, "fields of the step")
        assert s.digest(R.BUF_FIELDS) == O.fnv1a(st.fields)


def test_batched_256_all_scenes_bit_exact(rfmm_mod, oracle_mod):
    """All 256 scenes of the batched workload, 20 steps (one resident-order
    refresh at step 16), per-scene particles, moments and fields."""
    import torch
    O, R = oracle_mod, rfmm_mod
    from rfmm import workloads
    w = workloads.WORKLOADS["batched_256"]
    ps = workloads.batch_scenes(w)
    steps = 20
    prm = _params(R, w)
    with R.Batch([len(p) for p in ps], [prm] * len(ps)) as b:
        dev = [torch.from_numpy(p.view(np.uint8).copy()).cuda() for p in ps]
        b.upload_device_all([d.data_ptr() for d in dev])
        b.commit()
        b.step(steps)
        parts = [np.empty(len(p), R.PARTICLE_DTYPE) for p in ps]
        b.download_all_into(R.BUF_PARTICLES, [a.ctypes.data for a in parts])
        moms = [np.empty(pl[1], R.MOMENT_DTYPE) for pl in b.plans]
        b.download_all_into(R.BUF_MOMENTS, [a.ctypes.data for a in moms])
        flds = [np.empty(pl[1], R.FIELD_DTYPE) for pl in b.plans]
        b.download_all_into(R.BUF_FIELDS, [a.ctypes.data for a in flds])
    for i, p in enumerate(ps):
        st = _oracle(O, p, w)
        st.step(steps)
        _assert_same(parts[i], st.particles, "scene %d (n=%d) particles" % (i, len(p)))
        _assert_same(moms[i], st.moments, "scene %d moments" % i)
        _assert_same(flds[i], st.fields, "scene %d fields" % i)


def test_server_slot_reuse_across_depths_matches_oracle(rfmm_mod, oracle_mod):
    """Serving slots reused by requests of other tree depths (6 -> 4 -> 5 ...):
    every result equals the oracle run of that request alone."""
    O, R = oracle_mod, rfmm_mod
    from rfmm import scenes
    specs = [("plummer", 300000, 7), ("uniform", 16384, 5), ("clusters4", 150000, 9),
             ("plummer", 20000, 12), ("uniform", 280000, 3), ("plummer", 40000, 17),
             ("clusters4", 16384, 20), ("plummer", 262144, 6)]
    reqs = [(scenes.make(k, n, 900 + i), s) for i, (k, n, s) in enumerate(specs)]
    prm = R.default_params(gravity=1.0, softening=1e-3, dt=5e-4)
    got = []
    for slots in (1, 2):
        with R.Server(max_bodies=300000, memory_budget_bytes=2 << 30, max_slots=slots,
                      max_chunk_steps=4) as srv:
            ids = [srv.submit(p, steps, prm) for p, steps in reqs]
            out = []
            for rid in ids:
                srv.wait(rid, 300000)
                out.append(srv.result(rid))
            got.append(out)
    depths = set()
    for i, (p, steps) in enumerate(reqs):
        st = O.OracleState(p, O.make_params(len(p), gravity=1.0, softening=1e-3, dt=5e-4))
        depths.add(st.params.depth)
        st.step(steps)
        for slots, out in zip((1, 2), got):
            _assert_same(out[i], st.particles, "request %d (n=%d, %d slot(s))" % (i, len(p), slots))
    assert depths == {4, 5, 6}

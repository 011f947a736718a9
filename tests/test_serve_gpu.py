"""Serving: continuous batching of independent solves and heat sessions.  A request's result must be
bit-identical alone (one request at a time) and in the mix, and equal to the batched solve of the same
problem; sessions equal their steps solved one after another."""
import numpy as np
import pytest

import common as cm
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

pytestmark = pytest.mark.gpu


def mix(seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for i in range(10):
        if i % 3 == 2:
            n = int(rng.integers(24, 40))
            p = api.Problem([n, n, n], [1.0 / n] * 3, alpha=0.0, beta=1.0, loc=api.LocOnMesh.Center,
                            bc=api.BCType.Dirc if i % 2 else api.BCType.Neum)
            steps = 1
        elif i % 3 == 1:
            n = int(rng.integers(40, 200))
            dt = 1e-3
            p = api.Problem([n, n], [1.0 / n] * 2, alpha=1.0, beta=dt, loc=api.LocOnMesh.Center, bc=api.BCType.Dirc)
            steps = 3
        else:
            n = int(rng.integers(60, 300))
            p = api.Problem([n, n + 7], [1.0 / n, 1.0 / (n + 7)], alpha=0.0, beta=1.0, loc=api.LocOnMesh.Center,
                            bc=api.BCType.Neum if i % 2 else api.BCType.Dirc)
            steps = 1
        size = int(np.prod(p.n))
        f = rng.standard_normal(size)
        if p.bc == api.BCType.Neum and p.alpha == 0.0:
            f -= f.mean()
        reqs.append((p, f, steps))
    return reqs


def run(server, reqs):
    outs, ids = [], []
    for p, f, steps in reqs:
        out = np.zeros(f.size)
        outs.append(out)
        ids.append(server.submit(p, f, steps=steps, out=out))
    res = [server.result(i) for i in ids]
    return outs, res


def test_server_mix_equals_alone_and_batch(ctx):
    reqs = mix(3)
    params = api.StructSolverParams(tol=1e-10, maxIter=100, precision="mixed")
    s_mix = api.Server(params, max_active=8, ctx=ctx)
    outs_mix, res_mix = run(s_mix, reqs)
    st = s_mix.stats()
    s_mix.close()
    assert all(r["status"] == capi.OK for r in res_mix), res_mix
    assert st["completed"] == len(reqs) and st["max_active_seen"] > 1
    s_one = api.Server(params, max_active=1, ctx=ctx)
    outs_one, res_one = run(s_one, reqs)
    s_one.close()
    for k in range(len(reqs)):
        assert res_one[k]["iterations"] == res_mix[k]["iterations"], k
        assert np.array_equal(outs_one[k], outs_mix[k]), k
    # against the batched solve of the same problems (one-shot ones), and sessions step by step
    for k, (p, f, steps) in enumerate(reqs):
        B = api.Batch([p], api.StructSolverParams(tol=1e-10, maxIter=100, precision="mixed"), ctx)
        x = np.zeros(f.size)
        rhs = f
        for _ in range(steps):
            B.set(0, rhs, x)
            s = B.solve()[0]
            assert s.converged
            x = B.get(0)
            rhs = x
        if p.bc == api.BCType.Neum and p.alpha == 0.0:
            x = x - x[0]  # the server reports the pinned solution
            assert outs_mix[k][0] == 0.0
        assert np.abs(outs_mix[k] - x).max() <= 1e-9 * max(1.0, np.abs(x).max()), k


def test_server_rejects_nan_and_respects_budget(ctx):
    params = api.StructSolverParams(tol=1e-10, precision="mixed")
    s = api.Server(params, hbm_budget=1, max_active=8, ctx=ctx)  # budget below one request: one at a time
    p = api.Problem([64, 64], [1 / 64, 1 / 64], alpha=0.0, beta=1.0)
    f = np.ones(64 * 64)
    f[5] = np.nan
    with pytest.raises(capi.OpflowError) as e:
        s.submit(p, f)
    assert e.value.code == capi.E_NAN
    ids = [s.submit(p, np.random.default_rng(i).standard_normal(64 * 64)) for i in range(4)]
    res = [s.result(i) for i in ids]
    assert all(r["status"] == capi.OK for r in res)
    assert s.stats()["max_active_seen"] == 1
    s.close()


def test_failed_setup_leaves_the_others_served(ctx):
    """A request whose set-up fails (a boundary condition the problem form does not take) finishes with
    its error while the requests around it are served as usual."""
    params = api.StructSolverParams(tol=1e-10, maxIter=100, precision="mixed")
    s = api.Server(params, max_active=4, ctx=ctx)
    good = api.Problem([48, 40], [1 / 48, 1 / 40], alpha=1.0, beta=1e-3)
    bad = api.Problem([48, 40], [1 / 48, 1 / 40], alpha=1.0, beta=1e-3, bc=api.BCType.Periodic)
    rng = np.random.default_rng(7)
    fs = [rng.standard_normal(48 * 40) for _ in range(5)]
    ids = [s.submit(bad if k == 2 else good, fs[k]) for k in range(5)]
    res = [s.result(i) for i in ids]
    assert res[2]["status"] == capi.E_INVALID
    assert all(res[k]["status"] == capi.OK and res[k]["rel_residual"] <= 1e-10 for k in (0, 1, 3, 4)), res
    st = s.stats()
    assert st["completed"] == 5
    s.close()


def test_close_serves_what_was_submitted(ctx):
    """Closing a server with requests still queued or in set-up serves them all before it returns."""
    reqs = mix(11)
    params = api.StructSolverParams(tol=1e-10, maxIter=100, precision="mixed")
    s = api.Server(params, max_active=3, ctx=ctx)
    outs = []
    for p, f, steps in reqs:
        out = np.full(f.size, np.nan)
        outs.append(out)
        s.submit(p, f, steps=steps, out=out)
    s.close()
    ref = api.Server(params, max_active=8, ctx=ctx)
    outs_ref, res_ref = run(ref, reqs)
    ref.close()
    assert all(r["status"] == capi.OK for r in res_ref)
    for k in range(len(reqs)):
        assert np.array_equal(outs[k], outs_ref[k]), k


def test_session_checkpoint_to_disk_and_restore(ctx, tmp_path):
    """A heat session checkpointed at a step boundary, written to disk as a RawBinary field snapshot,
    read back and resubmitted (f = x0 = the state, the remaining steps) ends bit for bit where the
    uninterrupted session ends."""
    n, steps = 257, 30
    p = api.Problem([n, n], [1.0 / n] * 2, alpha=1.0, beta=1.0 / n, loc=api.LocOnMesh.Center, bc=api.BCType.Dirc)
    f = np.random.default_rng(21).standard_normal(n * n)
    params = api.StructSolverParams(tol=1e-10, maxIter=100, precision="mixed")
    ref = api.Server(params, ctx=ctx)
    whole = np.zeros(n * n)
    rid = ref.submit(p, f, steps=steps, out=whole)
    assert ref.result(rid)["status"] == capi.OK
    ref.close()
    s = api.Server(params, ctx=ctx)
    out = np.zeros(n * n)
    rid = s.submit(p, f, steps=steps, out=out)
    state, k = s.checkpoint(rid, n * n)
    assert 1 <= k < steps
    assert s.result(rid)["status"] == capi.OK
    s.close()
    assert np.array_equal(out, whole)  # the checkpoint did not disturb the session
    # to disk and back through a cell-centred field of the problem's shape
    mesh = cm.mesh_uniform([n + 1, n + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, ext=1)
    fld = api.CartesianField(mesh, fd, ctx, "session")
    a = fld.download()
    sl = fld.index_slices([tuple(fld.info.assignable[d]) for d in range(2)])
    a[sl] = state.reshape(n, n)
    fld.upload(a)
    api.RawBinaryOStream(str(tmp_path / "ckpt")) << api.TimeStamp(float(k)) << fld
    back = api.CartesianField(mesh, fd, ctx, "session")
    ist = api.RawBinaryIStream(str(tmp_path / "ckpt"))
    ist >> back
    assert ist.time == float(k)
    restored = back.download()[sl].reshape(-1).copy()
    assert np.array_equal(restored, state)
    s2 = api.Server(params, ctx=ctx)
    out2 = np.zeros(n * n)
    rid2 = s2.submit(p, restored, steps=steps - k, out=out2, x0=restored)
    assert s2.result(rid2)["status"] == capi.OK
    s2.close()
    assert np.array_equal(out2, whole)


def test_checkpoint_refusals(ctx):
    params = api.StructSolverParams(tol=1e-10, precision="mixed")
    s = api.Server(params, ctx=ctx)
    p = api.Problem([64, 64], [1 / 64, 1 / 64], alpha=1.0, beta=1e-3)
    rid = s.submit(p, np.ones(64 * 64))
    with pytest.raises(capi.OpflowError) as e:
        s.checkpoint(rid, 64 * 64)
    assert e.value.code == capi.E_INVALID and "single solve" in str(e.value)
    rid = s.submit(p, np.ones(64 * 64), steps=3)
    with pytest.raises(capi.OpflowError):
        s.checkpoint(rid, 10)
    s.result(rid)
    with pytest.raises(capi.OpflowError) as e:
        s.checkpoint(rid, 64 * 64)
    assert "finished" in str(e.value)
    s.close()


def test_device_resident_requests_equal_host_requests(ctx):
    """Right-hand sides and result buffers in device memory (unified addressing) give the host
    requests' results bit for bit; a non-finite device right-hand side finishes with OPFLOW_E_NAN."""
    torch = pytest.importorskip("torch")
    reqs = mix(5)
    params = api.StructSolverParams(tol=1e-10, maxIter=100, precision="mixed")
    s = api.Server(params, max_active=8, ctx=ctx)
    outs_h, res_h = run(s, reqs)
    dev = torch.device("cuda", 0)
    fd = [torch.from_numpy(f.copy()).to(dev) for _, f, _ in reqs]
    od = [torch.zeros(f.size, dtype=torch.float64, device=dev) for _, f, _ in reqs]
    torch.cuda.synchronize()
    ids = [s.submit(p, fd[k], steps=steps, out=od[k]) for k, (p, f, steps) in enumerate(reqs)]
    res_d = [s.result(i) for i in ids]
    bad = fd[0].clone()
    bad[7] = float("nan")
    torch.cuda.synchronize()
    rb = s.result(s.submit(reqs[0][0], bad, steps=1))
    s.close()
    assert all(r["status"] == capi.OK for r in res_d), res_d
    for k in range(len(reqs)):
        assert res_d[k]["iterations"] == res_h[k]["iterations"], k
        assert np.array_equal(od[k].cpu().numpy(), outs_h[k]), k
    assert rb["status"] == capi.E_NAN

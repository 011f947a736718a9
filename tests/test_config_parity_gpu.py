"""Parity at the benchmark configurations' own sizes: every solve the benchmarks time is re-checked by
the oracle, which assembles the reference's system itself (the generateAb restatement) and recomputes
||b - A x||_2 / ||b||_2 for the GPU's answer.

- 2D Poisson, 2048^2 cells, homogeneous Neumann, pinned (FP64 and mixed precision);
- 3D flux form div(exp(g) grad p) = f on 256^3 cells, Neumann, pinned (mixed precision);
- every problem of the 512-problem batched configuration (mixed precision, one batched solve);
- the 256^3 exp(g) equation served as a user-equation request, alone and in the serving mix;
- every request of a served stream of the serving configuration's mix (one-shot solves and heat
  sessions), whose sessions are checked step by step: a session of k - 1 steps gives, bit for bit,
  the right-hand side of the k-th step (results are deterministic alone and in any mix).
The inputs are the benchmark's own seeded inputs (opflow_gb300.workloads).
"""
import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api
from opflow_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def oracle_rel_residual(target, getter, pin):
    hf_t = orc.HostField(target.mesh, target.desc, data=target.download())
    leaf = cm.Leaf("t")
    nodes, leaves = api.serialize(getter(leaf).residual_expr(), [leaf])
    hosts = [hf_t if lf is leaf else orc.HostField(lf.mesh, lf.desc, data=lf.download()) for lf in leaves]
    off, coef, rhs = orc.assemble(hf_t, nodes, hosts, 0, int(pin))
    rng = hf_t.assignable()
    x = hf_t.data[hf_t.slices(rng)].reshape(-1)
    r, bn = orc.residual([q[1] - q[0] for q in rng], [0] * len(rng), off, coef, rhs, x)
    return r / bn


def cell_fields(ctx, n, ndim, count):
    mesh = api.MeshBuilder().newMesh(*([n + 1] * ndim))
    for d in range(ndim):
        mesh.setMeshOfDim(d, 0.0, 1.0)
    mesh = mesh.build()
    b = api.ExprBuilder().setMesh(mesh).setLoc(api.LocOnMesh.Center).setExt(1)
    for d in range(ndim):
        b.setBC(d, api.DimPos.start, api.BCType.Neum, 0.).setBC(d, api.DimPos.end, api.BCType.Neum, 0.)
    return [b.build(ctx) for _ in range(count)]


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_poisson2d_2048_neumann_on_the_oracles_system(ctx, prec):
    n = 2048
    p, f = cell_fields(ctx, n, 2, 2)
    a = f.download()
    sl = f.index_slices(f.assignableRange)
    v = np.random.default_rng(1234).standard_normal(a[sl].shape)  # the benchmark's rank-0 input
    a[sl] = v - v.mean()
    f.upload(a)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)
    p.assign(0.0)
    st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, maxIter=200, pinValue=True, precision=prec))
    assert st.converged and st.relerr <= 1e-10, st
    rel = oracle_rel_residual(p, getter, True)
    print("\n2048^2 Neumann %s: %d iterations, library %.3e, oracle %.3e" % (prec, st.niter, st.relerr, rel))
    assert rel <= 2e-10, rel
    assert abs(st.relerr - rel) <= 0.01 * rel, (st.relerr, rel)


def test_poisson3d_256_expg_on_the_oracles_system(ctx):
    n = 256
    p, f, K = cell_fields(ctx, n, 3, 3)
    rng = np.random.default_rng(4321)  # the benchmark's rank-0 input
    kk = K.download()
    sl = K.index_slices(K.assignableRange)
    kk[sl] = np.exp(wl.smooth_field(rng, n))
    K.upload(kk)
    ff = f.download()
    v = rng.standard_normal(ff[sl].shape)
    ff[sl] = v - v.mean()
    f.upload(ff)
    getter = lambda e: f == (api.dx(api.d1IntpCenterToCorner(K, 0) * api.dx(e)) + api.dy(api.d1IntpCenterToCorner(K, 1) * api.dy(e))
                             + api.dz(api.d1IntpCenterToCorner(K, 2) * api.dz(e)))
    p.assign(0.0)
    st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, maxIter=300, pinValue=True, precision="mixed"))
    assert st.converged and st.relerr <= 1e-10, st
    rel = oracle_rel_residual(p, getter, True)
    print("\n256^3 exp(g) mixed: %d iterations, library %.3e, oracle %.3e" % (st.niter, st.relerr, rel))
    assert rel <= 2e-10, rel
    assert abs(st.relerr - rel) <= 0.01 * rel, (st.relerr, rel)


def test_batched_512_every_problem_on_the_oracles_system(ctx):
    probs = wl.batched_problems(api, 99, 512)  # the benchmark's rank-0 batch
    params = api.StructSolverParams(tol=1e-10, maxIter=200, precision="mixed", zeroGuess=True)
    B = api.Batch([p for p, _ in probs], params, ctx)
    for i, (_, f) in enumerate(probs):
        B.set(i, f)
    st = B.solve()
    assert all(s.converged and s.relerr <= 1e-10 for s in st)
    worst = 0.0
    for i, (p, f) in enumerate(probs):
        rel = cm.problem_residual(p, f, B.get(i))
        worst = max(worst, rel)
        assert rel <= 2e-10, (i, p.n, p.beta, rel)
    B.close()
    print("\n512 batched problems: worst oracle residual %.3e, iterations %d..%d" % (worst, min(s.niter for s in st), max(s.niter for s in st)))


def test_every_served_result_on_the_oracles_system(ctx):
    reqs = wl.serve_mix(api, 5, 24)
    # keep the stream's shapes but bound the sessions' length so the step-by-step check stays short
    reqs = [(p, f, min(steps, 6)) for p, f, steps in reqs]
    params = api.StructSolverParams(tol=1e-10, maxIter=200, precision="mixed")
    srv = api.Server(params, max_active=16, ctx=ctx)
    outs, ids = [], []
    for p, f, steps in reqs:
        out = np.zeros(f.size)
        outs.append(out)
        ids.append(srv.submit(p, f, steps=steps, out=out))
    res = [srv.result(i) for i in ids]
    # sessions' intermediate states: the same session with one step fewer (bit-identical by determinism)
    prev = {}
    for k, (p, f, steps) in enumerate(reqs):
        if steps > 1:
            out = np.zeros(f.size)
            prev[k] = (srv.submit(p, f, steps=steps - 1, out=out), out)
    for k, (i, out) in prev.items():
        assert srv.result(i)["status"] == capi.OK
    srv.close()
    assert all(r["status"] == capi.OK for r in res), res
    worst = 0.0
    for k, (p, f, steps) in enumerate(reqs):
        rhs = f if steps == 1 else prev[k][1]
        rel = cm.problem_residual(p, rhs, outs[k])
        worst = max(worst, rel)
        assert rel <= 2e-10, (k, p.n, steps, rel)
    print("\n%d served requests (%d sessions): worst oracle residual %.3e" % (len(reqs), len(prev), worst))


def test_served_256_expg_equation_alone_and_in_the_mix(ctx):
    """The 256^3 exp(g) configuration's equation served as a user-equation request
    (opflow_request.equation): bit-identical alone and in a mix of the serving configuration's
    requests, and on the oracle's system to 2e-10."""
    n = 256
    p, f, K = cell_fields(ctx, n, 3, 3)
    rng = np.random.default_rng(4321)
    kk = K.download()
    sl = K.index_slices(K.assignableRange)
    kk[sl] = np.exp(wl.smooth_field(rng, n))
    K.upload(kk)
    ff = f.download()
    v = rng.standard_normal(ff[sl].shape)
    ff[sl] = v - v.mean()
    f.upload(ff)
    p.assign(0.0)
    getter = lambda e: f == (api.dx(api.d1IntpCenterToCorner(K, 0) * api.dx(e)) + api.dy(api.d1IntpCenterToCorner(K, 1) * api.dy(e))
                             + api.dz(api.d1IntpCenterToCorner(K, 2) * api.dz(e)))
    params = api.StructSolverParams(tol=1e-10, maxIter=300, pinValue=True, precision="mixed")
    outs = []
    for mixed in (False, True):
        srv = api.Server(params, max_active=16 if mixed else 1, ctx=ctx)
        others = []
        if mixed:
            for q, fq, _ in wl.serve_mix(api, 9, 6):
                o = np.zeros(fq.size)
                others.append((srv.submit(q, fq, out=o), o))
        out = np.zeros(n ** 3)
        rid = srv.submit_equation(getter, p, out=out)
        r = srv.result(rid)
        assert all(srv.result(i)["status"] == capi.OK for i, _ in others)
        srv.close()
        assert r["status"] == capi.OK and r["rel_residual"] <= 1e-10, r
        outs.append(out)
    assert np.array_equal(outs[0], outs[1])
    pa = p.download()
    pa[sl] = outs[1].reshape(pa[sl].shape)
    p.upload(pa)
    rel = oracle_rel_residual(p, getter, True)
    print("\nserved 256^3 exp(g): oracle %.3e" % rel)
    assert rel <= 2e-10, rel

"""Batching and serving user equations (opflow_batch_create_eqns, opflow_request.equation): any
StencilPad-generated equation of the kind makeEqnSolveHandler takes, next to the fixed-form problems.
The equations here:
- the 3D flux form div(exp(g) grad p) = f, Neumann on every side, pinned (the 256^3 benchmark
  configuration's operator, at 48^3 and 40^3);
- a 2D Helmholtz form (Lap - 1/2) e = f with mixed sides: nonzero Dirichlet values on x, Neumann on y.
Checked:
- a served equation request is bit-identical alone and in a mix of fixed-form and other equation
  requests of different sizes;
- every solution passes the oracle's residual check on the reference's own system (oracle assembly,
  the generateAb restatement, pinned row included);
- a batch of equations reaches the tolerance on each problem's oracle system, and gives the served
  request's solution to the tolerance's precision.
"""
import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api
from opflow_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL = 1e-10


def expg3d(ctx, n, seed):
    """(getter, target, fields): div(exp(g) grad p) = f on n^3 cells, Neumann, f of zero mean."""
    mesh = api.MeshBuilder().newMesh(n + 1, n + 1, n + 1)
    for d in range(3):
        mesh.setMeshOfDim(d, 0.0, 1.0)
    mesh = mesh.build()
    b = api.ExprBuilder().setMesh(mesh).setLoc(api.LocOnMesh.Center).setExt(1)
    for d in range(3):
        b.setBC(d, api.DimPos.start, api.BCType.Neum, 0.).setBC(d, api.DimPos.end, api.BCType.Neum, 0.)
    p, f, K = (b.setName(nm).build(ctx) for nm in ("p", "f", "K"))
    rng = np.random.default_rng(seed)
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
    return getter, p, (p, f, K), True


def helm2d_mixed(ctx, nx, ny, seed):
    """(getter, target, fields): (Lap - 1/2) e = f on nx x ny cells, Dirichlet 1 / -0.5 on the x sides,
    Neumann 0 on the y sides; the target starts from seeded values (the initial guess)."""
    mesh = api.MeshBuilder().newMesh(nx + 1, ny + 1).setMeshOfDim(0, 0.0, 1.0).setMeshOfDim(1, 0.0, ny / nx).build()
    b = api.ExprBuilder().setMesh(mesh).setLoc(api.LocOnMesh.Center).setExt(1)
    b.setBC(0, api.DimPos.start, api.BCType.Dirc, 1.0).setBC(0, api.DimPos.end, api.BCType.Dirc, -0.5)
    b.setBC(1, api.DimPos.start, api.BCType.Neum, 0.).setBC(1, api.DimPos.end, api.BCType.Neum, 0.)
    p, f = (b.setName(nm).build(ctx) for nm in ("p", "f"))
    rng = np.random.default_rng(seed)
    for fld in (p, f):
        a = fld.download()
        sl = fld.index_slices(fld.assignableRange)
        a[sl] = rng.standard_normal(a[sl].shape)
        fld.upload(a)
    getter = lambda e: f == api.d2x(e) + api.d2y(e) - 0.5 * e
    return getter, p, (p, f), False


def oracle_rel_residual(target, getter, pin, x):
    """||b - A x|| / ||b|| of the reference's system (oracle assembly) for x over the target's
    assignable cells (x fastest)."""
    hf_t = orc.HostField(target.mesh, target.desc, data=target.download())
    rng = hf_t.assignable()
    hf_t.data[hf_t.slices(rng)] = np.asarray(x).reshape(hf_t.data[hf_t.slices(rng)].shape)
    leaf = cm.Leaf("t")
    nodes, leaves = api.serialize(getter(leaf).residual_expr(), [leaf])
    hosts = [hf_t if lf is leaf else orc.HostField(lf.mesh, lf.desc, data=lf.download()) for lf in leaves]
    off, coef, rhs = orc.assemble(hf_t, nodes, hosts, 0, int(pin))
    r, bn = orc.residual([q[1] - q[0] for q in rng], [0] * len(rng), off, coef, rhs, hf_t.data[hf_t.slices(rng)].reshape(-1))
    return r / bn


def unknowns(target):
    return int(np.prod([hi - lo for lo, hi in target.assignableRange]))


def params():
    return api.StructSolverParams(tol=TOL, maxIter=100, pinValue=True, precision="mixed")


def serve(ctx, eqns, problems=(), max_active=16):
    """Serves the equation requests (with the fixed-form problems interleaved); returns their outputs
    and results."""
    s = api.Server(params(), max_active=max_active, ctx=ctx)
    outs, ids, fixed = [], [], []
    for k, (getter, target, _, _) in enumerate(eqns):
        if k < len(problems):
            p, f = problems[k]
            o = np.zeros(f.size)
            fixed.append((s.submit(p, f, out=o), o))
        out = np.zeros(unknowns(target))
        outs.append(out)
        ids.append(s.submit_equation(getter, target, out=out))
    res = [s.result(i) for i in ids]
    fres = [s.result(i) for i, _ in fixed]
    s.close()
    assert all(r["status"] == capi.OK for r in fres), fres
    return outs, res


def test_served_equations_alone_and_in_a_mix(ctx):
    e3 = expg3d(ctx, 48, 11)
    e3b = expg3d(ctx, 40, 12)
    e2 = helm2d_mixed(ctx, 96, 72, 13)
    # alone: one request per server
    alone = []
    for eq in (e3, e2):
        o, r = serve(ctx, [eq], max_active=1)
        assert r[0]["status"] == capi.OK and r[0]["rel_residual"] <= TOL, r
        alone.append(o[0])
    # in a mix with fixed-form problems and another equation
    rng = np.random.default_rng(5)
    probs = []
    for n in (70, 33, 150):
        ndim = 3 if n == 33 else 2
        p = api.Problem([n] * ndim, [1.0 / n] * ndim, alpha=0.0, beta=1.0, loc=api.LocOnMesh.Center, bc=api.BCType.Dirc)
        probs.append((p, rng.standard_normal(n ** ndim)))
    outs, res = serve(ctx, [e3b, e3, e2], problems=probs)
    assert all(r["status"] == capi.OK and r["rel_residual"] <= TOL for r in res), res
    assert np.array_equal(outs[1], alone[0])
    assert np.array_equal(outs[2], alone[1])
    for (getter, target, _, pin), x in zip((e3b, e3, e2), outs):
        rel = oracle_rel_residual(target, getter, pin, x)
        assert rel <= 2 * TOL, rel
    # the pinned problems' first unknown is held at 0, as the reference's pinned row says
    assert outs[0][0] == 0.0 and outs[1][0] == 0.0
    # the target fields themselves are not written
    assert not np.any(e3[1].download()[e3[1].index_slices(e3[1].assignableRange)])


def test_batch_of_equations_reaches_the_oracles_tolerance(ctx):
    eqs = [expg3d(ctx, 40, 21), helm2d_mixed(ctx, 128, 96, 22), helm2d_mixed(ctx, 64, 200, 23), expg3d(ctx, 24, 24)]
    B = api.Batch([(g, t) for g, t, _, _ in eqs], params(), ctx=ctx)
    st = B.solve()
    assert all(s.converged for s in st), [(s.niter, s.relerr) for s in st]
    xs = [B.get(i) for i in range(len(eqs))]
    B.close()
    for (getter, target, _, pin), x in zip(eqs, xs):
        assert x.size == unknowns(target)
        rel = oracle_rel_residual(target, getter, pin, x)
        assert rel <= 2 * TOL, rel
    # the same equation served: the same solution to the tolerance's precision
    o, r = serve(ctx, [eqs[1]], max_active=1)
    assert np.abs(o[0] - xs[1]).max() <= 1e-6 * np.abs(xs[1]).max()

"""Path I on the GPU: device StencilPad assembly against the reference's dumps (bit-exact), and the
multigrid-preconditioned solvers against the oracle's residual and FP64 CG solution."""
import os

import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api
from test_oracle_golden import _assemble_case, _by_offset

pytestmark = pytest.mark.gpu

ASM = sorted(f[:-4] for f in os.listdir(cm.GOLDEN) if f.startswith("asm_"))


def to_gpu(ctx, hf):
    f = api.CartesianField(hf.mesh, hf.desc, ctx)
    f.upload(hf.data, update_padding=False)
    return f


def gpu_case(ctx, name):
    meta, arr = cm.golden(name)
    target, fmap, eq_leaf, pin = _assemble_case(name, arr, meta)
    g = {k: to_gpu(ctx, v) for k, v in fmap.items()}
    # rebuild the equation over GPU fields by re-running the case builder's tree with a tag map
    nodes, leaves = api.serialize(eq_leaf.residual_expr())
    tags = [lf.tag for lf in leaves]
    tgt_tag = [t for t in tags if fmap[t] is target][0]
    return g, tgt_tag, nodes, tags, target, fmap, pin, arr, meta


@pytest.mark.parametrize("name", ASM)
def test_device_assembly_matches_reference_dump(ctx, name):
    g, tgt, nodes, tags, target, fmap, pin, arr, meta = gpu_case(ctx, name)
    import ctypes as C
    hs = (C.c_void_p * len(tags))(*[g[t].handle.value for t in tags])
    unknown = tags.index(tgt)
    ne, nc = C.c_int(0), C.c_size_t(0)
    L = capi.lib()
    capi.check(L.opflow_assemble(ctx.handle, g[tgt].handle, nodes, len(nodes), hs, len(tags), unknown, int(pin), C.byref(ne), None, None, None,
                                 C.byref(nc)))
    D = target.info.ndim
    off = np.zeros(ne.value * D, dtype=np.int32)
    coef = np.zeros(nc.value * ne.value)
    rhs = np.zeros(nc.value)
    capi.check(L.opflow_assemble(ctx.handle, g[tgt].handle, nodes, len(nodes), hs, len(tags), unknown, int(pin), C.byref(ne),
                                 off.ctypes.data_as(C.POINTER(C.c_int)), coef.ctypes.data_as(C.POINTER(C.c_double)),
                                 rhs.ctypes.data_as(C.POINTER(C.c_double)), C.byref(nc)))
    st = cm.record(meta, "stencil")
    want = _by_offset(np.array(st["offsets"]), arr["stencil__coef"])
    got = _by_offset(off.reshape(-1, D), coef.reshape(-1, ne.value))
    for k in want:
        assert np.array_equal(got[k], want[k]), (k, np.abs(got[k] - want[k]).max())
    assert np.array_equal(rhs, arr["stencil__rhs"])


def poisson_case(ctx, n, bc, ndim=2, seed=5, loc=capi.CENTER):
    mesh = cm.mesh_uniform([n + 1] * ndim if loc == capi.CENTER else [n] * ndim)
    fd = cm.field_desc(ndim, loc, [(bc, bc)] * ndim, ext=1 if loc == capi.CENTER else 0)
    p = api.CartesianField(mesh, fd, ctx)
    f = api.CartesianField(mesh, fd, ctx)
    a = f.download()
    rng = np.random.default_rng(seed)
    sl = f.index_slices([(max(f.info.assignable[d][0], f.info.local[d][0]), min(f.info.assignable[d][1], f.info.local[d][1]))
                         for d in range(ndim)])
    v = rng.standard_normal(a[sl].shape)
    if bc in (capi.BC_NEUM, capi.BC_PERIODIC):
        v -= v.mean()
    a[sl] = v
    f.upload(a)
    return mesh, fd, p, f


def oracle_check(target, getter, x_field, pin, tol):
    """Assemble the reference's system with the oracle and evaluate ||b - A x|| / ||b|| for the GPU x."""
    hf_t = orc.HostField(target.mesh, target.desc, data=x_field.download())
    leaf = cm.Leaf("t")
    eq = getter(leaf)
    nodes, leaves = api.serialize(eq.residual_expr(), [leaf])
    hosts = []
    for lf in leaves:
        if lf is leaf:
            hosts.append(hf_t)
        else:
            hosts.append(orc.HostField(lf.mesh, lf.desc, data=lf.download()))
    off, coef, rhs = orc.assemble(hf_t, nodes, hosts, 0, int(pin))
    rng = hf_t.assignable()
    x = hf_t.data[hf_t.slices(rng)].reshape(-1)
    dims = [r[1] - r[0] for r in rng]
    periodic = [int(target.desc.bc_type[d][0] == capi.BC_PERIODIC) for d in range(len(dims))]
    r, bn = orc.residual(dims, periodic, off, coef, rhs, x)
    return (r / bn if bn > 0 else r), (dims, periodic, off, coef, rhs, x)  # b = 0: the absolute residual


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("n,bc", [(64, capi.BC_NEUM), (96, capi.BC_DIRC), (50, capi.BC_NEUM), (64, capi.BC_PERIODIC)])
def test_poisson2d_reaches_tolerance_on_the_reference_system(ctx, prec, n, bc):
    mesh, fd, p, f = poisson_case(ctx, n, bc)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)  # SPD form: A = -L, b = -f
    pin = bc != capi.BC_DIRC
    params = api.StructSolverParams(tol=1e-10, maxIter=100, pinValue=pin, precision=prec)
    st = api.Solve(getter, p, params)
    assert st.converged and st.relerr <= 1e-10, st
    rel, sysd = oracle_check(p, getter, p, pin, 1e-10)
    assert rel <= 2e-10, rel
    # against an FP64 CG solution of the same system (error of the GPU solution stated, not only the residual)
    dims, periodic, off, coef, rhs, x = sysd
    xo, it, rr = orc.pcg(dims, periodic, off, coef, rhs, tol=1e-13)
    err = np.abs(x - xo).max() / np.abs(xo).max()
    assert err <= 1e-7, err
    if pin:
        assert x[0] == 0.0


def test_variable_coefficient_dirichlet_like_reference_test(ctx):
    """The DircEqnTest operator: dx(dx(e)/intp(r)) + dy(dy(e)/intp(r)) with a 1000:1 jump in r,
    b the discrete operator applied to p_true: the solve recovers p_true."""
    n = 64
    mesh = cm.mesh_uniform([n + 1, n + 1])
    mk = lambda v: cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(v, v)] * 2, ext=1)
    p, ptrue, b = (api.CartesianField(mesh, mk(0.0), ctx) for _ in range(3))
    r = api.CartesianField(mesh, mk(1.0), ctx)
    ptrue.initBy(lambda X: X[0] * (1. - X[0]) * X[1] * (1. - X[1]))
    h = 1.0 / n

    def rfun(X):
        dist = np.sqrt((X[0] - 0.5) ** 2 + (X[1] - 0.5) ** 2)
        w = h * 8
        hev = np.where(dist - 0.2 < -w, 0.0, np.where(dist - 0.2 > w, 1.0, 0.5 * (1 + (dist - 0.2) / w + np.sin(np.pi * (dist - 0.2) / w) / np.pi)))
        return 1. * hev + (1. - hev) * 1000

    r.initBy(rfun)
    op = lambda e: api.dx(api.dx(e) / api.d1IntpCenterToCorner(r, 0)) + api.dy(api.dy(e) / api.d1IntpCenterToCorner(r, 1))
    b.assign(op(ptrue))
    p.assign(0.0)
    for prec in ("fp64", "mixed"):
        p.assign(0.0)
        st = api.Solve(lambda e: api.Eq(b, op(e)), p, api.StructSolverParams(tol=1e-10, maxIter=200, precision=prec))
        assert st.converged, st
        got, want = p.download(), ptrue.download()
        sl = p.index_slices(p.assignableRange)
        rel = np.abs(got[sl] - want[sl]).max() / np.abs(want[sl]).max()
        assert rel <= 1e-7, (prec, rel)


def test_helmholtz_corner_dirichlet_and_3d_variable_coefficient(ctx):
    # (I - k Lap) u = f on a node grid with Dirichlet nodes
    n = 65
    mesh = cm.mesh_uniform([n, n])
    fd = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(0.0, 0.0)] * 2)
    u, f = api.CartesianField(mesh, fd, ctx), api.CartesianField(mesh, fd, ctx)
    a = f.download()
    a[1:-1, 1:-1] = np.random.default_rng(3).standard_normal((n - 2, n - 2))
    f.upload(a)
    k = 0.05
    getter = lambda e: api.Eq(e - k * (api.d2x(e) + api.d2y(e)), f)
    for prec in ("fp64", "mixed"):
        u.assign(0.0)
        st = api.Solve(getter, u, api.StructSolverParams(tol=1e-10, precision=prec))
        assert st.converged, st
        rel, _ = oracle_check(u, getter, u, False, 1e-10)
        assert rel <= 2e-10
    # 3D flux form with exp-like face coefficients, Neumann, pinned
    n = 24
    mesh = cm.mesh_uniform([n + 1] * 3)
    fd = cm.field_desc(3, capi.CENTER, [(capi.BC_NEUM, capi.BC_NEUM)] * 3, ext=1)
    p, K, g = (api.CartesianField(mesh, fd, ctx) for _ in range(3))
    K.initBy(lambda X: np.exp(np.sin(6.0 * X[0]) * np.cos(4.0 * X[1]) + 0.5 * X[2]))
    gv = g.download()
    sl = g.index_slices(g.assignableRange)
    v = np.random.default_rng(9).standard_normal(gv[sl].shape)
    gv[sl] = v - v.mean()
    g.upload(gv)
    getter = lambda e: g == (api.dx(api.d1IntpCenterToCorner(K, 0) * api.dx(e)) + api.dy(api.d1IntpCenterToCorner(K, 1) * api.dy(e))
                             + api.dz(api.d1IntpCenterToCorner(K, 2) * api.dz(e)))
    for prec in ("fp64", "mixed"):
        p.assign(0.0)
        st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, pinValue=True, precision=prec))
        assert st.converged, st
        rel, _ = oracle_check(p, getter, p, True, 1e-10)
        assert rel <= 2e-10, rel


def test_static_matrix_repeated_solves(ctx):
    """Backward-Euler heat steps: u_old == e - dt*(d2x(e)+d2y(e)), staticMat (generateb only)."""
    n = 64
    mesh = cm.mesh_uniform([n + 1, n + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, ext=1)
    u, uold = api.CartesianField(mesh, fd, ctx), api.CartesianField(mesh, fd, ctx)
    uold.initBy(lambda X: np.sin(np.pi * X[0]) * np.sin(np.pi * X[1]))
    dt = 1e-3
    h = api.makeEqnSolveHandler(lambda e: uold == e - dt * (api.d2x(e) + api.d2y(e)), u,
                                api.StructSolverParams(tol=1e-10, staticMat=True, precision="mixed"))
    for step in range(5):
        st = h.solve()
        assert st.converged, (step, st)
        rel, _ = oracle_check(u, lambda e: uold == e - dt * (api.d2x(e) + api.d2y(e)), u, False, 1e-10)
        assert rel <= 2e-10
        uold.assign(u)


def test_nonlinear_equation_is_rejected(ctx):
    mesh, fd, p, f = poisson_case(ctx, 16, capi.BC_DIRC)
    with pytest.raises(capi.OpflowError) as e:
        api.Solve(lambda e: f == e * api.d2x(e), p)
    assert e.value.code == capi.E_UNSUPPORTED


def test_logic_of_the_unknown_has_no_stencil_form(ctx):
    """Comparisons, conditionals and functions assemble only on values that do not depend on the
    unknown, and flux-limiter interpolation not at all: anything else is refused with E_UNSUPPORTED
    instead of being mis-assembled."""
    mesh, fd, p, f = poisson_case(ctx, 16, capi.BC_DIRC)
    for eq in (lambda e: f == api.d2x(e) + api.conditional(f > 0., e, 2. * e),
               lambda e: f == api.d2x(e) + api.abs(e),
               lambda e: f == api.d2x(e) + api.d1_flux_limiter_intp(f, e, 0, "QUICK")):
        with pytest.raises(capi.OpflowError) as err:
            api.Solve(eq, p)
        assert err.value.code == capi.E_UNSUPPORTED


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_iteration_cap_and_repeated_solves(ctx, prec):
    """The device-side solve loop stops at maxIter without converging, reports exactly maxIter
    iterations, and a handler solved again (graph replay) reaches the same answer as a fresh solve."""
    mesh, fd, p, f = poisson_case(ctx, 64, capi.BC_DIRC)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)
    p.assign(0.0)
    st = api.Solve(getter, p, api.StructSolverParams(tol=1e-30, maxIter=3, precision=prec))
    assert not st.converged and st.niter == 3, st
    p.assign(0.0)
    h = api.makeEqnSolveHandler(getter, p, api.StructSolverParams(tol=1e-10, maxIter=100, precision=prec, zeroGuess=True))
    s1 = h.solve()
    x1 = p.download()
    p.assign(1.0)  # a different guess: zeroGuess overrides it
    s2 = h.solve()
    x2 = p.download()
    h.close()
    assert s1.converged and s2.converged and s1.niter == s2.niter
    assert np.array_equal(x1, x2)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["neum_cell", "dirc_cell", "periodic_cell", "dirc_node"])
def test_fused_tiles_and_bottom_kernel_match_chunked_v_cycle(ctx, monkeypatch, prec, case):
    """The fused 2D tile kernels and the one-CTA bottom kernel reproduce the chunked V-cycle bit for
    bit (same per-cell arithmetic), on ragged extents with several tiles per level."""
    bc = {"neum": capi.BC_NEUM, "dirc": capi.BC_DIRC, "periodic": capi.BC_PERIODIC}[case.split("_")[0]]
    loc = capi.CENTER if case.endswith("cell") else capi.CORNER
    n = 300 if loc == capi.CENTER else 301
    mesh = cm.mesh_uniform([n + 1, n - 99] if loc == capi.CENTER else [n, n - 100])
    fd = cm.field_desc(2, loc, [(bc, bc)] * 2, ext=1 if loc == capi.CENTER else 0)
    p = api.CartesianField(mesh, fd, ctx)
    f = api.CartesianField(mesh, fd, ctx)
    a = f.download()
    sl = f.index_slices([(max(f.info.assignable[d][0], f.info.local[d][0]), min(f.info.assignable[d][1], f.info.local[d][1])) for d in range(2)])
    v = np.random.default_rng(11).standard_normal(a[sl].shape)
    if bc != capi.BC_DIRC:
        v -= v.mean()
    a[sl] = v
    f.upload(a)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)
    pin = bc != capi.BC_DIRC
    out = {}
    for mode, env in (("chunked", {"OPFLOW_MG_TILES": "0", "OPFLOW_MG_BOTTOM": "0"}), ("fused", {})):
        for k in ("OPFLOW_MG_TILES", "OPFLOW_MG_BOTTOM"):
            monkeypatch.delenv(k, raising=False)
        for k, val in env.items():
            monkeypatch.setenv(k, val)
        p.assign(0.0)
        st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, maxIter=100, pinValue=pin, precision=prec))
        out[mode] = (st.niter, st.relerr, p.download())
    assert out["chunked"][0] == out["fused"][0]
    assert out["chunked"][1] == out["fused"][1]
    assert np.array_equal(out["chunked"][2], out["fused"][2])
    assert out["fused"][1] <= 1e-10


@pytest.mark.parametrize("zb", ["tuned", "staged"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["neum_cell", "dirc_cell", "periodic_cell", "dirc_node", "neumvar_cell"])
def test_z_marching_smoother_matches_chunked_v_cycle(ctx, monkeypatch, prec, case, zb):
    """The z-marching 3D kernels reproduce the chunked V-cycle bit for bit, on ragged extents (tiles cut
    in x, y and z) with Neumann, Dirichlet, periodic and node-centred levels: with the tuner's choice
    per level, and with the TMA-staged smoother forced (OPFLOW_MG_ZB=16; float32 levels whose rows hold
    a multiple of 4 cells)."""
    if zb == "staged" and prec == "fp64":
        pytest.skip("the TMA-staged smoother runs float32 levels (the mixed-precision V-cycle) only")
    if zb == "staged":
        monkeypatch.setenv("OPFLOW_MG_ZB", "16")
    else:
        monkeypatch.delenv("OPFLOW_MG_ZB", raising=False)
    bc = {"neum": capi.BC_NEUM, "neumvar": capi.BC_NEUM, "dirc": capi.BC_DIRC, "periodic": capi.BC_PERIODIC}[case.split("_")[0]]
    loc = capi.CENTER if case.endswith("cell") else capi.CORNER
    # large enough for z tiles of at least 4 planes on level 0, ragged in x (30- and 32-wide tiles), y
    # and z; rows of 152 cells also take the staged smoother (a multiple of 4 cells)
    dims = [153, 84, 67] if loc == capi.CENTER else [129, 97, 65]  # (node levels: 2^k m + 1 nodes coarsen evenly)
    if bc == capi.BC_PERIODIC:
        dims = [153, 85, 67]  # even cell counts: red-black levels
    mesh = cm.mesh_uniform(dims)
    fd = cm.field_desc(3, loc, [(bc, bc)] * 3, ext=1 if loc == capi.CENTER else 0)
    p = api.CartesianField(mesh, fd, ctx)
    f = api.CartesianField(mesh, fd, ctx)
    a = f.download()
    sl = f.index_slices([(max(f.info.assignable[d][0], f.info.local[d][0]), min(f.info.assignable[d][1], f.info.local[d][1])) for d in range(3)])
    v = np.random.default_rng(13).standard_normal(a[sl].shape)
    if bc != capi.BC_DIRC:
        v -= v.mean()
    a[sl] = v
    f.upload(a)
    getter = lambda e: f == api.d2x(e) + api.d2y(e) + api.d2z(e)
    if case.startswith("neumvar"):
        # variable coefficient: coefficient arrays on every level instead of class tables
        K = api.CartesianField(mesh, fd, ctx)
        k = K.download()
        k[sl] = np.exp(0.5 * np.random.default_rng(14).standard_normal(k[sl].shape))
        K.upload(k)
        getter = lambda e: f == (api.dx(api.d1IntpCenterToCorner(K, 0) * api.dx(e)) + api.dy(api.d1IntpCenterToCorner(K, 1) * api.dy(e))
                                 + api.dz(api.d1IntpCenterToCorner(K, 2) * api.dz(e)))
    pin = bc != capi.BC_DIRC
    out = {}
    for mode, val in (("chunked", "0"), ("zmarch", "1")):
        monkeypatch.setenv("OPFLOW_MG_ZMARCH", val)
        p.assign(0.0)
        st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, maxIter=100, pinValue=pin, precision=prec))
        out[mode] = (st.niter, st.relerr, p.download())
    assert out["chunked"][0] == out["zmarch"][0]
    assert out["chunked"][1] == out["zmarch"][1]
    assert np.array_equal(out["chunked"][2], out["zmarch"][2])
    assert out["zmarch"][1] <= 1e-10

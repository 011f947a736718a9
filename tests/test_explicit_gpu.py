"""Path E on the GPU: the CUDA kernels against the reference's dumps (bit-exact) and the oracle."""
import ctypes as C
import os

import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

pytestmark = pytest.mark.gpu


def gpu_field(ctx, mesh, fd, host=None):
    f = api.CartesianField(mesh, fd, ctx)
    if host is not None:
        f.upload(host.data, update_padding=False)
    return f


def readable_of(f):
    return f.download()[f.index_slices(cm.readable(f.info))].reshape(-1)


@pytest.mark.parametrize("name", ["ftcs2d_n17", "ftcs2d_n33_bc1", "ftcs2d_n20_nonpow2", "ftcs2d_n65"])
def test_ftcs2d_gpu_matches_reference_dump(ctx, name):
    meta, arr = cm.golden(name)
    _, n, steps, seed, bcv, cfl = meta["args"]
    n, steps, seed, bcv, cfl = int(n), int(steps), int(seed), float(bcv), float(cfl)
    mesh = cm.mesh_uniform([n, n])
    fd = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(bcv, bcv)] * 2)
    h0 = orc.HostField(mesh, fd)
    cm.seeded_interior(h0, seed, n)
    h0.update_padding()
    u = gpu_field(ctx, mesh, fd, h0)
    h = 1.0 / (n - 1)
    u.assign(cm.ftcs_expr(u, cfl * h * h * 1.0, 2), steps=steps)
    got = readable_of(u)
    assert np.array_equal(got, arr["u__data"]), np.abs(got - arr["u__data"]).max()


@pytest.mark.parametrize("name", ["ftcs3d_n9", "ftcs3d_n12_nonpow2"])
def test_ftcs3d_gpu_matches_reference_dump(ctx, name):
    meta, arr = cm.golden(name)
    _, n, steps, seed, cfl = meta["args"]
    n, steps, cfl = int(n), int(steps), float(cfl)
    mesh = cm.mesh_uniform([n, n, n])
    fd = cm.field_desc(3, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 3)
    u = gpu_field(ctx, mesh, fd, orc.HostField(mesh, fd, data=arr["u0__data"]))
    h = 1.0 / (n - 1)
    u.assign(cm.ftcs_expr(u, cfl * h * h * 1.0, 3), steps=steps)
    assert np.array_equal(u.download().reshape(-1), arr["u__data"])


@pytest.mark.parametrize("name", ["weno_down_32x4", "weno_up_64x3", "weno_down_40x2_nonpow2"])
def test_weno_rk3_gpu_interpreter_matches_reference_dump(ctx, name):
    meta, arr = cm.golden(name)
    _, nx, ny, steps, seed, up = meta["args"]
    nx, ny, steps, up = int(nx), int(ny), int(steps), int(up)
    mesh = cm.mesh_uniform([nx + 1, ny + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_PERIODIC, capi.BC_PERIODIC)] * 2, ext=3)
    h0 = orc.HostField(mesh, fd, data=arr["u0__data"])
    u, u1, u2 = (gpu_field(ctx, mesh, fd, h0) for _ in range(3))
    dt = 0.5 * (1.0 / nx)
    e1, e2, e3 = cm.weno_stage_exprs(u, u1, u2, dt, upwind=bool(up))
    for _ in range(steps):
        u1.assign(e1)
        u2.assign(e2)
        u.assign(e3)
    assert np.array_equal(u.download().reshape(-1), arr["u__data"])


@pytest.mark.parametrize("name", ["weno_down_32x4", "weno_up_64x3", "weno_down_40x2_nonpow2"])
@pytest.mark.parametrize("fused_steps", [1, 0])
def test_weno_rk3_fused_kernel_matches_reference_dump(ctx, name, fused_steps):
    """The one-kernel RK3 step (all stages in shared memory), stepping once per call or all steps in
    one launch, against the reference's three-assignment result."""
    meta, arr = cm.golden(name)
    _, nx, ny, steps, seed, up = meta["args"]
    nx, ny, steps, up = int(nx), int(ny), int(steps), int(up)
    mesh = cm.mesh_uniform([nx + 1, ny + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_PERIODIC, capi.BC_PERIODIC)] * 2, ext=3)
    h0 = orc.HostField(mesh, fd, data=arr["u0__data"])
    u, u1, u2 = (gpu_field(ctx, mesh, fd, h0) for _ in range(3))
    dt = 0.5 * (1.0 / nx)
    if fused_steps:
        for _ in range(steps):
            api.weno_rk3(u, dt, 1, upwind=bool(up), u1=u1, u2=u2)
    else:
        api.weno_rk3(u, dt, steps, upwind=bool(up))
    assert np.array_equal(u.download().reshape(-1), arr["u__data"])


def test_weno_rk3_fused_4096_lines_matches_oracle(ctx):
    """Full line length of the WENO configuration (4096 periodic cells) on a few lines."""
    nx, ny, steps = 4096, 3, 2
    mesh = cm.mesh_uniform([nx + 1, ny + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_PERIODIC, capi.BC_PERIODIC)] * 2, ext=3)
    h0 = orc.HostField(mesh, fd)
    rng = h0.assignable()
    x = (np.arange(nx) + 0.5) / nx
    for j in range(ny):
        h0.data[h0.slices([rng[0], (j, j + 1)])] = (np.where((x > 0.2 + 0.1 * j) & (x < 0.5), 1.0, 0.0) + 0.3 * np.sin(2 * np.pi * (j + 1) * x))
    h0.update_padding()
    u = gpu_field(ctx, mesh, fd, h0)
    dt = 0.5 / nx
    api.weno_rk3(u, dt, steps)
    L = [cm.Leaf("u"), cm.Leaf("u1"), cm.Leaf("u2")]
    e = cm.weno_stage_exprs(L[0], L[1], L[2], dt)
    ns = [api.serialize(x, L)[0] for x in e]
    h1 = orc.HostField(mesh, fd, data=h0.data.copy())
    h2 = orc.HostField(mesh, fd, data=h0.data.copy())
    for _ in range(steps):
        orc.assign(h1, ns[0], [h0, h1, h2])
        orc.assign(h2, ns[1], [h0, h1, h2])
        orc.assign(h0, ns[2], [h0, h1, h2])
    assert np.array_equal(u.download(), h0.data)


def _weno_lines(ctx, nx, ny, seed):
    from opflow_gb300 import workloads as wl
    mesh = api.MeshBuilder().newMesh(nx + 1, ny + 1).setMeshOfDim(0, 0.0, 1.0).setMeshOfDim(1, 0.0, ny / nx).build()
    b = api.ExprBuilder().setMesh(mesh).setLoc(api.LocOnMesh.Center).setExt(3)
    for d in range(2):
        b.setBC(d, api.DimPos.start, api.BCType.Periodic, 0.0).setBC(d, api.DimPos.end, api.BCType.Periodic, 0.0)
    fields = [b.setName(nm).build(ctx) for nm in ("exact", "fast")]
    host = fields[0].download()
    host[fields[0].index_slices(fields[0].assignableRange)] = wl.weno_u0(seed, nx, ny)
    for f in fields:
        f.upload(host)
    return fields, float(np.abs(host).max())


@pytest.mark.parametrize("ny,steps,upwind", [(65536, 1, False), (65536, 20, False), (1024, 1, True)])
def test_weno_rk3_fast_mode_within_1e14_of_exact(ctx, ny, steps, upwind):
    """FAST mode (contracted arithmetic, one reciprocal for the nonlinear weights) against the bit-exact
    kernel on 4096-cell periodic lines with square and cosine pulses (the benchmark's data), at the
    benchmark's 65536 lines: within 4 ulps of max|u| after one RK3 step, within 1e-14 * max|u| after 20
    (the bound stated in opflow_weno_rk3_mode's contract).  The Upwind operator in u_t + L(u) = 0 is
    the downstream-biased stencil, which amplifies differences from step to step, so it is compared
    over one step."""
    nx = 4096
    (ue, uf), umax = _weno_lines(ctx, nx, ny, 77)
    dt = 0.5 / nx
    api.weno_rk3(ue, dt, steps, upwind=upwind)
    api.weno_rk3(uf, dt, steps, upwind=upwind, mode=capi.EVAL_FAST)
    a, b = ue.download(), uf.download()
    err = float(np.abs(a - b).max())
    assert np.isfinite(b).all()
    assert err <= (4 * 2.0 ** -52 if steps == 1 else 1e-14) * umax, err
    assert err > 0.0  # FAST is a different evaluation, not the exact one


def test_weno_rk3_fast_mode_long_runs_stay_within_the_schemes_own_sensitivity(ctx):
    """Over 100 RK3 steps WENO5-JS amplifies rounding-level differences at the pulses' edges (the
    nonlinear weights switch there): the exact scheme started from data moved by one ulp ends up to
    ~1e-8 away from itself.  FAST's distance from EXACT after 100 steps stays below that distance."""
    nx, ny, steps = 4096, 1024, 100
    (ue, uf), umax = _weno_lines(ctx, nx, ny, 77)
    host = ue.download()
    sl = ue.index_slices(ue.assignableRange)
    v = host[sl]
    nz = v != 0
    v[nz] = np.nextafter(v[nz], 2.0)
    host[sl] = v
    (up_, _), _ = _weno_lines(ctx, nx, ny, 77)
    up_.upload(host)
    dt = 0.5 / nx
    api.weno_rk3(ue, dt, steps)
    api.weno_rk3(up_, dt, steps)
    api.weno_rk3(uf, dt, steps, mode=capi.EVAL_FAST)
    a = ue.download()
    ulp_spread = float(np.abs(up_.download() - a).max())
    fast_err = float(np.abs(uf.download() - a).max())
    assert 0.0 < fast_err <= ulp_spread, (fast_err, ulp_spread)


PAD = sorted(f[:-4] for f in os.listdir(cm.GOLDEN) if f.startswith("pad_"))


@pytest.mark.parametrize("name", PAD)
def test_padding_gpu_matches_reference_dump(ctx, name):
    meta, arr = cm.golden(name)
    _, nx, ny, loc, lo, hi, ext = meta["args"]
    nx, ny, loc, lo, hi, ext = map(int, (nx, ny, loc, lo, hi, ext))
    code = [capi.BC_DIRC, capi.BC_NEUM, capi.BC_PERIODIC, capi.BC_SYMM, capi.BC_ASYMM]
    mesh = cm.mesh_uniform([nx, ny], [(0.0, 1.0), (0.0, 2.0)])
    fd = cm.field_desc(2, capi.CENTER if loc else capi.CORNER, [(code[lo], code[hi]), (code[hi], code[lo])],
                       [(0.25, -0.5), (0.75, 1.5)], ext=ext)
    f = api.CartesianField(mesh, fd, ctx)
    f.initBy(lambda X: 1.0 + X[0] * X[0] - 0.5 * X[1] + 0.25 * X[0] * X[1])
    assert np.array_equal(readable_of(f), arr["f__data"])


def _vc_case(ctx, n, seed):
    mesh = cm.mesh_uniform([n + 1, n + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_NEUM), (capi.BC_SYMM, capi.BC_DIRC)], [(0.5, -1.0), (0.0, 2.0)], ext=1)
    hosts = []
    for s in range(3):
        hf = orc.HostField(mesh, fd)
        rng = hf.assignable()
        j, i = np.meshgrid(np.arange(*rng[1]), np.arange(*rng[0]), indexing="ij")
        hf.data[hf.slices(rng)] = 0.5 + orc.u01(seed + s, j.astype(np.uint64) * np.uint64(977) + i.astype(np.uint64))
        hf.update_padding()
        hosts.append(hf)
    return mesh, fd, hosts


def test_generic_interpreter_matches_oracle(ctx):
    """Flux-form variable-coefficient operator, first-order centred derivatives, linear interpolation,
    negation and division on a mixed-BC cell-centred field: the generic kernel vs the oracle."""
    mesh, fd, hosts = _vc_case(ctx, 24, 3)
    g = [gpu_field(ctx, mesh, fd, h) for h in hosts]
    L = [cm.Leaf(k) for k in "uvr"]

    def expr(u, v, r):
        return (api.dx(api.dx(u) / api.d1IntpCenterToCorner(r, 0)) + api.dy(api.dy(u) / api.d1IntpCenterToCorner(r, 1))
                - (-v) / (u + 2.0) * 0.3)

    nodes, _ = api.serialize(expr(*L), L)
    out_h = orc.HostField(mesh, fd)
    orc.assign(out_h, nodes, hosts + [out_h])
    out = api.CartesianField(mesh, fd, ctx)
    out.assign(expr(*g))
    assert np.array_equal(readable_of(out), out_h.data[out_h.slices(cm.readable(out_h.info))].reshape(-1))


def test_aliased_incremental_assign_matches_oracle(ctx):
    """u += d2x(u) * v reads u while writing it: FieldAssigner's out-of-place semantics."""
    mesh, fd, hosts = _vc_case(ctx, 20, 11)
    u, v = gpu_field(ctx, mesh, fd, hosts[0]), gpu_field(ctx, mesh, fd, hosts[1])
    Lu, Lv = cm.Leaf("u"), cm.Leaf("v")
    nodes, _ = api.serialize(api.d2x(Lu) * Lv, [Lu, Lv])
    orc.assign(hosts[0], nodes, [hosts[0], hosts[1]], op=capi.ASSIGN_ADD)
    u.assign(api.d2x(u) * v, op="+")
    assert np.array_equal(readable_of(u), hosts[0].data[hosts[0].slices(cm.readable(hosts[0].info))].reshape(-1))


def test_out_of_range_stencil_is_an_error_not_a_fault(ctx):
    mesh = cm.mesh_uniform([17, 17])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_PERIODIC, capi.BC_PERIODIC)] * 2, ext=1)
    u, w = api.CartesianField(mesh, fd, ctx), api.CartesianField(mesh, fd, ctx)
    with pytest.raises(capi.OpflowError) as e:
        w.assign(api.d1_weno53_downwind(u, 0))  # needs 3 ghost cells, the field has 1
    assert e.value.code == capi.E_RANGE


def test_ftcs2d_full_config_1025_1000_steps_bitexact(ctx):
    """The CPU-runnable FTCS2D case at full size: 1025^2 nodes, Dirichlet 0, u0 ~ U[0,1), dt = 0.2 h^2,
    1000 steps; GPU field vs the oracle, every value."""
    n, steps = 1025, 1000
    mesh = cm.mesh_uniform([n, n])
    fd = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2)
    h0 = orc.HostField(mesh, fd)
    cm.seeded_interior(h0, 2024, n)
    h0.update_padding()
    u = gpu_field(ctx, mesh, fd, h0)
    h = 1.0 / (n - 1)
    s = 0.2 * h * h * 1.0
    u.assign(cm.ftcs_expr(u, s, 2), steps=steps)
    orc.lib().or_set_threads(os.cpu_count() or 1)
    leaf = cm.Leaf("u")
    nodes, _ = api.serialize(cm.ftcs_expr(leaf, s, 2))
    for _ in range(steps):
        orc.assign(h0, nodes, [h0])
    assert np.array_equal(u.download(), h0.data)


@pytest.mark.parametrize("dims,steps,cfl", [((257, 257), 400, 0.2), ((65, 65, 65), 120, 0.1), ((48, 40, 33), 60, 0.1)])
def test_fast_mode_within_1e14_of_exact(ctx, dims, steps, cfl):
    """OPFLOW_EVAL_FAST (fixed-point) against the bit-exact kernel: normwise relative error <= 1e-14."""
    D = len(dims)
    mesh = cm.mesh_uniform(list(dims))
    fd = cm.field_desc(D, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * D, [(0.25, 0.25)] * D)
    ue, uf = api.CartesianField(mesh, fd, ctx), api.CartesianField(mesh, fd, ctx)
    a = ue.download()
    rng = np.random.default_rng(1)
    inner = tuple(slice(1, -1) for _ in range(D))
    a[inner] = rng.random(a[inner].shape)
    ue.upload(a)
    uf.upload(a)
    hx = 1.0 / (dims[0] - 1)
    s = cfl * hx * hx
    ue.assign(cm.ftcs_expr(ue, s, D), steps=steps, mode="exact")
    uf.assign(cm.ftcs_expr(uf, s, D), steps=steps, mode="fast")
    e, f = ue.download(), uf.download()
    rel = np.abs(e - f).max() / np.abs(e).max()
    assert rel <= 1e-14, rel


@pytest.mark.parametrize("tiling", ["register", "smem"])
@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_ftcs3d_ragged_tiles_match_oracle(ctx, monkeypatch, tiling, mode):
    """3D FTCS on extents that cut every tile and z-chunk: exact mode bit-exact with the oracle, fast
    mode within 1e-14 normwise; both 3D tilings."""
    monkeypatch.setenv("OPFLOW_AXIS_TILING", tiling)
    dims, steps = (97, 43, 70), 6
    mesh = cm.mesh_uniform(list(dims))
    fd = cm.field_desc(3, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 3)
    h0 = orc.HostField(mesh, fd)
    sl = h0.slices(h0.assignable())
    h0.data[sl] = np.random.default_rng(77).random(h0.data[sl].shape)
    h0.update_padding()
    u = gpu_field(ctx, mesh, fd, h0)
    hx = 1.0 / (dims[0] - 1)
    s = 0.1 * hx * hx
    u.assign(cm.ftcs_expr(u, s, 3), steps=steps, mode=mode)
    leaf = cm.Leaf("u")
    nodes, _ = api.serialize(cm.ftcs_expr(leaf, s, 3))
    for _ in range(steps):
        orc.assign(h0, nodes, [h0])
    got = u.download()
    if mode == "exact":
        assert np.array_equal(got, h0.data)
    else:
        rel = np.abs(got - h0.data).max() / np.abs(h0.data).max()
        assert rel <= 1e-14, rel


def test_fast_resident_run_at_the_512_config_within_1e14_of_exact(ctx, monkeypatch):
    """The 512^3 x 200-step FTCS3D configuration (8 seeded Gaussians, Dirichlet 0, dt = 0.1 h^2): the
    fixed-point run that keeps the field in fixed point between steps is within 1e-14 (normwise
    relative) of the bit-exact IEEE run, and so is the per-step form it replaces."""
    torch = pytest.importorskip("torch")
    import bench
    n, steps = 512, 200
    mesh = cm.mesh_uniform([n] * 3)
    fd = cm.field_desc(3, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 3)
    u0 = bench.gaussians_u0(torch, n, 1234, torch.device("cuda", 0)).cpu().numpy()
    h = 1.0 / (n - 1)
    s = 0.1 * h * h
    out = {}
    for name, mode, env in (("exact", "exact", "1"), ("resident", "fast", "1"), ("per_step", "fast", "0")):
        monkeypatch.setenv("OPFLOW_FX_RESIDENT", env)
        u = api.CartesianField(mesh, fd, ctx)
        u.upload(u0)
        u.assign(cm.ftcs_expr(u, s, 3), steps=steps, mode=mode)
        out[name] = u.download()
        del u
    e = out["exact"]
    for name in ("resident", "per_step"):
        rel = np.abs(out[name] - e).max() / np.abs(e).max()
        print("\n512^3 x %d FTCS3D: %s fixed point vs exact: %.2e" % (steps, name, rel))
        assert rel <= 1e-14, (name, rel)


@pytest.mark.parametrize("dims,steps,bcv", [((1025, 1025), 1000, 0.0), ((100, 37), 300, 0.5), ((33, 70), 200, -0.75)])
def test_fast_resident_2d_runs_within_1e14_of_exact(ctx, monkeypatch, dims, steps, bcv):
    """Resident fixed-point runs on 2D node grids (axis2d_fxres_kernel): the FTCS2D configuration (1025^2,
    U[0,1) interior, Dirichlet 0, dt = 0.2 h^2, 1000 steps) and ragged grids with two weights and nonzero
    Dirichlet values, against the bit-exact IEEE run: normwise relative error <= 1e-14, and so is the
    per-step fixed-point form."""
    mesh = cm.mesh_uniform(list(dims))
    fd = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(bcv, bcv)] * 2)
    h0 = orc.HostField(mesh, fd)
    cm.seeded_interior(h0, 2024, dims[0])
    h0.update_padding()
    hmin = 1.0 / (max(dims) - 1)
    s = 0.2 * hmin * hmin
    out = {}
    for name, mode, env in (("exact", "exact", "1"), ("resident", "fast", "1"), ("per_step", "fast", "0")):
        monkeypatch.setenv("OPFLOW_FX_RESIDENT", env)
        u = gpu_field(ctx, mesh, fd, h0)
        u.assign(cm.ftcs_expr(u, s, 2), steps=steps, mode=mode)
        out[name] = u.download()
        del u
    e = out["exact"]
    for name in ("resident", "per_step"):
        rel = np.abs(out[name] - e).max() / np.abs(e).max()
        print("\n%s x %d FTCS2D: %s fixed point vs exact: %.2e" % (dims, steps, name, rel))
        assert rel <= 1e-14, (name, rel)
    # the boundary nodes hold their float64 constants again
    assert np.all(out["resident"][0, :] == bcv) and np.all(out["resident"][:, -1] == bcv)


@pytest.mark.parametrize("dims", [(150, 83, 70), (96, 96, 96), (67, 40, 37)])
def test_fast_resident_tma_staged_and_register_steps_bit_identical(ctx, monkeypatch, dims):
    """The steady-state step of a resident fixed-point run in its two forms - planes staged in shared
    memory by TMA (axis3d_fxtma_kernel) and register-blocked (axis3d_fxres_kernel) - gives the same
    fields bit for bit: ragged tiles in x, y and z, one weight (cube) and three weights, Dirichlet 0.5."""
    steps = 9
    mesh = cm.mesh_uniform(list(dims))
    fd = cm.field_desc(3, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 3, [(0.5, 0.5)] * 3)
    a = np.random.default_rng(sum(dims)).random([d for d in reversed(dims)])
    hmin = 1.0 / (max(dims) - 1)
    res = {}
    for env in ("1", "0"):
        monkeypatch.setenv("OPFLOW_FXRES_TMA", env)
        u = api.CartesianField(mesh, fd, ctx)
        b = u.download()
        b[1:-1, 1:-1, 1:-1] = a[1:-1, 1:-1, 1:-1]
        u.upload(b)
        u.assign(cm.ftcs_expr(u, 0.1 * hmin * hmin, 3), steps=steps, mode="fast")
        res[env] = u.download()
        del u
    assert np.array_equal(res["1"], res["0"])


def test_fast_resident_falls_back_when_weights_break_the_maximum_principle(ctx, monkeypatch):
    """dt = 0.4 hx^2 on a grid with hx > hy > hz (1 - 2 sum_d w_d < 0): no resident run, the per-step
    form runs (bit-identical with and without the switch)."""
    dims, steps = (40, 36, 33), 3
    mesh = cm.mesh_uniform(list(dims))
    fd = cm.field_desc(3, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 3, [(0.5, 0.5)] * 3)
    a = np.random.default_rng(4).random([d for d in reversed(dims)])
    res = {}
    for env in ("1", "0"):
        monkeypatch.setenv("OPFLOW_FX_RESIDENT", env)
        u = api.CartesianField(mesh, fd, ctx)
        b = u.download()
        b[1:-1, 1:-1, 1:-1] = a[1:-1, 1:-1, 1:-1]
        u.upload(b)
        hx = 1.0 / (dims[0] - 1)
        u.assign(cm.ftcs_expr(u, 0.4 * hx * hx, 3), steps=steps, mode="fast")
        res[env] = u.download()
    assert np.array_equal(res["1"], res["0"])

"""One-sided first differences (D1FirstOrderBiasedUpwind / D1FirstOrderBiasedDownwind) and corner-to-
centre interpolation (D1Linear Cor2Cen) against the reference's own outputs.

The fixtures ops_*, conv1d_n101 and asm_biased2d_n12 were written by OpFlow's CPU code
(tests/golden/make_golden.py running oracle/_ref/ref_driver): a stretched 2D mesh with a cell-centred
field (Dirichlet/Neumann along x, periodic along y) and a nodal field (Dirichlet along x,
Neumann/Dirichlet along y), each operator assigned into a field of the matching location, and the
reference's examples/CONV1D run for 100 steps.  The oracle must reproduce them bit for bit (CPU), and
so must the CUDA library (GPU tests, through the C ABI).
"""
import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

OPS = ["ops_12x9", "ops_16x20"]
C_DESC = dict(loc=capi.CENTER, bcs=[(capi.BC_DIRC, capi.BC_NEUM), (capi.BC_PERIODIC, capi.BC_PERIODIC)],
              values=[(0.5, -1.0), (0.0, 0.0)])
V_DESC = dict(loc=capi.CORNER, bcs=[(capi.BC_DIRC, capi.BC_DIRC), (capi.BC_NEUM, capi.BC_DIRC)],
              values=[(0.25, -0.75), (0.0, 1.0)])
W_BCS = [(capi.BC_DIRC, capi.BC_DIRC), (capi.BC_NEUM, capi.BC_DIRC)]


def _desc(d, ext=1):
    return cm.field_desc(2, d["loc"], d["bcs"], d["values"], ext=ext)


def _ops_case(name):
    meta, arr = cm.golden(name)
    _, nx, ny, seed = meta["args"]
    nx, ny, seed = int(nx), int(ny), int(seed)
    mesh = cm.mesh_points([cm.stretched_points(nx + 1), cm.stretched_points(ny + 1, 2.0)])
    return meta, arr, nx, ny, seed, mesh


def _seed(hf, seed, n_line):
    rng = hf.assignable()
    j, i = np.meshgrid(np.arange(*rng[1]), np.arange(*rng[0]), indexing="ij")
    hf.data[hf.slices(rng)] = orc.u01(seed, j.astype(np.uint64) * np.uint64(n_line) + i.astype(np.uint64))
    hf.update_padding()


def _exprs():
    """(output key, destination desc, expression of the leaves c, v)."""
    w0 = cm.field_desc(2, [capi.CENTER, capi.CORNER], W_BCS)
    w1 = cm.field_desc(2, [capi.CORNER, capi.CENTER], W_BCS)
    return [
        ("c_up0", _desc(C_DESC), lambda c, v: api.d1_biased_upwind(c, 0)),
        ("c_dn1", _desc(C_DESC), lambda c, v: api.d1_biased_downwind(c, 1)),
        ("c_mix", _desc(C_DESC), lambda c, v: c + 0.25 * api.d1IntpCornerToCenter(api.d1IntpCornerToCenter(v, 0), 1)
                                     - 0.3 * api.dx(c, api.D1FirstOrderBiasedDownwind)),
        ("v_up1", _desc(V_DESC), lambda c, v: api.dy(v, api.D1FirstOrderBiasedUpwind)),
        ("v_dn0", _desc(V_DESC), lambda c, v: api.dx(v, api.D1FirstOrderBiasedDownwind)),
        ("w0", w0, lambda c, v: api.d1IntpCornerToCenter(v, 0)),
        ("w1", w1, lambda c, v: api.d1IntpCornerToCenter(v, 1)),
    ]


def _readable(hf):
    return hf.data[hf.slices(cm.readable(hf.info))].reshape(-1)


@pytest.mark.parametrize("name", OPS)
def test_stretched_mesh_matches_reference(name):
    """MeshBuilder::setMeshOfDim(k, f) with the Symm extension, restated by the oracle."""
    meta, arr, nx, ny, seed, mesh = _ops_case(name)
    for d in range(2):
        assert np.array_equal(np.asarray(mesh.x[d]), arr["mesh_x%d__data" % d])
        assert np.array_equal(np.asarray(mesh.dx[d]), arr["mesh_dx%d__data" % d])


@pytest.mark.parametrize("name", OPS)
def test_one_sided_ops_oracle_bitexact(name):
    meta, arr, nx, ny, seed, mesh = _ops_case(name)
    c = orc.HostField(mesh, _desc(C_DESC))
    v = orc.HostField(mesh, _desc(V_DESC))
    _seed(c, seed, nx)
    _seed(v, seed + 1, nx + 1)
    assert np.array_equal(_readable(c), arr["c__data"])
    assert np.array_equal(_readable(v), arr["v__data"])
    Lc, Lv = cm.Leaf("c"), cm.Leaf("v")
    for key, fd, fn in _exprs():
        out = orc.HostField(mesh, fd)
        nodes, _ = api.serialize(fn(Lc, Lv), [Lc, Lv])
        orc.assign(out, nodes, [c, v, out])
        got = _readable(out)
        assert np.array_equal(got, arr[key + "__data"]), key


def _conv1d_setup(arr):
    mesh = cm.mesh_uniform([101])
    fd = cm.field_desc(1, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)])
    u = orc.HostField(mesh, fd)
    rng = u.assignable()
    x = np.array([mesh.x_at(0, i) for i in range(*rng[0])])
    u.data[u.slices(rng)] = np.where((0.2 <= x) & (x <= 0.4), 1.0, 0.0)
    u.update_padding()
    assert np.array_equal(_readable(u), arr["u0__data"])
    return mesh, fd, u


def _conv1d_expr(u):
    dt, c = 0.5e-2, 1.0
    return u - dt * c * api.dx(u, api.D1FirstOrderBiasedDownwind)


def test_conv1d_example_oracle_bitexact():
    meta, arr = cm.golden("conv1d_n101")
    mesh, fd, u = _conv1d_setup(arr)
    L = cm.Leaf("u")
    nodes, _ = api.serialize(_conv1d_expr(L))
    for _ in range(int(meta["args"][2])):
        orc.assign(u, nodes, [u])
    assert np.array_equal(_readable(u), arr["u__data"])


# ------------------------------------------------------------------------------------------- GPU
def _gpu_readable(f):
    return f.download()[f.index_slices(cm.readable(f.info))].reshape(-1)


@pytest.mark.gpu
@pytest.mark.parametrize("name", OPS)
def test_one_sided_ops_gpu_matches_reference_dump(ctx, name):
    meta, arr, nx, ny, seed, mesh = _ops_case(name)
    hc = orc.HostField(mesh, _desc(C_DESC))
    hv = orc.HostField(mesh, _desc(V_DESC))
    _seed(hc, seed, nx)
    _seed(hv, seed + 1, nx + 1)
    c = api.CartesianField(mesh, _desc(C_DESC), ctx)
    v = api.CartesianField(mesh, _desc(V_DESC), ctx)
    c.upload(hc.data, update_padding=False)
    v.upload(hv.data, update_padding=False)
    for key, fd, fn in _exprs():
        out = api.CartesianField(mesh, fd, ctx)
        out.assign(fn(c, v))
        assert np.array_equal(_gpu_readable(out), arr[key + "__data"]), key


@pytest.mark.gpu
@pytest.mark.parametrize("mode", ["exact", "fast"])
def test_conv1d_example_gpu(ctx, mode):
    """examples/CONV1D on the GPU: bit-exact in exact mode; in fast mode the fixed-point kernel
    (one rounding per point) stays within 1e-14 of the reference normwise."""
    meta, arr = cm.golden("conv1d_n101")
    mesh, fd, hu = _conv1d_setup(arr)
    u = api.CartesianField(mesh, fd, ctx)
    u.upload(hu.data, update_padding=False)
    for _ in range(int(meta["args"][2])):
        u.assign(_conv1d_expr(u), mode=mode)
    got, want = _gpu_readable(u), arr["u__data"]
    if mode == "exact":
        assert np.array_equal(got, want)
    else:
        assert np.linalg.norm(got - want) <= 1e-14 * np.linalg.norm(want)

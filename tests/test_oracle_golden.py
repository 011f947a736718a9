"""The CPU oracle (oracle/oracle.c) against the reference's own outputs.

The fixtures under tests/golden/ were produced by OpFlow's CPU code itself (tests/golden/make_golden.py
running oracle/_ref/ref_driver) and by the literal systems of the reference's
CSRMatrixGeneratorTest.cpp.  Every comparison here is bit-for-bit.
"""
import json
import os

import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

FTCS2D = ["ftcs2d_n17", "ftcs2d_n33_bc1", "ftcs2d_n20_nonpow2", "ftcs2d_n65"]


def _ranges_match(info, rec):
    for key in ("logical", "accessible", "assignable", "local"):
        got = [[getattr(info, key)[d][0], getattr(info, key)[d][1]] for d in range(info.ndim)]
        assert got == rec[key], key
    assert [list(r) for r in cm.readable(info)] == rec["readable"]


@pytest.mark.parametrize("name", FTCS2D)
def test_ftcs2d_oracle_bitexact(name):
    meta, arr = cm.golden(name)
    _, n, steps, seed, bcv, cfl = meta["args"]
    n, steps, seed, bcv, cfl = int(n), int(steps), int(seed), float(bcv), float(cfl)
    mesh = cm.mesh_uniform([n, n])
    fd = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(bcv, bcv)] * 2)
    u = orc.HostField(mesh, fd)
    _ranges_match(u.info, cm.record(meta, "u"))
    cm.seeded_interior(u, seed, n)
    u.update_padding()
    h = 1.0 / (n - 1)
    s = cfl * h * h * 1.0
    leaf = cm.Leaf("u")
    nodes, leaves = api.serialize(cm.ftcs_expr(leaf, s, 2))
    for _ in range(steps):
        orc.assign(u, nodes, [u])
    got = u.data[u.slices(cm.readable(u.info))].reshape(-1)
    want = arr["u__data"]
    assert np.array_equal(got, want), "max diff %g" % np.abs(got - want).max()


@pytest.mark.parametrize("name", ["ftcs3d_n9", "ftcs3d_n12_nonpow2"])
def test_ftcs3d_oracle_bitexact(name):
    meta, arr = cm.golden(name)
    _, n, steps, seed, cfl = meta["args"]
    n, steps, cfl = int(n), int(steps), float(cfl)
    mesh = cm.mesh_uniform([n, n, n])
    fd = cm.field_desc(3, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 3)
    u = orc.HostField(mesh, fd, data=arr["u0__data"])  # the reference's initBy (std::exp) output
    h = 1.0 / (n - 1)
    s = cfl * h * h * 1.0
    nodes, _ = api.serialize(cm.ftcs_expr(cm.Leaf("u"), s, 3))
    for _ in range(steps):
        orc.assign(u, nodes, [u])
    assert np.array_equal(u.data.reshape(-1), arr["u__data"])


@pytest.mark.parametrize("name", ["weno_down_32x4", "weno_up_64x3", "weno_down_40x2_nonpow2"])
def test_weno_rk3_oracle_bitexact(name):
    meta, arr = cm.golden(name)
    _, nx, ny, steps, seed, up = meta["args"]
    nx, ny, steps, up = int(nx), int(ny), int(steps), int(up)
    mesh = cm.mesh_uniform([nx + 1, ny + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_PERIODIC, capi.BC_PERIODIC)] * 2, ext=3)
    u = orc.HostField(mesh, fd, data=arr["u0__data"])
    _ranges_match(u.info, cm.record(meta, "u"))
    u1 = orc.HostField(mesh, fd, data=u.data.copy())
    u2 = orc.HostField(mesh, fd, data=u.data.copy())
    dt = 0.5 * (1.0 / nx)
    L = [cm.Leaf("u"), cm.Leaf("u1"), cm.Leaf("u2")]
    e1, e2, e3 = cm.weno_stage_exprs(L[0], L[1], L[2], dt, upwind=bool(up))
    n1, _ = api.serialize(e1, L)
    n2, _ = api.serialize(e2, L)
    n3, _ = api.serialize(e3, L)
    for _ in range(steps):
        orc.assign(u1, n1, [u, u1, u2])
        orc.assign(u2, n2, [u, u1, u2])
        orc.assign(u, n3, [u, u1, u2])
    assert np.array_equal(u.data.reshape(-1), arr["u__data"])


PAD = sorted(f[:-4] for f in os.listdir(cm.GOLDEN) if f.startswith("pad_"))


@pytest.mark.parametrize("name", PAD)
def test_padding_and_ranges_oracle_bitexact(name):
    meta, arr = cm.golden(name)
    _, nx, ny, loc, lo, hi, ext = meta["args"]
    nx, ny, loc, lo, hi, ext = map(int, (nx, ny, loc, lo, hi, ext))
    code = [capi.BC_DIRC, capi.BC_NEUM, capi.BC_PERIODIC, capi.BC_SYMM, capi.BC_ASYMM]
    mesh = cm.mesh_uniform([nx, ny], [(0.0, 1.0), (0.0, 2.0)])
    fd = cm.field_desc(2, capi.CENTER if loc else capi.CORNER, [(code[lo], code[hi]), (code[hi], code[lo])],
                       [(0.25, -0.5), (0.75, 1.5)], ext=ext)
    f = orc.HostField(mesh, fd)
    rec = cm.record(meta, "f")
    _ranges_match(f.info, rec)
    # the library's GPU-free range computation must agree too
    info2 = api.describe(mesh, fd)
    _ranges_match(info2, rec)
    rng = f.assignable()
    xs = []
    for d in range(2):
        idx = np.arange(*rng[d])
        x = np.array([mesh.x_at(d, i) for i in idx])
        if loc:
            x = x + .5 * np.array([mesh.dx_at(d, i) for i in idx])
        xs.append(x)
    X1, X0 = np.meshgrid(xs[1], xs[0], indexing="ij")
    f.data[f.slices(rng)] = 1.0 + X0 * X0 - 0.5 * X1 + 0.25 * X0 * X1
    f.update_padding()
    got = f.data[f.slices(cm.readable(f.info))].reshape(-1)
    assert np.array_equal(got, arr["f__data"])


def _assemble_case(name, arr, meta):
    """Builds the oracle-side fields and the `lhs - rhs` tree of each assembly case."""
    args = meta["args"]
    which = args[1]
    n = int(args[2]) if len(args) > 2 else 0
    if which.startswith("csr_"):
        mesh = cm.mesh_uniform([5, 5], [(0.0, 4.0), (0.0, 4.0)])
        bc = {"csr_dirc": capi.BC_DIRC, "csr_neum": capi.BC_NEUM, "csr_periodic": capi.BC_PERIODIC}[which]
        p = orc.HostField(mesh, cm.field_desc(2, capi.CENTER, [(bc, bc)] * 2, ext=1))
        e = cm.Leaf("p")
        eq = api.Eq(1.0, api.d2x(e) + api.d2y(e))
        return p, {"p": p}, eq, which == "csr_neum"
    if which in ("neum2d", "dirc2d", "periodic2d"):
        mesh = cm.mesh_uniform([n + 1, n + 1])
        bc = {"neum2d": capi.BC_NEUM, "dirc2d": capi.BC_DIRC, "periodic2d": capi.BC_PERIODIC}[which]
        fd = cm.field_desc(2, capi.CENTER, [(bc, bc)] * 2, ext=1)
        p = orc.HostField(mesh, fd)
        f = orc.HostField(mesh, fd)
        rng = f.assignable()
        j, i = np.meshgrid(np.arange(*rng[1]), np.arange(*rng[0]), indexing="ij")
        f.data[f.slices(rng)] = orc.u01(7, j.astype(np.uint64) * np.uint64(n) + i.astype(np.uint64)) - 0.5
        f.update_padding()
        e, F = cm.Leaf("p"), cm.Leaf("f")
        return p, {"p": p, "f": f}, api.Eq(F, api.d2x(e) + api.d2y(e)), which != "dirc2d"
    if which == "var2d":
        mesh = cm.mesh_uniform([n + 1, n + 1])
        mk = lambda v: cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(v, v)] * 2, ext=1)
        p = orc.HostField(mesh, mk(0.0))
        r = orc.HostField(mesh, mk(1.0), data=None)
        b = orc.HostField(mesh, mk(0.0), data=None)
        r.data[r.slices(cm.readable(r.info))] = arr["r__data"].reshape(r.data[r.slices(cm.readable(r.info))].shape)
        b.data[b.slices(cm.readable(b.info))] = arr["b__data"].reshape(b.data[b.slices(cm.readable(b.info))].shape)
        e, R, B = cm.Leaf("p"), cm.Leaf("r"), cm.Leaf("b")
        rhs = api.dx(api.dx(e) / api.d1IntpCenterToCorner(R, 0)) + api.dy(api.dy(e) / api.d1IntpCenterToCorner(R, 1))
        return p, {"p": p, "r": r, "b": b}, api.Eq(B, rhs), False
    if which == "helm_corner":
        mesh = cm.mesh_uniform([n, n])
        fd = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(0.125, 0.125)] * 2)
        u = orc.HostField(mesh, fd)
        f = orc.HostField(mesh, fd, data=u.data.copy())
        rng = f.assignable()
        j, i = np.meshgrid(np.arange(*rng[1]), np.arange(*rng[0]), indexing="ij")
        f.data[f.slices(rng)] = orc.u01(13, j.astype(np.uint64) * np.uint64(n) + i.astype(np.uint64))
        e, F = cm.Leaf("u"), cm.Leaf("f")
        k = 0.0123
        return u, {"u": u, "f": f}, api.Eq(e - k * (api.d2x(e) + api.d2y(e)), F), False
    if which == "var3d":
        mesh = cm.mesh_uniform([n + 1] * 3)
        fd = cm.field_desc(3, capi.CENTER, [(capi.BC_NEUM, capi.BC_NEUM)] * 3, ext=1)
        p = orc.HostField(mesh, fd)
        K = orc.HostField(mesh, fd)
        f = orc.HostField(mesh, fd)
        K.data[K.slices(cm.readable(K.info))] = arr["K__data"].reshape(K.data[K.slices(cm.readable(K.info))].shape)
        f.data[f.slices(cm.readable(f.info))] = arr["f__data"].reshape(f.data[f.slices(cm.readable(f.info))].shape)
        e, KK, F = cm.Leaf("p"), cm.Leaf("K"), cm.Leaf("f")
        rhs = (api.dx(api.d1IntpCenterToCorner(KK, 0) * api.dx(e)) + api.dy(api.d1IntpCenterToCorner(KK, 1) * api.dy(e))
               + api.dz(api.d1IntpCenterToCorner(KK, 2) * api.dz(e)))
        return p, {"p": p, "K": K, "f": f}, api.Eq(F, rhs), True
    if which == "biased2d":
        mesh = cm.mesh_points([cm.stretched_points(n + 1), cm.stretched_points(n + 1, 2.0)])
        mk = lambda v: cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(v, v)] * 2, ext=1)
        p = orc.HostField(mesh, mk(0.25))
        K = orc.HostField(mesh, mk(1.0))
        f = orc.HostField(mesh, mk(0.0))
        for h, key in ((K, "K"), (f, "f")):
            h.data[h.slices(cm.readable(h.info))] = arr[key + "__data"].reshape(h.data[h.slices(cm.readable(h.info))].shape)
        e, KK, F = cm.Leaf("p"), cm.Leaf("K"), cm.Leaf("f")
        rhs = (api.d1_biased_downwind(KK * api.d1_biased_upwind(e, 0), 0)
               + api.d1_biased_downwind(api.d1_biased_upwind(e, 1), 1) - 0.5 * e)
        return p, {"p": p, "K": K, "f": f}, api.Eq(F, rhs), False
    if which == "funcs2d":
        mesh = cm.mesh_uniform([n + 1, n + 1])
        mk = lambda v: cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC), (capi.BC_NEUM, capi.BC_NEUM)],
                                     [(v, v), (0.0, 0.0)], ext=1)
        p = orc.HostField(mesh, mk(0.5))
        fields = {"p": p}
        for key, v in (("K", 1.0), ("g", 0.0), ("f", 0.0)):
            h = orc.HostField(mesh, mk(v))
            h.data[h.slices(cm.readable(h.info))] = arr[key + "__data"].reshape(h.data[h.slices(cm.readable(h.info))].shape)
            fields[key] = h
        e, KK, G, F = cm.Leaf("p"), cm.Leaf("K"), cm.Leaf("g"), cm.Leaf("f")
        k0, k1 = api.d1IntpCenterToCorner(KK, 0), api.d1IntpCenterToCorner(KK, 1)
        rhs = (api.dx(api.max(k0, 1.25) * api.dx(e)) + api.dy(api.conditional(k1 > 1.5, api.sqrt(k1), k1) * api.dy(e))
               - (api.abs(G) + 0.5) * e)
        return p, fields, api.Eq(F, rhs), False
    raise KeyError(which)


ASM = sorted(f[:-4] for f in os.listdir(cm.GOLDEN) if f.startswith("asm_"))


def _by_offset(off, coef):
    return {tuple(int(v) for v in off[e]): coef[:, e] for e in range(off.shape[0])}


@pytest.mark.parametrize("name", ASM)
def test_assembly_oracle_bitexact(name):
    meta, arr = cm.golden(name)
    target, fmap, eq, pin = _assemble_case(name, arr, meta)
    nodes, leaves = api.serialize(eq.residual_expr())
    host = [fmap[lf.tag] for lf in leaves]
    unknown = [i for i, h in enumerate(host) if h is target][0]
    off, coef, rhs = orc.assemble(target, nodes, host, unknown, int(pin))
    st = cm.record(meta, "stencil")
    want_off = np.array(st["offsets"])
    want = _by_offset(want_off, arr["stencil__coef"])
    got = _by_offset(off, coef)
    assert set(want) == set(got)
    for k in want:
        assert np.array_equal(got[k], want[k]), (k, np.abs(got[k] - want[k]).max())
    assert np.array_equal(rhs, arr["stencil__rhs"])


def test_assembly_matches_csr_generator_test_literals():
    """Known answers of the reference's CSRMatrixGeneratorTest.cpp (rows pinned by that generator are
    its last rows; the HYPRE path pins the first, so only the unpinned rows are compared there)."""
    gold = json.load(open(os.path.join(cm.GOLDEN, "csr_generator_test.json")))
    for bc_name, bc in (("dirc", capi.BC_DIRC), ("neum", capi.BC_NEUM), ("periodic", capi.BC_PERIODIC)):
        g = gold[bc_name]
        mesh = cm.mesh_uniform([5, 5], [(0.0, 4.0), (0.0, 4.0)])
        p = orc.HostField(mesh, cm.field_desc(2, capi.CENTER, [(bc, bc)] * 2, ext=1))
        e = cm.Leaf("p")
        nodes, _ = api.serialize(api.Eq(1.0, api.d2x(e) + api.d2y(e)).residual_expr())
        off, coef, rhs = orc.assemble(p, nodes, [p], 0, 0)
        # dense rows from the stencil (periodic offsets wrap on the 4x4 grid)
        A = np.zeros((16, 16))
        for c in range(16):
            i, j = c % 4, c // 4
            for k in range(off.shape[0]):
                ii, jj = (i + off[k][0]) % 4, (j + off[k][1]) % 4
                if bc != capi.BC_PERIODIC and not (0 <= i + off[k][0] < 4 and 0 <= j + off[k][1] < 4):
                    continue
                A[c, jj * 4 + ii] += coef[c, k]
        G = np.zeros((16, 16))
        ptr, col, val = g["ptr"], g["col"], g["val"]
        for r in range(16):
            for q in range(ptr[r], ptr[r + 1]):
                G[r, col[q]] = val[q]
        rows = range(15) if g["pin_last_row"] else range(16)
        for r in rows:
            assert np.array_equal(A[r], G[r]), (bc_name, r, A[r], G[r])
            assert rhs[r] == g["rhs"][r]


def test_reference_raw_binary_files_hold_the_dumped_fields():
    """The .cart files the reference's RawBinaryOStream wrote (rawbinary_ref fixture) parse with the
    independent reader and hold the fields' local-range values, with the stream's time stamps and file
    counter."""
    meta, arr = cm.golden("rawbinary_ref")
    assert meta["files"] == ["c_0.cart", "c_2.cart", "v_1.cart"]
    for f, name, t in (("c_0", "c", 0.25), ("v_1", "v", 0.25), ("c_2", "c", 1.5)):
        rec = cm.parse_cart(raw=arr["file__" + f].tobytes())
        fm = cm.record(meta, name)
        assert rec["name"] == name and rec["dim"] == 2 and rec["nproc"] == 1 and rec["time"] == t
        assert [list(r) for r in rec["local"]] == fm["local"] and [list(r) for r in rec["accessible"]] == fm["accessible"]
        rd = fm["readable"]
        full = arr[name + "__data"].reshape(rd[1][1] - rd[1][0], rd[0][1] - rd[0][0])
        lo = fm["local"]
        want = full[lo[1][0] - rd[1][0]:lo[1][1] - rd[1][0], lo[0][0] - rd[0][0]:lo[0][1] - rd[0][0]].reshape(-1)
        assert np.array_equal(rec["values"], want)

"""Shared helpers for the tests: meshes, field descriptions, expressions and golden fixtures."""
import ctypes as C
import json
import os
import struct

import numpy as np

import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    return meta, {k: z[k] for k in z.files if k != "meta"}


def record(meta, key):
    for r in meta["records"]:
        if r["key"] == key:
            return r["meta"]
    raise KeyError(key)


def mesh_uniform(dims, ranges=None, pad=5):
    """CartesianMesh built by the oracle's restatement of MeshBuilder::set1DMesh (no GPU, no library)."""
    xs, dxs = [], []
    for k, n in enumerate(dims):
        lo, hi = (ranges[k] if ranges else (0.0, 1.0))
        x = np.zeros(n + 2 * pad)
        dx = np.zeros(n + 2 * pad - 1)
        orc.lib().or_mesh_uniform(n, 0, pad, lo, hi, orc.dptr(x), orc.dptr(dx))
        xs.append(x)
        dxs.append(dx)
    return api.CartesianMesh(len(dims), dims, [0] * len(dims), pad, xs, dxs)


def mesh_points(points, pad=5):
    """CartesianMesh from per-dim node positions (MeshBuilder::setMeshOfDim(k, f) restated by the oracle)."""
    xs, dxs = [], []
    for p in points:
        p = np.ascontiguousarray(p, dtype=np.float64)
        n = len(p)
        x = np.zeros(n + 2 * pad)
        dx = np.zeros(n + 2 * pad - 1)
        orc.lib().or_mesh_points(n, 0, pad, orc.dptr(p), orc.dptr(x), orc.dptr(dx))
        xs.append(x)
        dxs.append(dx)
    return api.CartesianMesh(len(points), [len(p) for p in points], [0] * len(points), pad, xs, dxs)


def stretched_points(n, scale=1.0):
    """Node positions t + 0.25*t*(1 - t), t = i/(n - 1), times scale: the nonuniform mesh of the
    reference driver's operator cases, evaluated in the same IEEE operation order."""
    out = np.empty(n)
    for i in range(n):
        t = float(i) / float(n - 1)
        out[i] = (t + 0.25 * t * (1.0 - t)) * scale
    return out


def field_desc(ndim, loc, bcs, values=None, ext=0, padding=0):
    """bcs: list per dim of (lo, hi) BC types; values likewise (default 0)."""
    fd = capi.FieldDesc()
    fd.ndim = ndim
    for d in range(ndim):
        fd.loc[d] = loc[d] if isinstance(loc, (list, tuple)) else loc
        for s in range(2):
            fd.bc_type[d][s] = bcs[d][s]
            fd.bc_value[d][s] = values[d][s] if values else 0.0
            e = ext[d][s] if isinstance(ext, (list, tuple)) else ext
            fd.ext[d][s] = e
    fd.padding = padding
    return fd


class Leaf(api.Expr):
    """Expression leaf standing for a field slot (oracle-side)."""
    _is_field = True

    def __init__(self, tag):
        self.tag = tag


def ftcs_expr(u, s, ndim):
    t = api.d2x(u) + api.d2y(u) if ndim >= 2 else api.d2x(u)
    if ndim == 3:
        t = t + api.d2z(u)
    return u + s * t


def weno_stage_exprs(u, u1, u2, dt, upwind=False):
    L = api.d1_weno53_upwind if upwind else api.d1_weno53_downwind
    e1 = u - dt * L(u, 0)
    e2 = 0.75 * u + 0.25 * (u1 - dt * L(u1, 0))
    e3 = 1.0 / 3.0 * u + 2.0 / 3.0 * (u2 - dt * L(u2, 0))
    return e1, e2, e3


def readable(info):
    return [(max(info.local[d][0] - info.padding, info.logical[d][0]), min(info.local[d][1] + info.padding, info.logical[d][1]))
            for d in range(info.ndim)]


def seeded_interior(hf, seed, n_line):
    """u01(seed, j*n + i) on the assignable range (the reference driver's initialisation)."""
    rng = hf.assignable()
    if hf.info.ndim == 2:
        j, i = np.meshgrid(np.arange(*rng[1]), np.arange(*rng[0]), indexing="ij")
        hf.data[hf.slices(rng)] = orc.u01(seed, (j.astype(np.uint64) * np.uint64(n_line) + i.astype(np.uint64)))
    else:
        raise NotImplementedError


def problem_system(p, f, pin=False):
    """The oracle's assembly of a problem-form system (api.Problem: alpha*u - beta*Lap(u) = f, the
    equation `alpha*e - beta*(d2x(e) + d2y(e) [+ d2z(e)]) == f` on its own mesh) with f over the
    unknowns (x fastest): (dims, offsets, coef, rhs).  pin: the reference's pinned form (pinValue) of
    a singular system."""
    nd = len(p.n)
    nodes_per_dim = [n + 1 if p.loc == capi.CENTER else n for n in p.n]
    mesh = mesh_uniform(nodes_per_dim, [(0.0, p.h[d] * (nodes_per_dim[d] - 1)) for d in range(nd)])
    ext = 1 if (p.loc == capi.CENTER or p.bc == capi.BC_NEUM) else 0
    fd = field_desc(nd, p.loc, [(p.bc, p.bc)] * nd, ext=ext)
    u, F = orc.HostField(mesh, fd), orc.HostField(mesh, fd)
    rng = F.assignable()
    F.data[F.slices(rng)] = np.asarray(f, dtype=np.float64).reshape(F.data[F.slices(rng)].shape)
    F.update_padding()
    L = [Leaf("u"), Leaf("f")]
    lap = api.d2x(L[0]) + api.d2y(L[0]) if nd >= 2 else api.d2x(L[0])
    if nd == 3:
        lap = lap + api.d2z(L[0])
    eq = api.Eq(float(p.alpha) * L[0] - float(p.beta) * lap, L[1])
    nodes, _ = api.serialize(eq.residual_expr(), L)
    off, coef, rhs = orc.assemble(u, nodes, [u, F], 0, int(pin))
    return [r[1] - r[0] for r in rng], off, coef, rhs


def problem_residual(p, f, x):
    """||b - A x||_2 / ||b||_2 of a problem-form system (see problem_system) assembled by the oracle,
    with f and x over the unknowns (x fastest).  A pure Neumann Poisson problem is the singular
    consistent system (no pinned row), so a solution shifted by a constant has the same residual."""
    dims, off, coef, rhs = problem_system(p, f)
    r, bn = orc.residual(dims, [0] * len(dims), off, coef, rhs, np.asarray(x, dtype=np.float64).reshape(-1))
    return r / bn if bn > 0 else r


def parse_cart(path=None, raw=None):
    """The layout RawBinaryOStream::operator<< writes (RawBinaryStream.hpp:97-150), read from a file or
    from its bytes."""
    raw = open(path, "rb").read() if raw is None else raw
    pos = 0

    def take(fmt):
        nonlocal pos
        v = struct.unpack_from("<" + fmt, raw, pos)
        pos += struct.calcsize("<" + fmt)
        return v

    (nlen,) = take("i")
    name = raw[pos:pos + nlen].decode()
    pos += nlen
    dim, nproc = take("ii")
    (time,) = take("d")
    mesh_range = [take("ii") for _ in range(dim)]
    coords = [np.array(take("%dd" % (e - s))) for s, e in mesh_range]
    acc = [take("ii") for _ in range(dim)]
    loc = [take("ii") for _ in range(dim)]
    n = int(np.prod([e - s for s, e in loc]))
    vals = np.array(take("%dd" % n))
    assert pos == len(raw)
    return dict(name=name, dim=dim, nproc=nproc, time=time, mesh_range=mesh_range, coords=coords, accessible=acc, local=loc,
                values=vals)

"""ctypes wrapper of the CPU oracle (oracle/oracle.c, built into oracle/_build/liboracle.so).

Test infrastructure: the checker the GPU results are compared against.  It takes the same mesh /
field / expression descriptions as the C ABI (the ctypes structs of opflow_gb300._capi).
"""
import ctypes as C
import os
import subprocess

import numpy as np

from opflow_gb300 import _capi as capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SO = os.path.join(ROOT, "oracle", "_build", "liboracle.so")
_lib = None


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(ROOT, "oracle", "oracle.c")
        if not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(src):
            subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
        L = C.CDLL(SO)
        P = C.POINTER
        L.or_mesh_uniform.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, P(C.c_double), P(C.c_double)]
        L.or_mesh_points.argtypes = [C.c_int, C.c_int, C.c_int, P(C.c_double), P(C.c_double), P(C.c_double)]
        L.or_field_info.argtypes = [P(capi.MeshDesc), P(capi.FieldDesc), P(capi.FieldInfo)]
        L.or_update_padding.argtypes = [P(capi.MeshDesc), P(capi.FieldDesc), P(C.c_double)]
        L.or_assign.argtypes = [P(capi.MeshDesc), P(capi.FieldDesc), P(P(C.c_double)), C.c_int, C.c_int, C.c_int,
                                P(capi.Node), C.c_int]
        L.or_assemble.argtypes = [P(capi.MeshDesc), P(capi.FieldDesc), P(P(C.c_double)), C.c_int, C.c_int, P(capi.Node),
                                  C.c_int, C.c_int, P(C.c_int), P(C.c_int), P(C.c_double), P(C.c_double), P(C.c_size_t)]
        L.or_pcg.argtypes = [C.c_int, P(C.c_int), P(C.c_int), C.c_int, P(C.c_int), P(C.c_double), P(C.c_double),
                             P(C.c_double), C.c_double, C.c_int, P(C.c_int), P(C.c_double)]
        L.or_residual.argtypes = [C.c_int, P(C.c_int), P(C.c_int), C.c_int, P(C.c_int), P(C.c_double), P(C.c_double),
                                  P(C.c_double), P(C.c_double)]
        L.or_residual.restype = C.c_double
        L.or_u01.argtypes = [C.c_uint64, C.c_uint64]
        L.or_u01.restype = C.c_double
        L.or_last_error.restype = C.c_char_p
        L.or_set_threads.argtypes = [C.c_int]
        L.or_set_threads.restype = C.c_int
        _lib = L
    return _lib


def _chk(rc):
    if rc != 0:
        raise RuntimeError("oracle error %d: %s" % (rc, lib().or_last_error().decode()))


def dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def field_info(mesh, desc):
    info = capi.FieldInfo()
    md = mesh.desc()
    _chk(lib().or_field_info(C.byref(md), C.byref(desc), C.byref(info)))
    return info


def shape_of(info):
    return tuple(info.data_dims[d] for d in reversed(range(info.ndim)))


class HostField:
    """A field for the oracle: description + host data array (PlainTensor layout)."""

    def __init__(self, mesh, desc, data=None):
        self.mesh, self.desc = mesh, desc
        self.info = field_info(mesh, desc)
        self.data = np.zeros(shape_of(self.info)) if data is None else np.array(data, dtype=np.float64).reshape(shape_of(self.info))
        if data is None:
            self.update_padding()

    def update_padding(self):
        md = self.mesh.desc()
        _chk(lib().or_update_padding(C.byref(md), C.byref(self.desc), dptr(self.data)))

    def slices(self, ranges):
        sl = []
        for d in reversed(range(self.info.ndim)):
            lo, hi = ranges[d]
            o = self.info.data_offset[d]
            sl.append(slice(lo - o, hi - o))
        return tuple(sl)

    def assignable(self):
        return [(max(self.info.assignable[d][0], self.info.local[d][0]), min(self.info.assignable[d][1], self.info.local[d][1]))
                for d in range(self.info.ndim)]


def _pack(fields):
    n = len(fields)
    descs = (capi.FieldDesc * n)(*[f.desc for f in fields])
    ptrs = (C.POINTER(C.c_double) * n)(*[dptr(f.data) for f in fields])
    return descs, ptrs


def assign(dst, nodes, leaves, op=capi.ASSIGN_EQ):
    """or_assign: `dst <op>= expr` with FieldAssigner semantics; `leaves` are HostFields by slot."""
    fields = list(leaves)
    if not any(f is dst for f in fields):
        fields.append(dst)
    slot = [i for i, f in enumerate(fields) if f is dst][0]
    descs, ptrs = _pack(fields)
    md = dst.mesh.desc()
    _chk(lib().or_assign(C.byref(md), descs, ptrs, len(fields), slot, op, nodes, len(nodes)))


def assemble(target, nodes, leaves, unknown_slot, pin):
    """or_assemble: StencilField/StencilPad assembly -> (offsets[n_ent, D], coef[cells, n_ent], rhs[cells])."""
    descs, ptrs = _pack(leaves)
    md = target.mesh.desc()
    ne = C.c_int(0)
    nc = C.c_size_t(0)
    _chk(lib().or_assemble(C.byref(md), descs, ptrs, len(leaves), unknown_slot, nodes, len(nodes), pin, C.byref(ne), None, None,
                           None, C.byref(nc)))
    D = target.info.ndim
    off = np.zeros(ne.value * D, dtype=np.int32)
    coef = np.zeros(nc.value * ne.value)
    rhs = np.zeros(nc.value)
    _chk(lib().or_assemble(C.byref(md), descs, ptrs, len(leaves), unknown_slot, nodes, len(nodes), pin, C.byref(ne),
                           off.ctypes.data_as(C.POINTER(C.c_int)), dptr(coef), dptr(rhs), C.byref(nc)))
    return off.reshape(ne.value, D), coef.reshape(nc.value, ne.value), rhs


def pcg(dims, periodic, offsets, coef, rhs, x0=None, tol=1e-12, maxit=100000):
    D = len(dims)
    d3 = (C.c_int * 3)(*(list(dims) + [1] * (3 - D)))
    per = (C.c_int * 3)(*(list(periodic) + [0] * (3 - D)))
    off = np.ascontiguousarray(offsets, dtype=np.int32).reshape(-1)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    rhs = np.ascontiguousarray(rhs, dtype=np.float64)
    x = np.zeros(rhs.size) if x0 is None else np.array(x0, dtype=np.float64).reshape(-1)
    it = C.c_int(0)
    rr = C.c_double(0)
    _chk(lib().or_pcg(D, d3, per, offsets.shape[0], off.ctypes.data_as(C.POINTER(C.c_int)), dptr(coef), dptr(rhs), dptr(x),
                      tol, maxit, C.byref(it), C.byref(rr)))
    return x, it.value, rr.value


def residual(dims, periodic, offsets, coef, rhs, x):
    D = len(dims)
    d3 = (C.c_int * 3)(*(list(dims) + [1] * (3 - D)))
    per = (C.c_int * 3)(*(list(periodic) + [0] * (3 - D)))
    off = np.ascontiguousarray(offsets, dtype=np.int32).reshape(-1)
    bn = C.c_double(0)
    r = lib().or_residual(D, d3, per, offsets.shape[0], off.ctypes.data_as(C.POINTER(C.c_int)), dptr(np.ascontiguousarray(coef)),
                          dptr(np.ascontiguousarray(rhs)), dptr(np.ascontiguousarray(x, dtype=np.float64)), C.byref(bn))
    return r, bn.value


# ---- seeded inputs (counter-based splitmix64, same as oracle.c / the reference driver) ----
def u01(seed, k):
    k = np.asarray(k, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + (k + np.uint64(1)) * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def pfmg_pcg(dims, offsets, coef, rhs, tol=1e-10, maxit=200, cycles=1, threads=1):
    """or_pfmg_pcg: the restated HYPRE PCG + PFMG solve of an assembled system (x0 = 0, two-norm test).
    cycles: PFMG V-cycles per preconditioner application (0: PFMG's defaults); threads: host threads
    sharing each loop.  Returns (x, iterations, final relative residual, levels).  Reentrant:
    independent solves may also run on several host threads at once (ctypes releases the GIL)."""
    D = len(dims)
    d3 = (C.c_int * 3)(*(list(dims) + [1] * (3 - D)))
    off = np.ascontiguousarray(offsets, dtype=np.int32).reshape(-1)
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    rhs = np.ascontiguousarray(rhs, dtype=np.float64)
    x = np.zeros(rhs.size)
    it, rr, nl = C.c_int(0), C.c_double(0), C.c_int(0)
    _chk(lib().or_pfmg_pcg(D, d3, offsets.shape[0], off.ctypes.data_as(C.POINTER(C.c_int)), dptr(coef), dptr(rhs), dptr(x),
                           C.c_double(tol), maxit, cycles, threads, C.byref(it), C.byref(rr), C.byref(nl)))
    return x, it.value, rr.value, nl.value

"""Replays a recording of an OpFlow example compiled unchanged against the adapter
(tests/golden/adapter_*.json.gz, made by tests/golden/make_adapter_golden.py): the fields the example
created and the node programs the adapter lowered from OpFlow's expression types, in order.

`replay_gpu` runs them through libopflow_gpu's C ABI (opflow_field_create / _upload / opflow_assign,
the calls the adapter makes); `replay_oracle` runs them through the oracle.  Both return the final
data arrays of the fields (the PlainTensor layout of the padded local range)."""
import ctypes as C
import gzip
import json
import os

import numpy as np

import oracle_lib as orc
from opflow_gb300 import _capi as capi

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with gzip.open(os.path.join(GOLDEN, "adapter_%s.json.gz" % name), "rt") as f:
        return json.load(f)


def _descs(rec):
    """(mesh desc, field desc, keep-alive arrays) of a recorded field."""
    md = capi.MeshDesc()
    md.ndim = rec["ndim"]
    md.pad_width = rec["pad_width"]
    keep = []
    for d in range(rec["ndim"]):
        md.dims[d] = rec["dims"][d]
        md.start[d] = rec["start"][d]
        x = np.ascontiguousarray(rec["x%d" % d], dtype=np.float64)
        dx = np.ascontiguousarray(rec["dx%d" % d], dtype=np.float64)
        keep += [x, dx]
        md.x[d] = x.ctypes.data_as(C.POINTER(C.c_double))
        md.dx[d] = dx.ctypes.data_as(C.POINTER(C.c_double))
    fd = capi.FieldDesc()
    fd.ndim = rec["ndim"]
    fd.padding = rec["padding"]
    for d in range(rec["ndim"]):
        fd.loc[d] = rec["loc"][d]
        for s in range(2):
            fd.bc_type[d][s] = rec["bc_type"][d][s]
            fd.bc_value[d][s] = rec["bc_value"][d][s]
            fd.ext[d][s] = rec["ext"][d][s]
    return md, fd, keep


def _nodes(ev):
    arr = (capi.Node * len(ev["nodes"]))()
    for k, (kind, a, b, dim, field, value, c) in enumerate(ev["nodes"]):
        arr[k].kind, arr[k].a, arr[k].b, arr[k].dim, arr[k].field, arr[k].value, arr[k].c = kind, a, b, dim, field, value, c
    return arr


def replay_gpu(rec, ctx, states=None):
    """`states` (a list) receives the opflow_solve_state of every recorded solve."""
    L = capi.lib()
    fields, info, keep, solvers = {}, {}, [], {}
    states = [] if states is None else states
    for fr in rec["fields"]:
        md, fd, k = _descs(fr)
        keep += k
        h = C.c_void_p()
        capi.check(L.opflow_field_create(ctx.handle, C.byref(md), C.byref(fd), C.byref(h)))
        inf = capi.FieldInfo()
        capi.check(L.opflow_field_get_info(h, C.byref(inf)))
        fields[fr["id"]], info[fr["id"]] = h, inf
    for ev in rec["events"]:
        if ev["ev"] == "upload":
            h, inf = fields[ev["id"]], info[ev["id"]]
            if ev["data"] is not None:
                a = np.ascontiguousarray(ev["data"], dtype=np.float64)
            else:
                # a large field's first state: the zero field with its padding applied (what
                # opflow_field_create leaves), which the recorder checked the uploaded data to be
                assert ev.get("zero_padded"), "a recorded upload that the replay cannot rebuild"
                continue
            capi.check(L.opflow_field_upload(h, a.ctypes.data_as(C.POINTER(C.c_double)), a.size))
        elif ev["ev"] == "solver":
            # makeEqnSolveHandler: the engine's solver over the recorded equation
            sp = capi.SolveParams()
            L.opflow_solve_params_default(C.byref(sp))
            for k, v in ev["params"].items():
                setattr(sp, k, v)
            nodes = _nodes(ev)
            leaves = (C.c_void_p * len(ev["leaves"]))(*[fields[i].value for i in ev["leaves"]])
            h = C.c_void_p()
            capi.check(L.opflow_solver_create(ctx.handle, fields[ev["target"]], nodes, len(ev["nodes"]), leaves, len(ev["leaves"]),
                                              ev["unknown"], C.byref(sp), C.byref(h)))
            keep.append((nodes, leaves))
            solvers.setdefault(ev["target"], []).append(h)
        elif ev["ev"] == "solve":
            st = capi.SolveState()
            capi.check(L.opflow_solver_solve(solvers[ev["target"]][-1], C.byref(st)))
            states.append(st)
        else:
            nodes = _nodes(ev)
            leaves = (C.c_void_p * max(1, len(ev["leaves"])))(*[fields[i].value for i in ev["leaves"]])
            for _ in range(ev["repeat"]):
                capi.check(L.opflow_assign(ctx.handle, fields[ev["dst"]], ev["arith"], nodes, len(ev["nodes"]), leaves, len(ev["leaves"]),
                                           ev["mode"]))
    for hs in solvers.values():
        for h in hs:
            L.opflow_solver_destroy(h)
    out = {}
    for fid, h in fields.items():
        a = np.zeros(info[fid].count)
        capi.check(L.opflow_field_download(h, a.ctypes.data_as(C.POINTER(C.c_double)), a.size))
        out[fid] = (a, info[fid])
        L.opflow_field_destroy(h)
    return out


def replay_oracle(rec):
    fields, descs, keep = {}, {}, []
    for fr in rec["fields"]:
        md, fd, k = _descs(fr)
        keep += k
        inf = capi.FieldInfo()
        orc._chk(orc.lib().or_field_info(C.byref(md), C.byref(fd), C.byref(inf)))
        a = np.zeros(inf.count)
        orc._chk(orc.lib().or_update_padding(C.byref(md), C.byref(fd), orc.dptr(a)))
        fields[fr["id"]] = a
        descs[fr["id"]] = (md, fd, inf)
    for ev in rec["events"]:
        if ev["ev"] in ("solver", "solve"):
            raise NotImplementedError("the oracle replay covers assignments (solves are replayed on the GPU)")
        if ev["ev"] == "upload":
            if ev["data"] is not None:
                fields[ev["id"]][:] = ev["data"]
            else:
                assert ev.get("zero_padded")
            continue
        ids = list(ev["leaves"])
        if ev["dst"] not in ids:
            ids.append(ev["dst"])
        fdarr = (capi.FieldDesc * len(ids))(*[descs[i][1] for i in ids])
        ptrs = (C.POINTER(C.c_double) * len(ids))(*[orc.dptr(fields[i]) for i in ids])
        nodes = _nodes(ev)
        md = descs[ev["dst"]][0]
        for _ in range(ev["repeat"]):
            orc._chk(orc.lib().or_assign(C.byref(md), fdarr, ptrs, len(ids), ids.index(ev["dst"]), ev["arith"], nodes, len(ev["nodes"])))
    return {fid: (a, descs[fid][2]) for fid, a in fields.items()}


def local_values(a, inf):
    """The local range of a field's data array (what RawBinaryOStream writes), x fastest."""
    D = inf.ndim
    dims = [inf.data_dims[d] for d in range(D)]
    arr = a.reshape(list(reversed(dims)))
    sl = tuple(slice(inf.local[d][0] - inf.data_offset[d], inf.local[d][1] - inf.data_offset[d]) for d in reversed(range(D)))
    return arr[sl].reshape(-1)

"""Many explicit assignments in one launch (opflow_assign_batch): uneven 2D and 3D grids, cell- and
node-centred fields with Dirichlet, Neumann and periodic boundaries, self-reading updates (FTCS), a
plain combination of other fields and a compound assignment, over several steps; every field equals
its own assignment run alone in exact mode, bit for bit, and the batch's misuse is refused."""
import numpy as np
import pytest

import common as cm
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

pytestmark = pytest.mark.gpu


def _field(ctx, dims, loc, bc, seed, ext=0):
    D = len(dims)
    mesh = cm.mesh_uniform(list(dims))
    fd = cm.field_desc(D, loc, [(bc, bc)] * D, ext=ext)
    f = api.CartesianField(mesh, fd, ctx)
    a = f.download()
    a[...] = 0.0
    sl = f.index_slices([tuple(f.info.assignable[d]) for d in range(D)])
    a[sl] = np.random.default_rng(seed).random(a[sl].shape)
    f.upload(a)
    return f


def _cases(ctx):
    """(dst, expression builder over the case's fields, op) for a set of uneven grids"""
    out = []
    for k, (dims, loc, bc, ext) in enumerate([((65, 65), capi.CORNER, capi.BC_DIRC, 0), ((129, 77), capi.CORNER, capi.BC_DIRC, 0),
                                              ((31, 40, 23), capi.CORNER, capi.BC_DIRC, 0), ((50, 37), capi.CENTER, capi.BC_NEUM, 1),
                                              ((24, 18, 30), capi.CENTER, capi.BC_PERIODIC, 1)]):
        u = _field(ctx, dims, loc, bc, 100 + k, ext)
        hx = 1.0 / (dims[0] - 1)
        out.append((u, lambda u=u, s=0.1 * hx * hx, D=len(dims): cm.ftcs_expr(u, s, D), "="))
    a = _field(ctx, (90, 70), capi.CORNER, capi.BC_DIRC, 7)
    b = _field(ctx, (90, 70), capi.CORNER, capi.BC_DIRC, 8)
    c = _field(ctx, (90, 70), capi.CORNER, capi.BC_DIRC, 9)
    out.append((c, lambda a=a, b=b: 2.0 * a - b * b + api.d2x(a), "="))
    d = _field(ctx, (90, 70), capi.CORNER, capi.BC_DIRC, 10)
    out.append((d, lambda a=a: 0.5 * api.d2y(a), "+"))
    return out


@pytest.mark.parametrize("steps", [1, 4])
def test_batch_equals_each_assignment_alone(ctx, steps):
    alone = _cases(ctx)
    for dst, expr, op in alone:
        dst.assign(expr(), op, mode="exact", steps=steps)
    want = [dst.download() for dst, _, _ in alone]
    batch = _cases(ctx)
    api.assign_batch([(dst, expr(), op) for dst, expr, op in batch], steps=steps)
    for k, (dst, _, _) in enumerate(batch):
        assert np.array_equal(dst.download(), want[k]), k


def test_batch_misuse_is_refused(ctx):
    u = _field(ctx, (33, 33), capi.CORNER, capi.BC_DIRC, 1)
    v = _field(ctx, (33, 33), capi.CORNER, capi.BC_DIRC, 2)
    with pytest.raises(capi.OpflowError) as e:
        api.assign_batch([(u, 2.0 * v), (u, v + 1.0)])
    assert e.value.code == capi.E_INVALID and "same field" in str(e.value)
    with pytest.raises(capi.OpflowError) as e:
        api.assign_batch([(u, 2.0 * v), (v, u + 1.0)])
    assert e.value.code == capi.E_INVALID and "reads the destination" in str(e.value)

"""C ABI host-side checks that need no GPU: the library loads, exports every symbol the header
declares, and its host logic (mesh generation, field ranges) equals the oracle's."""
import ctypes as C

import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    syms = capi.declared_symbols()
    assert len(syms) >= 30
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    assert L.opflow_abi_version() == 3


@pytest.mark.parametrize("n,lo,hi,pad", [(1025, 0.0, 1.0, 5), (512, 0.0, 1.0, 5), (20, -1.0, 3.0, 3), (2049, 0.0, 1.0, 5)])
def test_mesh_uniform_matches_oracle(n, lo, hi, pad):
    x1, dx1 = np.zeros(n + 2 * pad), np.zeros(n + 2 * pad - 1)
    x2, dx2 = np.zeros(n + 2 * pad), np.zeros(n + 2 * pad - 1)
    capi.check(capi.lib().opflow_mesh_uniform(n, 0, pad, lo, hi, orc.dptr(x1), orc.dptr(dx1)))
    orc.lib().or_mesh_uniform(n, 0, pad, lo, hi, orc.dptr(x2), orc.dptr(dx2))
    assert np.array_equal(x1, x2) and np.array_equal(dx1, dx2)


def test_describe_rejects_bad_fields():
    mesh = cm.mesh_uniform([9, 9])
    with pytest.raises(capi.OpflowError) as e:
        api.describe(mesh, cm.field_desc(2, capi.CENTER, [(capi.BC_PERIODIC, capi.BC_DIRC)] * 2))
    assert e.value.code == capi.E_INVALID
    with pytest.raises(capi.OpflowError) as e:
        api.describe(mesh, cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, ext=6))
    assert e.value.code == capi.E_INVALID


def test_describe_matches_oracle_on_many_fields():
    mesh = cm.mesh_uniform([13, 10, 7])
    kinds = [capi.BC_DIRC, capi.BC_NEUM, capi.BC_SYMM, capi.BC_ASYMM, capi.BC_UNDEFINED]
    rng = np.random.default_rng(0)
    for _ in range(200):
        loc = [int(v) for v in rng.integers(0, 2, 3)]
        bcs = []
        for d in range(3):
            if rng.random() < 0.2:
                bcs.append((capi.BC_PERIODIC, capi.BC_PERIODIC))
            else:
                bcs.append((kinds[rng.integers(0, 5)], kinds[rng.integers(0, 5)]))
        ext = [[int(rng.integers(0, 4)), int(rng.integers(0, 4))] for _ in range(3)]
        fd = cm.field_desc(3, loc, bcs, ext=ext, padding=int(rng.integers(0, 3)))
        a = api.describe(mesh, fd)
        b = orc.field_info(mesh, fd)
        for key in ("logical", "accessible", "assignable", "local"):
            assert [list(getattr(a, key)[d]) for d in range(3)] == [list(getattr(b, key)[d]) for d in range(3)]
        assert list(a.data_dims) == list(b.data_dims) and list(a.data_offset) == list(b.data_offset) and a.count == b.count


def test_serialize_keeps_operand_order_and_shares_leaves():
    u, v = cm.Leaf("u"), cm.Leaf("v")
    nodes, leaves = api.serialize(2.0 - u / v + api.d2x(u))
    kinds = [nodes[i].kind for i in range(len(nodes))]
    assert kinds[-1] == capi.NODE_ADD
    assert len(leaves) == 2 and leaves[0] is u and leaves[1] is v
    sub = [nodes[i] for i in range(len(nodes)) if nodes[i].kind == capi.NODE_SUB][0]
    assert nodes[sub.a].kind == capi.NODE_CONST and nodes[sub.a].value == 2.0
    assert nodes[sub.b].kind == capi.NODE_DIV


def test_expression_functions_do_not_shadow_builtins():
    """api.max / api.abs / ... are expression builders, reachable as module attributes, while the
    module's own code keeps Python's builtins of the same names."""
    from opflow_gb300 import api
    for name in ("max", "min", "abs", "round", "pow"):
        assert name not in vars(api)
        assert callable(getattr(api, name))
    assert isinstance(api.max(api.ScalarExpr(1.0), 2.0), api.ExprNode)

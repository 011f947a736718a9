"""Host-side logic that needs no GPU: the synthetic workload generators (seeded, with the
configurations' shapes and distributions), the problem descriptors handed to the C ABI, and the
expression serialisation (children first, root last, one slot per distinct field)."""
import numpy as np

import common as cm
from opflow_gb300 import _capi as capi
from opflow_gb300 import api
from opflow_gb300 import workloads as wl


def test_batched_problems_are_seeded_and_follow_the_configuration():
    """512-problem batch configuration, first 24 problems: (I - k Lap) u = f on corner-node Dirichlet
    grids, k in [1e-4, 1], side 2^m + 1 within [65, 1025], f over the (n - 2)^2 inner nodes."""
    a = wl.batched_problems(api, 7, 24)
    b = wl.batched_problems(api, 7, 24)
    c = wl.batched_problems(api, 8, 24)
    assert len(a) == 24
    for (pa, fa), (pb, fb) in zip(a, b):
        assert pa.n == pb.n and pa.beta == pb.beta and np.array_equal(fa, fb)
    assert any(pa.n != pc.n or pa.beta != pc.beta for (pa, _), (pc, _) in zip(a, c))
    for p, f in a:
        n = p.n[0]
        assert p.n == [n, n] and n in (65, 129, 257, 513, 1025)
        assert p.alpha == 1.0 and 1e-4 <= p.beta <= 1.0
        assert p.loc == api.LocOnMesh.Corner and p.bc == api.BCType.Dirc
        assert p.h == [1.0 / (n - 1)] * 2
        assert f.shape == ((n - 2) * (n - 2),)


def test_problem_descriptor_carries_every_field():
    p = api.Problem([40, 33, 17], [0.25, 0.5, 0.125], alpha=0.5, beta=2.0, loc=api.LocOnMesh.Corner, bc=api.BCType.Neum)
    d = p.to_c()
    assert d.ndim == 3 and list(d.n[:3]) == [40, 33, 17] and list(d.h[:3]) == [0.25, 0.5, 0.125]
    assert d.alpha == 0.5 and d.beta == 2.0 and d.loc == int(api.LocOnMesh.Corner) and d.bc == int(api.BCType.Neum)


def test_rhs_is_projected_only_for_singular_operators():
    rng = np.random.default_rng(1)
    neum = wl.poisson_problem(api, 24, 2, api.BCType.Neum)
    dirc = wl.poisson_problem(api, 24, 2, api.BCType.Dirc)
    fn, fd = wl.rhs_for(rng, neum), wl.rhs_for(rng, dirc)
    assert fn.size == fd.size == 24 * 24
    assert abs(fn.mean()) < 1e-15
    assert abs(fd.mean()) > 1e-6


def test_smooth_coefficient_field_has_unit_spread():
    g = wl.smooth_field(np.random.default_rng(5), 16)
    assert g.shape == (16, 16, 16)
    assert abs(g.mean()) < 1e-12 and abs(g.std() - 1.0) < 1e-12


def test_weno_initial_lines_are_seeded_pulses():
    u = wl.weno_u0(3, 256, 8)
    assert u.shape == (8, 256)
    assert np.array_equal(u, wl.weno_u0(3, 256, 8))
    assert u.min() >= 0.0 and u.max() <= 1.8
    assert np.all((u > 0).sum(axis=1) > 0)  # every line holds its pulses


def test_ftcs_expression_serialises_children_first():
    """u + s * (d2x(u) + d2y(u)): one leaf slot for u, the constant and the operators after their
    operands, the root last."""
    u = cm.Leaf("u")
    arr, leaves = api.serialize(cm.ftcs_expr(u, 0.25, 2))
    assert len(leaves) == 1 and leaves[0] is u  # (== on expressions builds an equation)
    nodes = [(n.kind, n.a, n.b, n.dim, n.field, n.value, n.c) for n in arr]  # the C ABI's opflow_node array
    kinds = [n[0] for n in nodes]
    assert kinds.count(capi.NODE_FIELD) >= 1 and kinds.count(capi.NODE_CONST) == 1
    assert [n[5] for n in nodes if n[0] == capi.NODE_CONST] == [0.25]
    for i, n in enumerate(nodes):
        for child in (n[1], n[2], n[6]):
            assert child < i  # children precede their parent
        if n[0] == capi.NODE_FIELD:
            assert n[4] == 0  # the only leaf slot
    referenced = {c for n in nodes for c in (n[1], n[2], n[6]) if c >= 0}
    assert referenced == set(range(len(nodes) - 1))  # every node but the root is used once or more
    assert nodes[-1][0] not in (capi.NODE_FIELD, capi.NODE_CONST)

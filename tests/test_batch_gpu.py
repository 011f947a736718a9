"""Batched uneven solves: one launch per multigrid operation for the whole batch.  Every problem's
result must equal its single-problem solve bit for bit (deterministic per-problem reductions) and
reach the tolerance on the reference's system (checked with the oracle)."""
import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

pytestmark = pytest.mark.gpu


def problems(seed, count):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        m = int(rng.integers(4, 8))
        n = 2 ** m + 1
        k = float(10 ** rng.uniform(-4, 0))
        h = 1.0 / (n - 1)
        out.append(api.Problem([n, n], [h, h], alpha=1.0, beta=k, loc=api.LocOnMesh.Corner, bc=api.BCType.Dirc))
    # a cell-centred Neumann Helmholtz problem and a Dirichlet Poisson one in the mix
    out.append(api.Problem([48, 40], [1 / 48, 1 / 40], alpha=1.0, beta=0.5, loc=api.LocOnMesh.Center, bc=api.BCType.Neum))
    out.append(api.Problem([33, 33, 33], [1 / 32] * 3, alpha=0.0, beta=1.0, loc=api.LocOnMesh.Corner, bc=api.BCType.Dirc))
    return out


@pytest.mark.parametrize("prec", ["mixed", "fp64"])
def test_batch_alone_equals_mix_and_reaches_tolerance(ctx, prec):
    probs = problems(7, 10)
    params = api.StructSolverParams(tol=1e-10, maxIter=100, precision=prec, zeroGuess=True)
    B = api.Batch(probs, params, ctx)
    rng = np.random.default_rng(1)
    fs = []
    for i in range(len(probs)):
        f = rng.standard_normal(B.size(i))
        fs.append(f)
        B.set(i, f)
    st = B.solve()
    assert all(s.converged for s in st), [(s.niter, s.relerr) for s in st]
    for i in (0, 3, len(probs) - 2, len(probs) - 1):
        alone = api.Batch([probs[i]], params, ctx)
        alone.set(0, fs[i])
        s1 = alone.solve()[0]
        assert s1.niter == st[i].niter
        assert np.array_equal(alone.get(0), B.get(i)), i
    # independent check of problem 0 with the oracle: (I - k Lap) x = f on the interior nodes
    p = probs[0]
    n = p.n[0]
    mesh = cm.mesh_uniform([n, n])
    fd = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2)
    u, F = orc.HostField(mesh, fd), orc.HostField(mesh, fd)
    F.data[1:-1, 1:-1] = fs[0].reshape(n - 2, n - 2)
    L = [cm.Leaf("u"), cm.Leaf("f")]
    eq = api.Eq(1.0 * L[0] - p.beta * (api.d2x(L[0]) + api.d2y(L[0])), L[1])
    nodes, _ = api.serialize(eq.residual_expr(), L)
    off, coef, rhs = orc.assemble(u, nodes, [u, F], 0, 0)
    r, bn = orc.residual([n - 2, n - 2], [0, 0], off, coef, rhs, B.get(0))
    assert r / bn <= 1e-10

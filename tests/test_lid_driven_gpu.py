"""The reference's lid-driven cavity (examples/LidDriven/LidDriven2D.cpp) on the engine, end to end:
staggered velocities, Crank-Nicolson diffusion with semi-implicit convection, GMRES + PFMG momentum
solves (non-symmetric systems), a GMRES + PFMG pinned pressure-correction Poisson solve with a static
matrix, and the explicit updates between them, all written with the reference's operators.

Checks per time step:
  - every solve reaches the relative residual 1e-10 on the reference's own system, as assembled and
    evaluated by the oracle;
  - the projection keeps the discrete divergence dx(u) + dy(v) at the level the solver tolerance
    allows (it starts at zero).
"""
import numpy as np
import pytest

import common as cm
from opflow_gb300 import _capi as capi
from opflow_gb300 import api
from test_implicit_gpu import oracle_check

pytestmark = pytest.mark.gpu

Co, Cn = api.LocOnMesh.Corner, api.LocOnMesh.Center
D1C = api.D1FirstOrderCentered


def _fields(ctx, n):
    mesh = api.MeshBuilder().newMesh(n, n).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build()
    b = api.ExprBuilder().setMesh(mesh).setExt(1)
    for d in range(2):
        for pos in (api.DimPos.start, api.DimPos.end):
            b.setBC(d, pos, api.BCType.Dirc, 0.)
    u = b.setName("u").setBC(1, api.DimPos.end, api.BCType.Dirc, 1.).setLoc([Co, Cn]).build(ctx)
    du = b.setName("du").setBC(1, api.DimPos.end, api.BCType.Dirc, 0.).build(ctx)
    v = b.setName("v").setBC(1, api.DimPos.end, api.BCType.Dirc, 0.).setLoc([Cn, Co]).build(ctx)
    dv = b.setName("dv").build(ctx)
    for d in range(2):
        for pos in (api.DimPos.start, api.DimPos.end):
            b.setBC(d, pos, api.BCType.Neum, 0.)
    p = b.setName("p").setLoc([Cn, Cn]).build(ctx)
    dp = b.setName("dp").build(ctx)
    for f in (u, du, v, dv, p, dp):
        f.assign(0.)
    return u, du, v, dv, p, dp


def _ops():
    i2c0 = lambda e: api.d1IntpCornerToCenter(e, 0)
    i2c1 = lambda e: api.d1IntpCornerToCenter(e, 1)
    c2i0 = lambda e: api.d1IntpCenterToCorner(e, 0)
    c2i1 = lambda e: api.d1IntpCenterToCorner(e, 1)
    conv_xx = lambda a, b: api.dx(i2c0(a) * i2c0(b))
    conv_xy = lambda a, b: api.dy(c2i1(a) * c2i0(b))
    conv_yx = lambda a, b: api.dx(c2i1(a) * c2i0(b))
    conv_yy = lambda a, b: api.dy(i2c1(a) * i2c1(b))
    lap = lambda e: api.d2x(e) + api.d2y(e)
    return conv_xx, conv_xy, conv_yx, conv_yy, lap


def run_cavity(ctx, n, steps, check=True):
    """The cavity's time steps; with `check`, every solve is verified against the oracle and the
    divergence after each projection is bounded.  Returns the final u, v, p fields."""
    dt, nu = 0.5e-2, 1.0e-2
    u, du, v, dv, p, dp = _fields(ctx, n)
    conv_xx, conv_xy, conv_yx, conv_yy, lap = _ops()
    prm = dict(tol=1e-10, maxIter=100, solver="GMRES", precond="PFMG")

    def u_eq(e):
        return (e / dt + conv_xx(u, e) + 0.5 * conv_xy(e, v)
                == nu * lap(u) + 0.5 * nu * lap(e) - (conv_xx(u, u) + conv_xy(u, v)) - api.dx(p, D1C))

    def v_eq(e):
        return (e / dt + conv_yy(v, e) + conv_yy(v, v) + conv_yx(u, v) + 0.5 * conv_yx(u, e) + 0.5 * conv_yx(du, v)
                == nu * lap(v) + 0.5 * nu * lap(e) - api.dy(p, D1C))

    def p_eq(e):
        return lap(e) == (api.dx(du, D1C) + api.dy(dv, D1C)) / dt

    hu = api.makeEqnSolveHandler(u_eq, du, api.StructSolverParams(**prm))
    hv = api.makeEqnSolveHandler(v_eq, dv, api.StructSolverParams(**prm))
    hp = api.makeEqnSolveHandler(p_eq, dp, api.StructSolverParams(staticMat=True, pinValue=True, **prm))
    div = api.CartesianField(p.mesh, p.desc, ctx)
    for step in range(steps):
        for h, eq, tgt, pin in ((hu, u_eq, du, False), (hv, v_eq, dv, False)):
            st = h.solve()
            assert st.converged and st.relerr <= 1e-10, (step, st)
            if check:
                rel, _ = oracle_check(tgt, eq, tgt, pin, 1e-10)
                assert rel <= 2e-10, (step, rel)
        du.assign(du - 0.5 * dt * conv_xy(u, dv))
        u.assign(u + du)
        v.assign(v + dv)
        st = hp.solve()
        assert st.converged and st.relerr <= 1e-10, (step, st)
        if check:
            rel, _ = oracle_check(dp, p_eq, dp, True, 1e-10)
            assert rel <= 2e-10, (step, rel)
        u.assign(u - dt * api.dx(dp, D1C))
        v.assign(v - dt * api.dy(dp, D1C))
        p.assign(p + dp)
        if check:
            div.assign(api.dx(u, D1C) + api.dy(v, D1C))
            d = div.download()[div.index_slices([tuple(div.info.assignable[q]) for q in range(2)])]
            assert np.abs(d).max() <= 1e-6, (step, np.abs(d).max())
    return u, v, p


def test_lid_driven_cavity_steps(ctx):
    u, v, p = run_cavity(ctx, 33, 4)
    # the lid drags the fluid: the top row moves along +x, a return flow develops below
    U = u.download()[u.index_slices([tuple(u.info.assignable[q]) for q in range(2)])]
    assert U[-1].mean() > 0.05 and U.min() < 0

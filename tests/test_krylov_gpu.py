"""The outer iterations besides the fused flexible PCG (krylov.cu): restarted flexible GMRES (GMRES,
FGMRES, LGMRES), BiCGSTAB, PCG with Jacobi or no preconditioner, and the preconditioner iterated alone
(PFMG / SMG / Jacobi as the solver), with the multigrid V-cycle, Jacobi or no preconditioner.  Every
solve is checked on the reference's own system, assembled and evaluated by the oracle: the relative
residual ||b - A x||_2 / ||b||_2 must reach the requested tolerance (1e-10, checked at 2e-10)."""
import numpy as np
import pytest

import common as cm
from opflow_gb300 import _capi as capi
from opflow_gb300 import api
from test_implicit_gpu import oracle_check, poisson_case

pytestmark = pytest.mark.gpu

# (solver, precond, kDim, maxIter) of PrecondStructSolver<solver, precond>
SYMMETRIC = [
    ("GMRES", "PFMG", 5, 200), ("FGMRES", "PFMG", 5, 200), ("LGMRES", "SMG", 10, 200), ("BICGSTAB", "PFMG", 5, 200),
    ("PCG", "Jacobi", 5, 2000), ("PCG", "None", 5, 2000), ("GMRES", "Jacobi", 30, 4000), ("BICGSTAB", "None", 5, 4000),
    ("PFMG", "None", 5, 200),
]


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("solver,precond,kdim,maxit", SYMMETRIC)
@pytest.mark.parametrize("bc", [capi.BC_DIRC, capi.BC_NEUM])
def test_poisson_with_every_outer_iteration(ctx, solver, precond, kdim, maxit, bc, prec):
    if prec == "mixed" and "PFMG" not in (solver, precond) and "SMG" not in (solver, precond):
        pytest.skip("the precision switch only changes the V-cycle")
    n = 40
    mesh, fd, p, f = poisson_case(ctx, n, bc)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)
    pin = bc != capi.BC_DIRC
    params = api.StructSolverParams(tol=1e-10, maxIter=maxit, pinValue=pin, precision=prec, solver=solver, precond=precond,
                                    kDim=kdim, zeroGuess=True)
    st = api.Solve(getter, p, params)
    assert st.converged and st.relerr <= 1e-10, (solver, precond, st)
    rel, _ = oracle_check(p, getter, p, pin, 1e-10)
    assert rel <= 2e-10, rel
    if pin:
        assert p.download()[p.index_slices([(0, 1), (0, 1)])].item() == 0.0


def test_jacobi_iterated_alone_converges_on_a_small_grid(ctx):
    mesh, fd, p, f = poisson_case(ctx, 12, capi.BC_DIRC)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)
    params = api.StructSolverParams(tol=1e-10, maxIter=3000, solver="Jacobi", precond="None", zeroGuess=True)
    st = api.Solve(getter, p, params)
    assert st.converged, st
    rel, _ = oracle_check(p, getter, p, False, 1e-10)
    assert rel <= 2e-10


def _convection_case(ctx, n, seed=3):
    """Backward-Euler convection-diffusion with first-order upwind convection: a non-symmetric system
    e + dt*(cx*dx<Downwind>(e) + cy*dy<Downwind>(e) - nu*(d2x(e) + d2y(e))) == f, Dirichlet cells."""
    mesh = cm.mesh_uniform([n + 1, n + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, [(0.25, 0.25), (-0.5, 0.5)], ext=1)
    p = api.CartesianField(mesh, fd, ctx)
    f = api.CartesianField(mesh, fd, ctx)
    a = f.download()
    rng = np.random.default_rng(seed)
    sl = f.index_slices([tuple(f.info.assignable[d]) for d in range(2)])
    a[sl] = rng.standard_normal(a[sl].shape)
    f.upload(a)
    dt, cx, cy, nu = 0.05, 1.0, 0.6, 1e-3
    D = api.D1FirstOrderBiasedDownwind

    def getter(e):
        return f == e + dt * (cx * api.dx(e, D) + cy * api.dy(e, D) - nu * (api.d2x(e) + api.d2y(e)))
    return p, getter


NONSYMMETRIC = [("GMRES", "PFMG", 5, "fp64"), ("FGMRES", "PFMG", 10, "mixed"), ("LGMRES", "PFMG", 5, "fp64"),
                ("BICGSTAB", "PFMG", 5, "fp64"), ("BICGSTAB", "PFMG", 5, "mixed"), ("GMRES", "Jacobi", 20, "fp64"),
                ("BICGSTAB", "Jacobi", 5, "fp64")]


@pytest.mark.parametrize("solver,precond,kdim,prec", NONSYMMETRIC)
def test_nonsymmetric_convection_diffusion(ctx, solver, precond, kdim, prec):
    p, getter = _convection_case(ctx, 64)
    params = api.StructSolverParams(tol=1e-10, maxIter=500, solver=solver, precond=precond, kDim=kdim, precision=prec,
                                    zeroGuess=True)
    st = api.Solve(getter, p, params)
    assert st.converged and st.relerr <= 1e-10, (solver, precond, st)
    rel, _ = oracle_check(p, getter, p, False, 1e-10)
    assert rel <= 2e-10, rel


def test_absolute_tolerance_stops_early(ctx):
    p, getter = _convection_case(ctx, 32)
    loose = api.StructSolverParams(tol=1e-30, absTol=1e-6, maxIter=500, solver="GMRES", precond="PFMG", zeroGuess=True)
    st = api.Solve(getter, p, loose)
    assert st.converged and st.abserr <= 1e-6 and st.relerr > 1e-30


def test_bad_solver_combinations_are_refused(ctx):
    mesh, fd, p, f = poisson_case(ctx, 16, capi.BC_DIRC)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)
    with pytest.raises(ValueError):
        api.Solve(getter, p, api.StructSolverParams(solver="PFMG", precond="Jacobi"))
    prm = api.StructSolverParams().to_c()
    prm.krylov, prm.precond = capi.KRYLOV_NONE, capi.PRECOND_NONE
    import ctypes as C
    nodes, leaves = api.serialize(getter(p).residual_expr(), [p])
    hs = (C.c_void_p * len(leaves))(*[x.handle.value for x in leaves])
    h = C.c_void_p()
    rc = capi.lib().opflow_solver_create(ctx.handle, p.handle, nodes, len(nodes), hs, len(leaves), 0, C.byref(prm), C.byref(h))
    assert rc == capi.E_INVALID

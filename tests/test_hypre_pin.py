"""Solve parity pinned to the reference's own answer.

The fixtures tests/golden/hypre_*.npz hold the solution that OpFlow's HYPREEqnSolveHandler with
PrecondStructSolver<PCG, PFMG> returns (HYPREEqnSolveHandler.hpp:190-209 over the vendored HYPRE
2.33.0, krylov/pcg.c and struct_ls/pfmg_*.c), generated by tests/golden/make_golden.py through
oracle/_ref/ref_solve.  The CPU tests check the fixtures against the oracle (regenerated right-hand
side, the oracle's assembly of the same system, HYPRE's solution residual on it); the GPU tests solve
the same systems through this library and compare the solution with HYPRE's.

Stated error: the GPU solution at ||b - Ax||_2 / ||b||_2 <= 1e-10 differs from HYPRE's (itself at
<= 1.2e-12) by at most 1e-7 of max|x| in the max norm, after removing the mean for the pinned Neumann
systems as NeumEqnTest.cpp:212-215 does (the pinned cell is 0 in both, so this only removes the
constant the two tolerances leave); the measured errors are printed by the tests.
"""
import hashlib

import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

CASES = ["hypre_neum2d_n256", "hypre_dirc2d_n256", "hypre_var3d_n32"]


def regenerate_f(which, n, seed, ndim):
    """The reference driver's right-hand side: u01(seed, linear index) - 0.5 on the cells, minus its
    mean accumulated in the x-fastest order of rangeFor_s for the Neumann cases (np.cumsum adds
    sequentially, so the mean is the same float64)."""
    idx = np.arange(n ** ndim, dtype=np.uint64)
    v = orc.u01(seed, idx) - 0.5
    if which != "dirc2d":
        s = np.cumsum(v)[-1] / float(v.size)
        v = v - s
    return v.reshape([n] * ndim)  # C order: x fastest, the field's own layout


def host_case(name):
    """Oracle-side fields, the equation over leaves and the HYPRE record of one fixture."""
    meta, arr = cm.golden(name)
    which, n, seed = meta["args"][0], int(meta["args"][1]), int(meta["args"][2])
    ndim = 3 if which == "var3d" else 2
    bc = capi.BC_DIRC if which == "dirc2d" else capi.BC_NEUM
    mesh = cm.mesh_uniform([n + 1] * ndim)
    fd = cm.field_desc(ndim, capi.CENTER, [(bc, bc)] * ndim, ext=1)
    f = orc.HostField(mesh, fd)
    fv = regenerate_f(which, n, seed, ndim)
    f.data[f.slices(f.assignable())] = fv
    f.update_padding()
    x = orc.HostField(mesh, fd)
    rd = cm.readable(x.info)
    x.data[x.slices(rd)] = arr["x__data"].reshape(x.data[x.slices(rd)].shape)
    fields = {"f": f}
    e, F = cm.Leaf("p"), cm.Leaf("f")
    if which == "var3d":
        K = orc.HostField(mesh, fd)
        K.data[K.slices(rd)] = arr["K__data"].reshape(K.data[K.slices(rd)].shape)
        fields["K"] = K
        KK = cm.Leaf("K")
        getter = lambda u, F=F, KK=KK: api.Eq(F, api.dx(api.d1IntpCenterToCorner(KK, 0) * api.dx(u))
                                              + api.dy(api.d1IntpCenterToCorner(KK, 1) * api.dy(u))
                                              + api.dz(api.d1IntpCenterToCorner(KK, 2) * api.dz(u)))
    else:
        getter = lambda u, F=F: api.Eq(F, api.d2x(u) + api.d2y(u))
    return dict(meta=meta, which=which, n=n, ndim=ndim, mesh=mesh, fd=fd, fields=fields, x=x, getter=getter,
                leaf=e, pin=which != "dirc2d", f_readable=f.data[f.slices(rd)])


def oracle_system(c, x_host):
    """The oracle's assembly of the reference's system (the generateAb restatement) with x_host as the
    unknown's field; returns the residual pieces."""
    leaf = c["leaf"]
    nodes, leaves = api.serialize(c["getter"](leaf).residual_expr(), [leaf])
    hosts = [x_host if lf is leaf else c["fields"][lf.tag] for lf in leaves]
    off, coef, rhs = orc.assemble(x_host, nodes, hosts, 0, int(c["pin"]))
    rng = x_host.assignable()
    dims = [r[1] - r[0] for r in rng]
    xv = x_host.data[x_host.slices(rng)].reshape(-1)
    return dims, off, coef, rhs, xv


@pytest.mark.parametrize("name", CASES)
def test_fixture_rhs_is_the_reference_drivers(name):
    c = host_case(name)
    want = cm.record(c["meta"], "f")["sha256"]
    # the dump covers the readable range: the cells plus the ghosts the oracle's padding rules fill
    got = hashlib.sha256(np.ascontiguousarray(c["f_readable"], dtype="<f8").tobytes()).hexdigest()
    assert got == want


@pytest.mark.parametrize("name", CASES)
def test_hypre_solution_solves_the_oracles_system(name):
    """HYPRE's answer, put into the oracle's own assembly of the same equation, has the residual HYPRE
    reported: the oracle's system is the one the reference solved."""
    c = host_case(name)
    dims, off, coef, rhs, xv = oracle_system(c, c["x"])
    r, bn = orc.residual(dims, [0] * len(dims), off, coef, rhs, xv)
    st = cm.record(c["meta"], "solve")
    assert st["relres"] <= 1e-10 and st["niter"] >= 1
    assert r / bn <= max(10 * st["relres"], 1e-13), (r / bn, st)
    if c["pin"]:
        assert xv[0] == 0.0  # the pinned cell (HYPREEqnSolveHandler.hpp:148-160)
    # one PFMG V-cycle per PCG iteration: the iteration count the CPU baseline runs at
    assert cm.record(c["meta"], "solve_pfmg1")["relres"] <= 1e-10


@pytest.mark.parametrize("cycles", [1, 0])
@pytest.mark.parametrize("name", CASES)
def test_restated_pcg_pfmg_reproduces_hypre(name, cycles):
    """The oracle's restatement of PCG + PFMG (or_pfmg_pcg, the CPU baseline of the benchmark) takes
    HYPRE's iteration count and ends at HYPRE's final residual, with one PFMG V-cycle per PCG iteration
    (cycles = 1) and with PFMG's default parameters (cycles = 0, V-cycles to 1e-6 per application)."""
    c = host_case(name)
    dims, off, coef, rhs, _ = oracle_system(c, c["x"])
    x, it, rel, levels = orc.pfmg_pcg(dims, off, coef, rhs, tol=1e-10, maxit=100, cycles=cycles)
    h = cm.record(c["meta"], "solve_pfmg1" if cycles == 1 else "solve")
    assert it == h["niter"], (it, h)
    if cycles == 1:
        assert abs(rel - h["relres"]) <= 0.01 * h["relres"], (rel, h)
    else:
        assert rel <= 1e-10 and h["relres"] <= 1e-10
    a = x.copy()
    b = c["x"].data[c["x"].slices(c["x"].assignable())].reshape(-1).copy()
    if c["pin"]:
        a -= a.mean()
        b -= b.mean()
    assert np.abs(a - b).max() <= 1e-9 * np.abs(b).max()


def gpu_solve(ctx, c, prec):
    p = api.CartesianField(c["mesh"], c["fd"], ctx)
    g = {k: api.CartesianField(c["mesh"], c["fd"], ctx) for k in c["fields"]}
    for k, hf in c["fields"].items():
        g[k].upload(hf.data, update_padding=False)
    F = g["f"]
    if c["which"] == "var3d":
        K = g["K"]
        getter = lambda e: api.Eq(F, api.dx(api.d1IntpCenterToCorner(K, 0) * api.dx(e))
                                  + api.dy(api.d1IntpCenterToCorner(K, 1) * api.dy(e))
                                  + api.dz(api.d1IntpCenterToCorner(K, 2) * api.dz(e)))
    else:
        getter = lambda e: api.Eq(F, api.d2x(e) + api.d2y(e))
    p.assign(0.0)
    st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, maxIter=100, pinValue=c["pin"], precision=prec))
    return st, p


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("name", CASES)
def test_gpu_solution_matches_hypre(ctx, name, prec):
    c = host_case(name)
    st, p = gpu_solve(ctx, c, prec)
    assert st.converged and st.relerr <= 1e-10, st
    xg = orc.HostField(c["mesh"], c["fd"], data=p.download())
    dims, off, coef, rhs, xv = oracle_system(c, xg)
    r, bn = orc.residual(dims, [0] * len(dims), off, coef, rhs, xv)
    assert r / bn <= 2e-10, r / bn
    # the residual the library reports (EqnSolveState::relerr) is the one the oracle recomputes
    assert abs(st.relerr - r / bn) <= 0.01 * r / bn, (st.relerr, r / bn)
    rng = xg.assignable()
    a = xg.data[xg.slices(rng)].copy()
    b = c["x"].data[c["x"].slices(rng)].copy()
    if c["pin"]:
        assert a.reshape(-1)[0] == 0.0
        a -= a.mean()
        b -= b.mean()
    err = np.abs(a - b).max() / np.abs(b).max()
    hy = cm.record(c["meta"], "solve_pfmg1")
    print("\n%s %s: GPU %d iterations, residual %.2e (oracle %.2e); HYPRE PCG+PFMG(1 V-cycle) %d iterations; "
          "max error vs HYPRE's solution %.2e of max|x|" % (name, prec, st.niter, st.relerr, r / bn, hy["niter"], err))
    assert err <= 1e-7, err

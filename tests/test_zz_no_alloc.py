"""The residual entry point that allocates nothing (opflow_residual_norms_noalloc), for callers that
cannot allocate device memory where they need a residual: inside a CUDA stream capture, under a
host-owned pool allocator, or in a loop that must not synchronise the device.  Its output must match
the residual the allocating solver reports for the same system and solution, on two calls in a row
(the second call reuses the static scratch the first one left behind).

Collected last on purpose: if it fails, a run that stops at the first failure has already run every
other test.  It also passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest

import common as cm
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

pytestmark = pytest.mark.gpu


def test_noalloc_residual_matches_solver_residual_twice(ctx):
    torch = pytest.importorskip("torch")
    n0, n1 = 96, 80
    mesh = cm.mesh_uniform([n0 + 1, n1 + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2, ext=1)
    p, f = api.CartesianField(mesh, fd, ctx), api.CartesianField(mesh, fd, ctx)
    a = f.download()
    sl = f.index_slices(f.assignableRange)
    a[sl] = np.random.default_rng(5).standard_normal(a[sl].shape)
    f.upload(a)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)
    # the existing entry point: the allocating solver and the residual it reports
    st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, maxIter=100))
    assert st.converged
    # the same system in the solver's slot layout
    off, coef, rhs = api.assemble(getter, p)
    N = n0 * n1
    A = np.zeros((7, N))
    for e, o in enumerate(off):
        o = [int(v) for v in o]
        if o == [0, 0]:
            A[0] += coef[:, e]
        else:
            d = 0 if o[0] else 1
            A[1 + 2 * d + (1 if o[d] > 0 else 0)] += coef[:, e]
    x = np.ascontiguousarray(p.download()[sl]).reshape(-1)
    dev = torch.device("cuda", 0)
    tA = torch.from_numpy(A.reshape(-1)).to(dev)
    tb = torch.from_numpy(rhs).to(dev)
    tx = torch.from_numpy(x).to(dev)
    tr = torch.zeros(N, dtype=torch.float64, device=dev)
    tn = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
    n = (C.c_int * 2)(n0, n1)
    per = (C.c_int * 2)(0, 0)
    stream = torch.cuda.current_stream().cuda_stream
    # reference residual on the host
    X = x.reshape(n1, n0)
    Ax = A[0].reshape(n1, n0) * X
    Ax[:, 1:] += A[1].reshape(n1, n0)[:, 1:] * X[:, :-1]
    Ax[:, :-1] += A[2].reshape(n1, n0)[:, :-1] * X[:, 1:]
    Ax[1:, :] += A[3].reshape(n1, n0)[1:, :] * X[:-1, :]
    Ax[:-1, :] += A[4].reshape(n1, n0)[:-1, :] * X[1:, :]
    r_ref = rhs - Ax.reshape(-1)
    for call in range(2):
        tr.zero_()
        tn.fill_(-1.0)
        rc = capi.lib().opflow_residual_norms_noalloc(C.c_void_p(stream), 2, n, per, C.c_void_p(tA.data_ptr()), C.c_void_p(tb.data_ptr()),
                                                      C.c_void_p(tx.data_ptr()), C.c_void_p(tr.data_ptr()), C.c_void_p(tn.data_ptr()))
        capi.check(rc)
        torch.cuda.synchronize()
        norms = tn.cpu().numpy()
        assert abs(norms[1] / norms[0] - st.relerr) <= 1e-14, (call, norms, st.relerr)
        assert abs(norms[0] - np.linalg.norm(rhs)) <= 1e-12 * np.linalg.norm(rhs)
        assert np.abs(tr.cpu().numpy() - r_ref).max() <= 1e-12 * np.abs(rhs).max(), call


def host_residual(A, b, x, n, per):
    """r = b - A x of the seven-slot operator on an n[0] x n[1] x n[2] grid (x fastest), periodic axes
    wrapped: the host restatement the device result is checked against."""
    n0, n1, n2 = n
    X = x.reshape(n2, n1, n0)
    S = [a.reshape(n2, n1, n0) for a in A]
    Ax = S[0] * X
    for d, ax in ((0, 2), (1, 1), (2, 0)):
        for side, slot in ((-1, 1 + 2 * d), (1, 2 + 2 * d)):
            nb = np.roll(X, -side, axis=ax)  # nb[..i..] = X[..i+side..]
            w = S[slot].copy()
            if not per[d]:
                idx = [slice(None)] * 3
                idx[ax] = 0 if side < 0 else -1
                w[tuple(idx)] = 0.0
            Ax += w * nb
    return b - Ax.reshape(-1)


def test_noalloc_3d_periodic_and_long_rows_twice(ctx):
    """A 3D grid with one periodic axis (the z- and z+ slots and the wrapped neighbours) whose x-rows are
    longer than one chunk (1280 cells: two chunks per row, the second starting at i0 = 1024)."""
    torch = pytest.importorskip("torch")
    n0, n1, n2 = 1280, 8, 8
    # equal spacing in every dimension (an isotropic operator, which the multigrid solver converges on)
    mesh = cm.mesh_uniform([n0 + 1, n1 + 1, n2 + 1], [(0.0, n0 / 64.0), (0.0, n1 / 64.0), (0.0, n2 / 64.0)])
    fd = cm.field_desc(3, capi.CENTER, [(capi.BC_DIRC, capi.BC_DIRC), (capi.BC_DIRC, capi.BC_DIRC), (capi.BC_PERIODIC, capi.BC_PERIODIC)], ext=1)
    p, f = api.CartesianField(mesh, fd, ctx), api.CartesianField(mesh, fd, ctx)
    a = f.download()
    sl = f.index_slices(f.assignableRange)
    a[sl] = np.random.default_rng(6).standard_normal(a[sl].shape)
    f.upload(a)
    getter = lambda e: f == api.d2x(e) + api.d2y(e) + api.d2z(e)
    st = api.Solve(getter, p, api.StructSolverParams(tol=1e-10, maxIter=400))
    assert st.converged, st
    off, coef, rhs = api.assemble(getter, p)
    N = n0 * n1 * n2
    A = np.zeros((7, N))
    for e, o in enumerate(off):
        o = [int(v) for v in o]
        if o == [0, 0, 0]:
            A[0] += coef[:, e]
        else:
            d = [k for k in range(3) if o[k]][0]
            A[1 + 2 * d + (1 if o[d] > 0 else 0)] += coef[:, e]
    x = np.ascontiguousarray(p.download()[sl]).reshape(-1)
    r_ref = host_residual(A, rhs, x, (n0, n1, n2), (0, 0, 1))
    dev = torch.device("cuda", 0)
    tA = torch.from_numpy(A.reshape(-1)).to(dev)
    tb = torch.from_numpy(rhs).to(dev)
    tx = torch.from_numpy(x).to(dev)
    tr = torch.zeros(N, dtype=torch.float64, device=dev)
    tn = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
    n = (C.c_int * 3)(n0, n1, n2)
    per = (C.c_int * 3)(0, 0, 1)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        tr.fill_(np.nan)
        tn.fill_(-1.0)
        rc = capi.lib().opflow_residual_norms_noalloc(C.c_void_p(stream), 3, n, per, C.c_void_p(tA.data_ptr()), C.c_void_p(tb.data_ptr()),
                                                      C.c_void_p(tx.data_ptr()), C.c_void_p(tr.data_ptr()), C.c_void_p(tn.data_ptr()))
        capi.check(rc)
        torch.cuda.synchronize()
        norms = tn.cpu().numpy()
        assert abs(norms[1] / norms[0] - st.relerr) <= 1e-14, (call, norms, st.relerr)
        assert abs(norms[0] - np.linalg.norm(rhs)) <= 1e-12 * np.linalg.norm(rhs)
        assert abs(norms[1] - np.linalg.norm(r_ref)) <= 1e-12 * np.linalg.norm(rhs), (norms[1], np.linalg.norm(r_ref))
        assert np.abs(tr.cpu().numpy() - r_ref).max() <= 1e-12 * np.abs(rhs).max(), call


def test_noalloc_rejects_grids_beyond_its_scratch(ctx):
    # 65537 rows of one chunk each need more partial sums than the static array holds; rejected before
    # any pointer is touched
    n = (C.c_int * 3)(8, 65537, 1)
    dummy = C.c_void_p(16)
    rc = capi.lib().opflow_residual_norms_noalloc(None, 3, n, None, dummy, dummy, dummy, dummy, dummy)
    assert rc == capi.E_INVALID
    assert b"static scratch" in capi.lib().opflow_last_error()

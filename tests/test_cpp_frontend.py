"""The C++ front end (include/opflow_gb300/OpFlowGPU.hpp): programs written with OpFlow's user API
compile against it (CPU) and produce the oracle's results on the GPU."""
import os
import subprocess

import numpy as np
import pytest

import common as cm
import oracle_lib as orc
from opflow_gb300 import _capi as capi
from opflow_gb300 import api

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "opflow_gb300")


def build_example(name, outdir):
    exe = os.path.join(outdir, name)
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "opflow_gb300", "examples", name + ".cpp"), "-L", LIBDIR, "-lopflow_gpu",
           "-Wl,-rpath," + LIBDIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("name", ["ftcs2d", "poisson", "conv1d", "lid_driven"])
def test_examples_compile_and_link(tmp_path, name):
    build_example(name, str(tmp_path))


@pytest.mark.gpu
def test_ftcs2d_program_matches_oracle(ctx, tmp_path):
    n, steps, seed = 129, 50, 2024
    exe = build_example("ftcs2d", str(tmp_path))
    out = str(tmp_path / "u.bin")
    r = subprocess.run([exe, str(n), str(steps), str(seed), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    mesh = cm.mesh_uniform([n, n])
    fd = cm.field_desc(2, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * 2)
    h0 = orc.HostField(mesh, fd)
    cm.seeded_interior(h0, seed, n)
    h0.update_padding()
    h = 1.0 / (n - 1)
    s = 0.2 * h * h * 1.0
    nodes, _ = api.serialize(cm.ftcs_expr(cm.Leaf("u"), s, 2))
    for _ in range(steps):
        orc.assign(h0, nodes, [h0])
    got = np.fromfile(out, dtype=np.float64)
    assert got.size == h0.data.size
    assert np.array_equal(got.reshape(h0.data.shape), h0.data)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_poisson_program_recovers_manufactured_solution(ctx, tmp_path, prec):
    exe = build_example("poisson", str(tmp_path))
    r = subprocess.run([exe, "64", prec], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "converged 1" in r.stdout


def _conv1d_oracle(n, steps, scheme):
    """The conv1d program's fields and updates, run by the oracle."""
    mesh = cm.mesh_uniform([n])
    fu = cm.field_desc(1, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)], ext=2)
    fc = cm.field_desc(1, capi.CENTER, [(capi.BC_NEUM, capi.BC_NEUM)], ext=1)
    u, c = orc.HostField(mesh, fu), orc.HostField(mesh, fc)
    rng = u.assignable()
    x = np.array([mesh.x_at(0, i) for i in range(*rng[0])])
    u.data[u.slices(rng)] = np.where((0.2 <= x) & (x <= 0.4), 1.0, 0.0)
    u.update_padding()
    c.data[c.slices(c.assignable())] = 1.0
    c.update_padding()
    U, Cf = cm.Leaf("u"), cm.Leaf("c")
    dt, cv = 0.5e-2, 1.0
    if scheme == "upwind":
        e = U - dt * cv * api.dx(U, api.D1FirstOrderBiasedDownwind)
    elif scheme == "cond":
        e = U - dt * cv * api.conditional(1.0, api.dx(U, api.D1FirstOrderBiasedDownwind), api.dx(U, api.D1FirstOrderBiasedUpwind))
    else:
        e = U - dt * api.dx(Cf * api.d1_flux_limiter_intp(Cf, U, 0, "Minmod", to_corner=False))
    nodes, _ = api.serialize(e, [U, Cf])
    for _ in range(steps):
        orc.assign(u, nodes, [u, c])
    return u


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["upwind", "cond", "minmod"])
def test_conv1d_program_matches_oracle_and_reference(ctx, tmp_path, scheme):
    """examples/CONV1D through the C++ front end: bit-identical to the oracle; the upwind scheme also to
    the reference's own run of the example (fixture conv1d_n101)."""
    n, steps = 101, 100
    exe = build_example("conv1d", str(tmp_path))
    out = str(tmp_path / "u.bin")
    r = subprocess.run([exe, str(n), str(steps), scheme, out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    h = _conv1d_oracle(n, steps, scheme)
    got = np.fromfile(out, dtype=np.float64)
    assert got.size == h.data.size
    assert np.array_equal(got.reshape(h.data.shape), h.data)
    if scheme != "minmod":
        _, arr = cm.golden("conv1d_n101")
        assert np.array_equal(h.data[h.slices([(0, n)])], arr["u__data"])


@pytest.mark.gpu
def test_lid_driven_program_matches_the_python_run(ctx, tmp_path):
    """examples/LidDriven through the C++ front end (GMRES + PFMG solves, staticMat / pinValue pressure
    equation): every solve converges, the divergence stays at solver-tolerance level, and u, v, p are
    bit-identical to the same steps taken through the Python API (whose solves the oracle checks in
    test_lid_driven_gpu.py)."""
    from test_lid_driven_gpu import run_cavity
    n, steps = 33, 3
    exe = build_example("lid_driven", str(tmp_path))
    out = str(tmp_path / "uvp.bin")
    r = subprocess.run([exe, str(n), str(steps), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for line in r.stdout.splitlines():
        assert float(line.split("div")[1]) <= 1e-6, line
    u, v, p = run_cavity(ctx, n, steps, check=False)
    got = np.fromfile(out, dtype=np.float64)
    want = np.concatenate([f.download().reshape(-1) for f in (u, v, p)])
    assert got.size == want.size
    assert np.array_equal(got, want)

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


@pytest.mark.parametrize("name", ["ftcs2d", "poisson"])
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

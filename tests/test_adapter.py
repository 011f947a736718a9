"""The OpFlow adapter (include/opflow_gb300/adapter): OpFlow's own example programs, compiled unchanged
against OpFlow's real headers with the adapter ahead of them on the include path, run their
assignments through the engine's C ABI.

The recordings tests/golden/adapter_*.json.gz (tests/golden/make_adapter_golden.py) hold what the
examples asked of the engine: the fields they created and the node programs the adapter lowered from
OpFlow's expression types.  Checked here:
- the recordings' structure: one field, the lowered program of the example's update, the step counts;
- CONV1D's recording, replayed through the oracle, gives the reference's own result bit for bit
  (fixture conv1d_n101: OpFlow's code, run here);
- on the GPU, both recordings replayed through libopflow_gpu give the reference's result bit for bit
  (FTCS-OMP's 1025^2 x 5000 steps through the SHA-256 of the field and its centre value);
- a solve program on OpFlow's API (tests/adapter/poisson_solve.cpp: Solve, then makeEqnSolveHandler
  solved twice): its recording holds the lowered equation and the solver parameters, and on the GPU the
  engine's solves reach the tolerance and agree with the reference's HYPRE solution;
- examples/EqnHandler/EqnHandler.cpp (GMRES + PFMG, staticMat): on the GPU its solve meets the
  handler's tolerance on the reference's system (oracle assembly);
- where the OpFlow tree is named by OPFLOW_REFERENCE: the examples compile unchanged against the
  adapter and link against libopflow_gpu, and CONV1D, run on the host stand-in of the C ABI, writes the
  reference's values (the recording step, repeated).
"""
import hashlib
import os
import subprocess

import numpy as np
import pytest

import adapter_replay as ar
import oracle_lib as orc
import common as cm
from opflow_gb300 import _capi as capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_ftcs_omp_recording_is_the_examples_update():
    rec = ar.load("ftcs_omp")
    assert rec["example"] == "examples/FTCS2D/FTCS-OMP.cpp"
    assert len(rec["fields"]) == 1
    f = rec["fields"][0]
    assert f["ndim"] == 2 and f["dims"][:2] == [1025, 1025] and f["loc"][:2] == [capi.CORNER, capi.CORNER]
    assert f["bc_type"][:2] == [[capi.BC_DIRC] * 2] * 2 and f["bc_value"][:2] == [[1.0, 1.0], [1.0, 1.0]]
    # u = 0 (a scalar fill on the host side of the field: uploaded before the first assignment), then
    # 5000 x u = u + dt*alpha*(d2x(u) + d2y(u))
    assert rec["events"][0]["ev"] == "upload" and rec["events"][0]["zero_padded"]
    assigns = [e for e in rec["events"] if e["ev"] == "assign"]
    assert [e["repeat"] for e in assigns] == [5000]
    kinds = [n[0] for n in assigns[0]["nodes"]]
    assert kinds.count(capi.NODE_D2) == 2 and kinds.count(capi.NODE_FIELD) == 3 and kinds[-1] == capi.NODE_ADD
    assert sorted(n[3] for n in assigns[0]["nodes"] if n[0] == capi.NODE_D2) == [0, 1]
    assert all(e["mode"] == 0 and e["arith"] == capi.ASSIGN_EQ for e in assigns)  # EXACT, `=`


def test_conv1d_recording_replays_to_the_reference_on_the_oracle():
    rec = ar.load("conv1d")
    assigns = [e for e in rec["events"] if e["ev"] == "assign"]
    assert [e["repeat"] for e in assigns] == [100]
    assert [n[0] for n in assigns[0]["nodes"]].count(capi.NODE_D1_BIASED_DOWN) == 1
    out = ar.replay_oracle(rec)
    a, inf = out[rec["fields"][0]["id"]]
    _, arr = cm.golden("conv1d_n101")
    assert np.array_equal(ar.local_values(a, inf), arr["u__data"])


@pytest.mark.gpu
def test_recorded_examples_replay_to_the_reference_on_the_gpu(ctx):
    rec = ar.load("ftcs_omp")
    a, inf = ar.replay_gpu(rec, ctx)[rec["fields"][0]["id"]]
    loc = ar.local_values(a, inf)
    ref = rec["reference"]
    assert hashlib.sha256(np.ascontiguousarray(loc, dtype="<f8").tobytes()).hexdigest() == ref["sha256_local"]
    n = inf.data_dims[0]
    assert loc.reshape(-1, n)[512 - inf.local[1][0], 512 - inf.local[0][0]] == ref["center"]
    rec = ar.load("conv1d")
    a, inf = ar.replay_gpu(rec, ctx)[rec["fields"][0]["id"]]
    _, arr = cm.golden("conv1d_n101")
    assert np.array_equal(ar.local_values(a, inf), arr["u__data"])


def _compile(ref, src, out, lib_dir, lib):
    flags = open(os.path.join(ROOT, "oracle", "_ref", "hypre", "include_flags.txt")).read().split()
    cmd = (["g++", "-std=c++23", "-O2", "-ffp-contract=off", "-w", "-include", "numeric",
            "-I", os.path.join(ROOT, "include", "opflow_gb300", "adapter"), "-I", os.path.join(ROOT, "include"),
            "-I", os.path.join(ROOT, "oracle", "_ref", "gen"), "-I", os.path.join(ROOT, "oracle", "ref", "shim")] + flags +
           ["-I", os.path.join(ref, "src"), "-I", os.path.join(ref, "include"),
            os.path.join(ROOT, src) if src.startswith("tests/") else os.path.join(ref, src), "-o", out,
            "-L", lib_dir, "-l" + lib, "-Wl,-rpath," + lib_dir,
            # PrecondStructSolver's constructor creates HYPRE objects (the adapter's handler never solves with them)
            os.path.join(ROOT, "oracle", "_ref", "hypre", "libHYPRE_struct.a"), "-fopenmp"])
    subprocess.check_call(cmd)


def test_examples_compile_unchanged_against_the_adapter(tmp_path):
    ref = os.environ.get("OPFLOW_REFERENCE")
    if not ref or not os.path.isdir(os.path.join(ref, "examples")):
        pytest.skip("the OpFlow tree (OPFLOW_REFERENCE) is not here")
    if not os.path.exists(os.path.join(ROOT, "oracle", "_ref", "hypre", "include_flags.txt")):
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")], env=dict(os.environ))
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    # linked against the engine itself
    for name, src in (("ftcs_omp", "examples/FTCS2D/FTCS-OMP.cpp"), ("conv1d", "examples/CONV1D/CONV1D.cpp"),
                      ("poisson_solve", "tests/adapter/poisson_solve.cpp"), ("eqnhandler", "examples/EqnHandler/EqnHandler.cpp"),
                      ("ftcs1d", "examples/FTCS/FTCS.cpp"), ("liddriven2d", "examples/LidDriven/LidDriven2D.cpp")):
        _compile(ref, src, str(tmp_path / name), os.path.join(ROOT, "opflow_gb300"), "opflow_gpu")
    # CONV1D on the host stand-in of the C ABI writes the reference's values
    exe = str(tmp_path / "conv1d_double")
    _compile(ref, "examples/CONV1D/CONV1D.cpp", exe, os.path.join(ROOT, "oracle", "_build"), "opflow_abi_double")
    run = tmp_path / "run"
    run.mkdir()
    subprocess.check_call([exe], cwd=str(run), stdout=subprocess.DEVNULL)
    _, arr = cm.golden("conv1d_n101")
    want = arr["u__data"]
    zones = (run / "u.tec").read_text().split("ZONE")
    vals = np.array([float(t) for t in zones[-1].split("\n")[4:] if t.strip()][-want.size:])
    assert np.abs(vals - want).max() <= 1e-9


def test_poisson_solve_recording_is_the_programs_equation():
    rec = ar.load("poisson_solve")
    solvers = [e for e in rec["events"] if e["ev"] == "solver"]
    solves = [e for e in rec["events"] if e["ev"] == "solve"]
    assert len(solvers) == 2 and len(solves) == 3  # Solve(...), then one handler solved twice
    assert [st["niter"] for st in rec["reference"]["solves"]][1:] == [1, 1]  # warm starts (initx)
    for s in solvers:
        assert s["params"]["krylov"] == capi.KRYLOV_PCG and s["params"]["precond"] == capi.PRECOND_MG
        assert s["params"]["tol"] == 1e-10 and s["params"]["max_iter"] == 100
        kinds = [n[0] for n in s["nodes"]]
        assert kinds[-1] == capi.NODE_SUB and kinds.count(capi.NODE_D2) == 2  # lhs - rhs of f == d2x(e) + d2y(e)


@pytest.mark.gpu
def test_recorded_solve_program_replays_on_the_gpu(ctx):
    """The program's solves, lowered by the adapter from OpFlow's Equation type, run on the engine's
    PCG + multigrid: every solve reaches 1e-10 (relative 2-norm) and the solution agrees with the
    reference's own (the same program on OpFlow + HYPRE PCG + PFMG, tol 1e-10) to 1e-8 of its maximum."""
    rec = ar.load("poisson_solve")
    states = []
    out = ar.replay_gpu(rec, ctx, states)
    assert len(states) == 3 and all(st.converged and st.rel_residual <= 1e-10 for st in states), [(s.iterations, s.rel_residual) for s in states]
    target = [e for e in rec["events"] if e["ev"] == "solver"][0]["target"]
    a, inf = out[target]
    got = ar.local_values(a, inf)
    want = np.array(rec["reference"]["values"])
    assert np.abs(got - want).max() <= 1e-8 * np.abs(want).max()


def test_eqnhandler_recording_is_a_gmres_pfmg_handler():
    """examples/EqnHandler/EqnHandler.cpp: makeEqnSolveHandler(d2x(e) + d2y(e) == 1.0, u,
    PrecondStructSolver<GMRES, PFMG>) with staticMat, lowered by the adapter."""
    rec = ar.load("eqnhandler")
    assert rec["example"] == "examples/EqnHandler/EqnHandler.cpp"
    solvers = [e for e in rec["events"] if e["ev"] == "solver"]
    assert len(solvers) == 1 and sum(e["ev"] == "solve" for e in rec["events"]) == 1
    p = solvers[0]["params"]
    assert p["krylov"] == capi.KRYLOV_GMRES and p["precond"] == capi.PRECOND_MG and p["static_mat"] == 1
    kinds = [n[0] for n in solvers[0]["nodes"]]
    assert kinds.count(capi.NODE_D2) == 2 and kinds[-1] == capi.NODE_SUB and capi.NODE_CONST in kinds


@pytest.mark.gpu
def test_recorded_gmres_handler_replays_to_the_reference_system_on_the_gpu(ctx):
    """The EqnHandler example's GMRES + multigrid solve, replayed through libopflow_gpu: the solution
    meets the handler's tolerance on the reference's own system (the oracle's assembly of the recorded
    equation, Dirichlet 0 on the 11 x 11 node mesh of [0, 10]^2)."""
    rec = ar.load("eqnhandler")
    states = []
    out = ar.replay_gpu(rec, ctx, states)
    assert len(states) == 1 and states[0].converged, (states[0].iterations, states[0].rel_residual)
    ev = [e for e in rec["events"] if e["ev"] == "solver"][0]
    fr = rec["fields"][0]
    a, inf = out[fr["id"]]
    from opflow_gb300 import api
    # the recorded mesh and field description, as the example built them
    mesh = api.CartesianMesh(2, fr["dims"][:2], fr["start"][:2], fr["pad_width"], [np.array(fr["x0"]), np.array(fr["x1"])],
                             [np.array(fr["dx0"]), np.array(fr["dx1"])])
    _, fd, _ = ar._descs(fr)
    hf = orc.HostField(mesh, fd, data=a)
    assert list(hf.data.shape) == [inf.data_dims[1], inf.data_dims[0]]
    off, coef, rhs = orc.assemble(hf, ar._nodes(ev), [hf], 0, 0)
    rng = hf.assignable()
    x = hf.data[hf.slices(rng)].reshape(-1)
    r, bn = orc.residual([q[1] - q[0] for q in rng], [0] * len(rng), off, coef, rhs, x)
    assert r / bn <= 1e-8, r / bn

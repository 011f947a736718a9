"""Builds the OpFlow examples unchanged against the adapter and records what they ask of the engine.

    OPFLOW_REFERENCE=<OpFlow tree> python tests/golden/make_adapter_golden.py

For each example (examples/FTCS2D/FTCS-OMP.cpp, examples/CONV1D/CONV1D.cpp and
examples/EqnHandler/EqnHandler.cpp of the OpFlow tree, and tests/adapter/poisson_solve.cpp, a solve
program on OpFlow's API) the source file is compiled as it is, with include/opflow_gb300/adapter ahead of OpFlow's include
directories (its `#include <OpFlow>` then reads OpFlow's headers with CartesianField assignments routed
to the engine), and linked with oracle/abi_double.c, the host stand-in of the engine's C ABI computed
by the oracle.  The program runs with OPFLOW_ABI_RECORD set; the fields it creates and the assignment
programs the adapter lowered from OpFlow's expression types are stored (consecutive identical
assignments run-length encoded) as tests/golden/adapter_<example>.json.gz, next to the reference's
own result of the same computation (oracle/_ref/ref_driver: ftcs_omp, conv1d; oracle/_ref/ref_solve:
program2d), which the recorded run must reproduce: FTCS-OMP's last snapshot bit for bit (it writes
RawBinary files through the adapter's H5Stream stand-in), CONV1D's last Tecplot zone to its ten printed
digits, poisson_solve's solution (tests/adapter/poisson_solve.cpp, Solve and makeEqnSolveHandler on
OpFlow's API) to 1e-12 of the HYPRE solution.  The GPU tests replay the recordings through
libopflow_gpu.

Needs the OpFlow tree (compiler shims: oracle/ref/shim, oracle/_ref/gen, the HYPRE headers of
oracle/build_hypre.sh); the fixtures are committed so the replays run anywhere.
"""
import gzip
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import make_golden as mg  # noqa: E402

# name -> (source, relative to the OpFlow tree unless it starts with "tests/")
EXAMPLES = {"ftcs_omp": "examples/FTCS2D/FTCS-OMP.cpp", "conv1d": "examples/CONV1D/CONV1D.cpp",
            "poisson_solve": "tests/adapter/poisson_solve.cpp", "eqnhandler": "examples/EqnHandler/EqnHandler.cpp"}


def source_path(ref, src):
    return os.path.join(ROOT, src) if src.startswith("tests/") else os.path.join(ref, src)


def compile_example(ref, src, out):
    flags = open(os.path.join(ROOT, "oracle", "_ref", "hypre", "include_flags.txt")).read().split()
    cmd = (["g++", "-std=c++23", "-O2", "-ffp-contract=off", "-w", "-include", "numeric",
            "-I", os.path.join(ROOT, "include", "opflow_gb300", "adapter"), "-I", os.path.join(ROOT, "include"),
            "-I", os.path.join(ROOT, "oracle", "_ref", "gen"), "-I", os.path.join(ROOT, "oracle", "ref", "shim")] + flags +
           ["-I", os.path.join(ref, "src"), "-I", os.path.join(ref, "include"), source_path(ref, src), "-o", out,
            "-L", os.path.join(ROOT, "oracle", "_build"), "-lopflow_abi_double", "-Wl,-rpath," + os.path.join(ROOT, "oracle", "_build"),
            # PrecondStructSolver's constructor creates HYPRE objects (never solved with here)
            os.path.join(ROOT, "oracle", "_ref", "hypre", "libHYPRE_struct.a"), "-fopenmp"])
    subprocess.check_call(cmd)


def compress(lines):
    """JSON-lines record -> {fields, events}: consecutive identical assignments merged with a count."""
    fields, events = [], []
    for ln in lines:
        r = json.loads(ln)
        op = r.pop("op")
        if op == "field":
            fields.append(r)
        elif op in ("upload", "solver", "solve"):
            events.append(dict(r, ev=op))
        else:
            ev = dict(r, ev="assign", repeat=1)
            if events and events[-1]["ev"] == "assign" and all(events[-1][k] == ev[k] for k in ("dst", "arith", "mode", "leaves", "nodes")):
                events[-1]["repeat"] += 1
            else:
                events.append(ev)
    return {"fields": fields, "events": events}


def field_sha(values):
    return hashlib.sha256(np.ascontiguousarray(values, dtype="<f8").tobytes()).hexdigest()


def main():
    ref = os.environ.get("OPFLOW_REFERENCE")
    if not ref:
        sys.exit("set OPFLOW_REFERENCE to the OpFlow source tree")
    if not os.path.exists(mg.DRIVER):
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.dirname(HERE))
    import common as cm
    wanted = set(sys.argv[1:]) or set(EXAMPLES)
    for name, src in EXAMPLES.items():
        if name not in wanted:
            continue
        with tempfile.TemporaryDirectory() as td:
            exe = os.path.join(td, name)
            compile_example(ref, src, exe)
            rec = os.path.join(td, "rec.jsonl")
            subprocess.check_call([exe], cwd=td, env=dict(os.environ, OPFLOW_ABI_RECORD=rec), stdout=subprocess.DEVNULL)
            out = compress(open(rec).read().splitlines())
            out["example"] = src
            out["how"] = ("compiled unchanged with include/opflow_gb300/adapter ahead of OpFlow's include directories, linked with "
                          "oracle/abi_double.c (the oracle behind the engine's C ABI), run with OPFLOW_ABI_RECORD")
            if name == "ftcs_omp":
                # the reference's own result of the same computation, and the adapter run's last snapshot
                refout = os.path.join(td, "ref.bin")
                subprocess.check_call([mg.DRIVER, refout, "ftcs_omp", "1025", "5000"])
                _, meta, arrs = mg.parse(refout)[0]
                rd, lo = meta["readable"], meta["local"]
                full = arrs["data"].reshape(rd[1][1] - rd[1][0], rd[0][1] - rd[0][0])
                local = full[lo[1][0] - rd[1][0]:lo[1][1] - rd[1][0], lo[0][0] - rd[0][0]:lo[0][1] - rd[0][0]]
                snaps = sorted(f for f in os.listdir(td) if f.endswith(".cart"))
                last = cm.parse_cart(os.path.join(td, snaps[-1]))
                assert np.array_equal(last["values"], local.reshape(-1)), "the adapter run differs from the reference"
                out["reference"] = {"readable": rd, "local": lo, "sha256_readable": field_sha(arrs["data"]), "sha256_local": field_sha(local),
                                    "center": float(full[512 - rd[1][0], 512 - rd[0][0]]), "snapshots": snaps,
                                    "note": "oracle/_ref/ref_driver ftcs_omp 1025 5000; the adapter run's last .cart equals it bit for bit"}
            elif name == "poisson_solve":
                # the same program on the reference itself (HYPRE PCG + PFMG): its solution and solve states
                refout = os.path.join(td, "ref.bin")
                subprocess.check_call([mg.SOLVER, refout, "program2d", "64", "0", "1e-10", "100"])
                recs = mg.parse(refout)
                _, meta, arrs = recs[-1]
                rd, lo = meta["readable"], meta["local"]
                full = arrs["data"].reshape(rd[1][1] - rd[1][0], rd[0][1] - rd[0][0])
                local = full[lo[1][0] - rd[1][0]:lo[1][1] - rd[1][0], lo[0][0] - rd[0][0]:lo[0][1] - rd[0][0]].reshape(-1)
                last = cm.parse_cart(os.path.join(td, "p_0.cart"))
                assert np.abs(last["values"] - local).max() <= 1e-12 * np.abs(local).max(), "the adapter run differs from the reference"
                out["reference"] = {"values": local.tolist(), "solves": [m for k, m, _ in recs if k == "SOLVE"],
                                    "note": "oracle/_ref/ref_solve program2d 64 0 1e-10 100 (the program on OpFlow + HYPRE); the "
                                            "adapter run on the stand-in C ABI (restated PCG + PFMG, warm starts) agrees to 1e-12"}
            elif name == "eqnhandler":
                # the example writes no field: the replay's solution is checked on the reference's system
                # (the oracle's assembly of the recorded equation)
                out["reference"] = {"note": "EqnHandler solves d2x(u) + d2y(u) == 1 with GMRES + PFMG and writes nothing; the "
                                            "GPU replay's solution is checked against the oracle's assembly of that system"}
            else:
                _, arr = cm.golden("conv1d_n101")
                want = arr["u__data"]
                zones = open(os.path.join(td, "u.tec")).read().split("ZONE")
                vals = np.array([float(t) for t in zones[-1].split("\n")[4:] if t.strip()][-want.size:])
                assert np.abs(vals - want).max() <= 1e-9, "the adapter run differs from the reference"
                out["reference"] = {"fixture": "conv1d_n101", "note": "oracle/_ref/ref_driver conv1d 101 100; the adapter run's last "
                                                                      "Tecplot zone equals it to its printed digits"}
        with gzip.open(os.path.join(HERE, "adapter_%s.json.gz" % name), "wt") as fo:
            json.dump(out, fo)
        print(name, len(out["fields"]), "fields,", sum(e.get("repeat", 0) for e in out["events"]), "assignments in",
              sum(1 for e in out["events"] if e["ev"] == "assign"), "programs")


if __name__ == "__main__":
    main()

"""Regenerates the golden fixtures in this directory from the reference itself.

Runs oracle/_ref/ref_driver and oracle/_ref/ref_solve (OpFlow's own CPU code and, for the solves, its
HYPREEqnSolveHandler over the vendored HYPRE PCG + PFMG, built by oracle/build_ref.sh from the reference
sources) on small cases and stores every dump as a .npz next to this script.  Needs the reference tree
(named by $OPFLOW_REFERENCE, present only where the fixtures are generated); the fixtures themselves are
committed so the tests run anywhere.

    OPFLOW_REFERENCE=<OpFlow tree> python tests/golden/make_golden.py [case ...]   (all cases when none is named)
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
SOLVER = os.path.join(ROOT, "oracle", "_ref", "ref_solve")

CASES = {
    # FTCS2D (Corner, Dirichlet all sides): n, steps, seed, bc value, dt/h^2
    "ftcs2d_n17": ["ftcs2d", "17", "50", "1", "0.0", "0.2"],
    "ftcs2d_n33_bc1": ["ftcs2d", "33", "20", "2", "1.0", "0.2"],
    "ftcs2d_n20_nonpow2": ["ftcs2d", "20", "30", "3", "0.5", "0.2"],
    "ftcs2d_n65": ["ftcs2d", "65", "100", "4", "0.0", "0.25"],
    # FTCS3D (Corner, Dirichlet 0, 8 Gaussians): n, steps, seed, dt/h^2
    "ftcs3d_n9": ["ftcs3d", "9", "10", "5", "0.1"],
    "ftcs3d_n12_nonpow2": ["ftcs3d", "12", "6", "6", "0.1"],
    # WENO5-JS + RK3, periodic cell-centred lines: nx, ny, steps, seed, upwind-kernel flag
    "weno_down_32x4": ["weno", "32", "4", "5", "7", "0"],
    "weno_up_64x3": ["weno", "64", "3", "8", "8", "1"],
    "weno_down_40x2_nonpow2": ["weno", "40", "2", "3", "9", "0"],
    # assembly (StencilField + StencilPad, generateAb without HYPRE)
    "asm_csr_dirc": ["assemble", "csr_dirc"],
    "asm_csr_neum": ["assemble", "csr_neum"],
    "asm_csr_periodic": ["assemble", "csr_periodic"],
    "asm_neum2d_n8": ["assemble", "neum2d", "8"],
    "asm_dirc2d_n8": ["assemble", "dirc2d", "8"],
    "asm_periodic2d_n8": ["assemble", "periodic2d", "8"],
    "asm_var2d_n16": ["assemble", "var2d", "16"],
    "asm_helm_corner_n9": ["assemble", "helm_corner", "9"],
    "asm_var3d_n6": ["assemble", "var3d", "6"],
    "asm_biased2d_n12": ["assemble", "biased2d", "12"],
    "asm_funcs2d_n10": ["assemble", "funcs2d", "10"],
    # one-sided differences and corner-to-centre interpolation on a stretched mesh: nx, ny, seed
    "ops_12x9": ["ops", "12", "9", "21"],
    "ops_16x20": ["ops", "16", "20", "22"],
    # comparisons, logic, conditionals, per-element functions, flux-limiter interpolation: nx, ny, seed
    "logic_12x9": ["logic", "12", "9", "31"],
    "logic_16x20": ["logic", "16", "20", "32"],
    # examples/CONV1D: nodes, steps
    "conv1d_n101": ["conv1d", "101", "100"],
}
# HYPREEqnSolveHandler + PrecondStructSolver<PCG, PFMG> (tol 1e-10, maxIter 100, twoNorm): case, cells per
# side, seed.  The solution stored is the one PFMG with HYPRE's default parameters gives (the reference
# tests' usage, NeumEqnTest.cpp:204-216); a second run with one PFMG V-cycle per PCG iteration (the CPU
# baseline's setting) contributes only its iteration count and residual.  The right-hand side f is not
# stored: the tests regenerate it from the seed and check it against the stored SHA-256 of its bytes.
HYPRE_CASES = {
    "hypre_neum2d_n256": ["neum2d", "256", "7"],
    "hypre_dirc2d_n256": ["dirc2d", "256", "8"],
    "hypre_var3d_n32": ["var3d", "32", "9"],
}

# field construction + padding: nx, ny, loc (0 corner / 1 centre), bc_lo, bc_hi, ext
# bc codes: 0 Dirc, 1 Neum, 2 Periodic, 3 Symm, 4 ASymm
for loc in (0, 1):
    for lo, hi in ((0, 0), (0, 1), (1, 0), (1, 1), (2, 2), (3, 4), (4, 3), (0, 3), (1, 4)):
        for ext in (1, 2):
            CASES["pad_l%d_b%d%d_e%d" % (loc, lo, hi, ext)] = ["padding", "9", "7", str(loc), str(lo), str(hi), str(ext)]


def parse(path):
    raw = open(path, "rb").read()
    pos, out = 0, []
    while pos < len(raw):
        nl = raw.index(b"\n", pos)
        kind, js = raw[pos:nl].decode().split(" ", 1)
        meta = json.loads(js)
        pos = nl + 1
        if kind == "SOLVE":
            out.append((kind, meta, {}))
            continue
        if kind == "FIELD":
            n = meta["count"]
            arr = np.frombuffer(raw[pos:pos + 8 * n], dtype="<f8").copy()
            pos += 8 * n
            out.append((kind, meta, {"data": arr}))
        else:
            n, ne = meta["count"], meta["nent"]
            coef = np.frombuffer(raw[pos:pos + 8 * n * ne], dtype="<f8").copy().reshape(n, ne)
            pos += 8 * n * ne
            rhs = np.frombuffer(raw[pos:pos + 8 * n], dtype="<f8").copy()
            pos += 8 * n
            out.append((kind, meta, {"coef": coef, "rhs": rhs}))
    return out


def hypre_case(name, args):
    import hashlib
    arrays, metas = {}, []
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        subprocess.check_call([SOLVER, out] + args + ["1e-10", "100", "1", "0"])
        recs = parse(out)
        subprocess.check_call([SOLVER, out] + args + ["1e-10", "100", "1", "1"])
        one_cycle = [m for k, m, _ in parse(out) if k == "SOLVE"][0]
    for kind, meta, arrs in recs:
        if kind == "SOLVE":
            metas.append({"kind": kind, "key": "solve", "meta": meta})
            metas.append({"kind": kind, "key": "solve_pfmg1", "meta": one_cycle})
            continue
        key = meta["name"]
        if key == "f":
            meta = dict(meta, sha256=hashlib.sha256(arrs["data"].astype("<f8").tobytes()).hexdigest())
        else:
            arrays["%s__data" % key] = arrs["data"]
        metas.append({"kind": kind, "key": key, "meta": meta})
    arrays["meta"] = np.array(json.dumps({"args": args, "records": metas}))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print(name, [m["key"] for m in metas], metas[-1]["meta"] if metas else None)


def rawbinary_case(name, seed):
    """Files written by the reference's Utils::RawBinaryOStream, stored byte for byte."""
    arrays, metas = {}, []
    with tempfile.TemporaryDirectory() as td:
        out = os.path.join(td, "o.bin")
        subprocess.check_call([DRIVER, out, "rawbinary", td, str(seed)])
        for kind, meta, arrs in parse(out):
            arrays["%s__data" % meta["name"]] = arrs["data"]
            metas.append({"kind": kind, "key": meta["name"], "meta": meta})
        files = sorted(f for f in os.listdir(td) if f.endswith(".cart"))
        for f in files:
            arrays["file__" + f[:-5]] = np.frombuffer(open(os.path.join(td, f), "rb").read(), dtype=np.uint8)
    arrays["meta"] = np.array(json.dumps({"args": ["rawbinary", str(seed)], "records": metas, "files": files}))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
    print(name, files)


def main():
    if not (os.path.exists(DRIVER) and os.path.exists(SOLVER)):
        subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh")])
    wanted = set(sys.argv[1:]) or (set(CASES) | set(HYPRE_CASES))
    for name, args in sorted(HYPRE_CASES.items()):
        if name in wanted:
            hypre_case(name, args)
    if "rawbinary_ref" in wanted or not sys.argv[1:]:
        rawbinary_case("rawbinary_ref", 51)
    for name, args in sorted(CASES.items()):
        if name not in wanted:
            continue
        with tempfile.TemporaryDirectory() as td:
            out = os.path.join(td, "o.bin")
            subprocess.check_call([DRIVER, out] + args)
            recs = parse(out)
        arrays, metas = {}, []
        for kind, meta, arrs in recs:
            key = meta.get("name", "stencil")
            metas.append({"kind": kind, "key": key, "meta": meta})
            for k, v in arrs.items():
                arrays["%s__%s" % (key, k)] = v
        arrays["meta"] = np.array(json.dumps({"args": args, "records": metas}))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **arrays)
        print(name, [m["key"] for m in metas])


if __name__ == "__main__":
    sys.exit(main())

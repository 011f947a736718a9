#!/usr/bin/env python3
"""Benchmark of the GB300 engine for OpFlow's hot paths; prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workloads (seeded synthetic inputs with the configurations' shapes and value distributions):
  ftcs3d  7-point FTCS heat update, 512^3 node grid, Dirichlet 0, u0 = 8 seeded Gaussians,
          dt = 0.1 h^2 (one step = one update of the whole grid; GLUP/s)
  ftcs2d  the CPU-runnable FTCS2D case: 1025^2 nodes, Dirichlet 0, u0 ~ U[0,1), dt = 0.2 h^2
  poisson2d  -Lap(p) = f on 2048^2 cells, homogeneous Neumann, pinned (the reference's pinValue), f ~ N(0,1)
          projected to zero mean, to 1e-10 relative residual: mixed (FP32 V-cycle in FP64 flexible PCG)
          next to plain FP64 (solves/s)
  serve   (default) Poisson-process arrivals of 70% one-shot Poisson solves (2D side LogU[129,2049],
          3D side LogU[64,256], Neumann / Dirichlet 50/50) and 30% backward-Euler heat sessions of
          10-100 steps, mixed precision to 1e-10, at arrival rates 50, 200 and 2000 req/s: value =
          device-resident batched solves/s of the window's one-shot requests, e2e = the request
          server's host-to-host solves/s with p50/p99 at the highest rate, next to plain FP64 serving
          one request at a time (the whole sweep is in config)
  poisson3d  div(exp(g) grad p) = f on 256^3 cells, Neumann, pinned, mixed next to plain FP64
          (--const-coef: d2x + d2y + d2z instead, the serving workload's 3D operator)
  batched 512 corner-node Dirichlet problems (I - k Lap) u = f of sides 65..1025 in one batched
          solve, mixed precision, next to a loop of plain FP64 single solves
  weno    WENO5-JS + RK3 on 65536 periodic lines of 4096 cells (one RK3 step per bench step)
  ftcs_batch  explicit steps of 256 uneven 2D grids (side LogU[65,513]) in one launch per step
          (opflow_assign_batch), next to the same grids stepped one after another

`--impl reference` times the reference's CPU algorithm (the C restatement under oracle/, the
reference itself does not build on the Arm machine) on the host cores for the same metric.

Multi-GPU (torchrun): the explicit path does not shard inside one grid here ("replicas only"):
every rank runs its own replica, the timed region is bracketed by barriers and the max time over
ranks is used; value = all ranks' lattice updates / that time.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
from opflow_gb300 import workloads as wl  # noqa: E402  (numpy-only seeded inputs)

METRIC = "served mixed-prec vs plain FP64 GPU: solves/s, p99 @1e-10 resid; GLUP/s %HBM"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM = 6800.0


def peak_hbm():
    try:
        return float(json.load(open(PEAKS))["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM, "fallback"


def traffic_for(workload):
    """dram bytes per launch of the dominant kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        return json.load(open(p)).get(workload)
    except Exception:
        return None


# ------------------------------------------------------------------------------------------- clocks
class ClockSampler:
    """Samples nvidia-smi during the timed region (SM clock, max clock, throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


# ------------------------------------------------------------------------------------------ inputs
def gaussians_u0(torch, n, seed, dev):
    """u0 = sum of 8 Gaussians (centres in [0.2,0.8]^3, widths [0.03,0.1], amplitudes [0.5,1])."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    c = 0.2 + 0.6 * torch.rand(8, 3, generator=g, dtype=torch.float64)
    w = 0.03 + 0.07 * torch.rand(8, generator=g, dtype=torch.float64)
    a = 0.5 + 0.5 * torch.rand(8, generator=g, dtype=torch.float64)
    x = torch.linspace(0, 1, n, dtype=torch.float64, device=dev)
    u = torch.zeros((n, n, n), dtype=torch.float64, device=dev)
    for k in range(8):
        ex = torch.exp(-(x - c[k, 0]) ** 2 / w[k] ** 2)
        ey = torch.exp(-(x - c[k, 1]) ** 2 / w[k] ** 2)
        ez = torch.exp(-(x - c[k, 2]) ** 2 / w[k] ** 2)
        u += a[k] * ez[:, None, None] * ey[None, :, None] * ex[None, None, :]
    u[0, :, :] = u[-1, :, :] = 0
    u[:, 0, :] = u[:, -1, :] = 0
    u[:, :, 0] = u[:, :, -1] = 0
    return u


def ftcs_kernel_label(D, mode, steps):
    """The dominant kernel of a timed FTCS run (the switches are the library's own)."""
    resident = mode == "fast" and steps >= 2 and os.environ.get("OPFLOW_FX_RESIDENT", "1") != "0"
    if D == 2:
        if resident:
            return "axis2d_fxres_kernel<0> (resident fixed-point run; its first step converts float64 in, its last float64 out)"
        return "axis2d_kernel<FAST>" if mode == "fast" else "axis2d_kernel<EXACT>"
    if resident and os.environ.get("OPFLOW_FXRES_TMA", "1") != "0":
        return ("axis3d_fxtma_kernel (resident fixed-point run, planes staged in shared memory by TMA; its first and last steps "
                "run axis3d_fxres_kernel<1|2, 6>: float64 in, float64 out)")
    if resident:
        return "axis3d_fxres_kernel<0, 6> (resident fixed-point run; its first step converts float64 in, its last float64 out)"
    return "axis3d_rb_kernel<FAST>" if mode == "fast" else "axis3d_kernel<EXACT>"


def replica_max(x, world, dist, device):
    """The largest of the ranks' x: a time, the job's time being its slowest replica's; x at one rank."""
    if world <= 1:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_min(x, world, dist, device):
    """The smallest of the ranks' x: a rate, every replica doing the same work; x at one rank."""
    if world <= 1:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MIN)
    return float(t.item())


def workload_cfg(name):
    if name == "ftcs3d":
        return dict(workload="ftcs3d", grid=[512, 512, 512], loc="node", bc="dirichlet 0", dt="0.1*h^2", init="8 seeded Gaussians",
                    expression="u = u + dt*alpha*(d2x(u)+d2y(u)+d2z(u))", l2="field 1.07 GB > L2 (129 MB): no flush needed")
    if name == "ftcs2d":
        return dict(workload="ftcs2d", grid=[1025, 1025], loc="node", bc="dirichlet 0", dt="0.2*h^2", init="U[0,1) seeded",
                    expression="u = u + dt*alpha*(d2x(u)+d2y(u))", l2="field 8.4 MB fits in L2: L2-resident")
    if name == "ftcs_batch":
        return dict(workload="ftcs_batch", grids=256, side="LogU[65,513] nodes", mode="exact",
                    sample="the host port steps one 1025^2 grid (the same update, one grid at a time)")
    raise SystemExit("unknown workload " + name)


# ---------------------------------------------------------------------------------- reference (CPU)
def cpu_ftcs_sample(workload, threads, reps):
    """The oracle's FTCS on a bounded sample of the workload; returns (GLUP/s, sample description)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    import common as cm
    import oracle_lib as orc
    from opflow_gb300 import _capi as capi
    from opflow_gb300 import api
    used = orc.lib().or_set_threads(threads)
    if workload == "ftcs3d":
        n = 192
        D = 3
        cfl = 0.1
    else:
        n = 1025
        D = 2
        cfl = 0.2
    mesh = cm.mesh_uniform([n] * D)
    fd = cm.field_desc(D, capi.CORNER, [(capi.BC_DIRC, capi.BC_DIRC)] * D)
    u = orc.HostField(mesh, fd)
    inner = tuple(slice(1, -1) for _ in range(D))
    u.data[inner] = np.random.default_rng(0).random(u.data[inner].shape)
    h = 1.0 / (n - 1)
    nodes, _ = api.serialize(cm.ftcs_expr(cm.Leaf("u"), cfl * h * h, D))
    orc.assign(u, nodes, [u])  # warm
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.assign(u, nodes, [u])
    dt = time.perf_counter() - t0
    pts = (n - 2) ** D * reps
    return pts / dt / 1e9, "%s: %d^%d nodes x %d steps on %d host threads (oracle port, %.1f s)" % (workload, n, D, reps, used, dt), used


def cpu_weno_sample(threads, lines=16384, reps=1):
    """The oracle's three WENO5-RK3 stage assignments (the reference's operation order) on a bounded
    sample of the workload: `lines` periodic lines of 4096 cells with the benchmark's pulses, `reps` RK3
    steps, on all host threads; returns (G cell-updates per RK3 step / s, sample description, threads)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import common as cm
    import oracle_lib as orc
    from opflow_gb300 import _capi as capi
    from opflow_gb300 import api
    used = orc.lib().or_set_threads(threads)
    nx = 4096
    mesh = cm.mesh_uniform([nx + 1, lines + 1])
    fd = cm.field_desc(2, capi.CENTER, [(capi.BC_PERIODIC, capi.BC_PERIODIC)] * 2, ext=3)
    h0 = orc.HostField(mesh, fd)
    rng = h0.assignable()
    h0.data[h0.slices(rng)] = wl.weno_u0(2024, nx, lines)
    h0.update_padding()
    h1 = orc.HostField(mesh, fd, data=h0.data.copy())
    h2 = orc.HostField(mesh, fd, data=h0.data.copy())
    L = [cm.Leaf("u"), cm.Leaf("u1"), cm.Leaf("u2")]
    ns = [api.serialize(x, L)[0] for x in cm.weno_stage_exprs(L[0], L[1], L[2], 0.5 / nx)]
    t0 = time.perf_counter()
    for _ in range(reps):
        orc.assign(h1, ns[0], [h0, h1, h2])
        orc.assign(h2, ns[1], [h0, h1, h2])
        orc.assign(h0, ns[2], [h0, h1, h2])
    dt = time.perf_counter() - t0
    return (nx * lines * reps / dt / 1e9,
            "weno: %d lines x 4096 cells x %d RK3 step(s) on %d host threads (oracle port of the three stage assignments, %.1f s)"
            % (lines, reps, used, dt), used)


def served_population(reqs):
    """Every linear system a served window solves: a one-shot request once, a session once per step
    (each step re-solves the session's operator with a new right-hand side)."""
    out = []
    for p, f, steps in reqs:
        out.extend([(p, f, steps)] * steps)
    return out


def reference_requests(args):
    """The systems of the workload in problem form, as (problem, f, steps), without a GPU."""
    from opflow_gb300 import api
    if args.workload == "serve":
        return served_population(wl.serve_mix(api, 77, args.requests))
    if args.workload == "batched":
        return [(p, f, 1) for p, f in wl.batched_problems(api, 99, args.problems)]
    if args.workload == "poisson2d":
        n = args.grid or 2048
        v = np.random.default_rng(1234).standard_normal((n, n))
        return [(wl.poisson_problem(api, n, 2, api.BCType.Neum), (v - v.mean()).reshape(-1), 1)]
    raise SystemExit("the reference arm restates problem-form systems only (serve, batched, poisson2d)")


def run_reference_solves(args, threads):
    """The reference's CPU path for the solve workloads: every timed step solves one system of the
    workload's window, picked by systematic sampling over the window sorted by size (so --steps K
    systems cover its size distribution), with the restated HYPRE PCG + PFMG on all host threads,
    assembly and set-up included as in HYPREEqnSolveHandler::solve.  value = systems / total seconds."""
    reqs = reference_requests(args)  # the served window's systems, session steps included
    # warm-up: the smallest systems (page in the oracle, the thread pool)
    small = sorted(reqs, key=lambda r: int(np.prod(r[0].n)))[:max(1, args.warmup)]
    cpu_pfmg_sample(small, len(small), threads)
    v, secs, its, used, desc = cpu_pfmg_sample(reqs, max(1, args.steps), threads)
    one, _, _, _, desc1 = cpu_pfmg_sample(reqs, 3, 1)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "requests": len(reqs), "sample": desc, "iterations": its,
                       "seconds_per_system": secs, "one_core": {"value": one, "unit": "solves/s", "sample": desc1},
                       "unit_is": "one linear system solved to ||b-Ax||/||b|| <= 1e-10 (a one-shot request or one session step)",
                       "note": "the reference (OpFlow + vendored HYPRE) is not built on this host; its PCG + PFMG is restated by the "
                               "oracle, which reproduces HYPRE's iteration counts and residuals on the committed fixtures"},
            "cpu_baseline": {"value": v, "unit": "solves/s", "cores": used, "kind": "port", "sample": desc},
            "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    if args.workload in SOLVE_WORKLOADS:
        return run_reference_solves(args, threads)
    if args.workload == "weno":
        vals = []
        for _ in range(max(1, min(args.steps, 3))):
            v, sample, used = cpu_weno_sample(threads)
            vals.append(v)
        value = statistics.median(vals)
        line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "Gpts/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "config": {"workload": "weno", "sample": sample},
                "cpu_baseline": {"value": value, "unit": "Gpts/s", "cores": used, "kind": "port", "sample": sample},
                "e2e": {"value": value, "unit": "Gpts/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return 0
    vals = []
    sample = ""
    for _ in range(args.warmup):
        cpu_ftcs_sample(args.workload, threads, 1)
    for _ in range(args.steps):
        v, sample, used = cpu_ftcs_sample(args.workload, threads, 2)
        vals.append(v)
    value = statistics.median(vals)
    cfg = workload_cfg(args.workload)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "GLUP/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "GLUP/s", "cores": used, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "GLUP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------------------ solves
SOLVE_WORKLOADS = ("poisson2d", "serve", "batched", "poisson3d")


def iter_bytes_per_cell(ndim, precision="mixed", var_coef=False):
    """Algorithmic bytes per level-0 cell and flexible-PCG iteration (the measurement table's figures):
    the float64 Krylov step (SpMV 16 B, vector updates 56 B, dot products 16 B: ~100 B with the
    preconditioned-vector read) plus one V-cycle at the level precision, (4/3 in 2D, 8/7 in 3D) x
    (smoother 2 x (16 + 8) + residual 24 + restriction 10 + prolongation 16 = 98 B at float64, half at
    float32).  Variable coefficients add the (2 ndim + 1) coefficient arrays read by the float64 SpMV
    and by the two level-0 smoother sweeps at the level precision, over the hierarchy."""
    h = 4.0 / 3.0 if ndim == 2 else 8.0 / 7.0
    lvl = 0.5 if precision == "mixed" else 1.0
    b = 100.0 + h * 98.0 * lvl
    if var_coef:
        b += (2 * ndim + 1) * (8.0 + 2 * 8.0 * lvl * h)
    return b


def cpu_pfmg_sample(reqs, nsample, threads, order_key=None):
    """The reference's CPU solve restated (oracle: assembly as in HYPREEqnSolveHandler::generateAb, then
    HYPRE PCG + PFMG with one V-cycle per iteration, two-norm test at 1e-10) on a systematic sample of
    the window's linear systems: sorted by size, every (len/nsample)-th, so the sample covers the
    window's size distribution.  One-shot requests are timed with their assembly and set-up (a fresh
    handler's solve()); a session's step without the matrix assembly (staticMat: generateb + setup +
    solve), the b generation left out.  Returns (solves/s, per-system seconds, iterations, threads, desc)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    import common as cm
    import oracle_lib as orc
    from opflow_gb300 import api
    used = orc.lib().or_set_threads(threads)
    order = sorted(range(len(reqs)), key=lambda i: int(np.prod(reqs[i][0].n)))
    idx = [order[min(len(order) - 1, int((k + 0.5) * len(order) / nsample))] for k in range(nsample)]
    secs, its = [], []
    for i in idx:
        p, f, steps = reqs[i]
        pin = p.alpha == 0.0 and p.bc == api.BCType.Neum
        t0 = time.perf_counter()
        dims, off, coef, rhs = cm.problem_system(p, np.asarray(f), pin)
        t1 = time.perf_counter()
        x, it, rel, nl = orc.pfmg_pcg(dims, off, coef, rhs, tol=1e-10, maxit=200, cycles=1, threads=used)
        t2 = time.perf_counter()
        if rel > 1e-10:
            raise RuntimeError("restated PCG+PFMG did not reach 1e-10 on system %d (%g)" % (i, rel))
        secs.append((t2 - t0) if steps == 1 else (t2 - t1))
        its.append(it)
    desc = ("restated HYPRE PCG+PFMG(1 V-cycle), tol 1e-10 two-norm, incl. assembly + setup per one-shot solve (setup + solve per "
            "session step); %d of the window's %d systems sampled by size (%s unknowns), %d host threads" %
            (nsample, len(reqs), ",".join(str(int(np.prod(reqs[i][0].n))) for i in idx), used))
    return nsample / sum(secs), secs, its, used, desc


def run_poisson2d(args, torch, api, capi, np, ctx, stream, world, rank, local):
    n = args.grid or 2048
    mesh = api.MeshBuilder().newMesh(n + 1, n + 1).setMeshOfDim(0, 0., 1.).setMeshOfDim(1, 0., 1.).build()
    b = api.ExprBuilder().setMesh(mesh).setLoc(api.LocOnMesh.Center).setExt(1)
    for d in range(2):
        b.setBC(d, api.DimPos.start, api.BCType.Neum, 0.).setBC(d, api.DimPos.end, api.BCType.Neum, 0.)
    p = b.build(ctx)
    f = b.build(ctx)
    a = f.download()
    sl = f.index_slices(f.assignableRange)
    rng = np.random.default_rng(1234 + rank)
    v = rng.standard_normal(a[sl].shape)
    a[sl] = v - v.mean()
    f.upload(a)
    getter = lambda e: f == api.d2x(e) + api.d2y(e)
    out = {}
    for prec in ("mixed", "fp64"):
        h = api.makeEqnSolveHandler(getter, p, api.StructSolverParams(tol=1e-10, maxIter=200, pinValue=True, staticMat=True,
                                                                        precision=prec, zeroGuess=True, preSweeps=args.sweeps,
                                                                        postSweeps=args.sweeps))
        for _ in range(args.warmup):
            st = h.solve()
        torch.cuda.synchronize()
        l0 = capi.launch_count()
        t0 = time.perf_counter()
        its, rels = [], []
        for _ in range(args.steps):
            st = h.solve()
            its.append(st.niter)
            rels.append(st.relerr)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out[prec] = dict(solves_per_s=args.steps / dt, ms_per_solve=dt / args.steps * 1e3, iterations=its[-1], rel_residual=max(rels),
                         launches=capi.launch_count() - l0)
        h.close()
    # end-to-end: host f in (upload), solve, host solution out (download)
    h = api.makeEqnSolveHandler(getter, p, api.StructSolverParams(tol=1e-10, maxIter=200, pinValue=True, staticMat=True,
                                                                    precision="mixed", zeroGuess=True))
    h.solve()
    host = a.copy()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 5))
    for _ in range(e2e_steps):
        f.upload(host)
        h.solve()
        _ = p.download()
    e2e = e2e_steps / (time.perf_counter() - t0)
    h.close()
    N = n * n
    m = out["mixed"]
    bpc = iter_bytes_per_cell(2, "mixed")
    achieved = bpc * N * m["iterations"] / (m["ms_per_solve"] * 1e-3) / 1e9
    peak, src = peak_hbm()
    return dict(value=m["solves_per_s"], unit="solves/s", ms=m["ms_per_solve"], launches=m["launches"], dtype="f64 outer / f32 V-cycle",
                config=dict(workload="poisson2d", grid=[n, n], loc="cell", bc="neumann 0, pinned", rhs="N(0,1) zero mean", tol=1e-10,
                            mixed=m, fp64=out["fp64"], mixed_over_fp64=m["solves_per_s"] / out["fp64"]["solves_per_s"],
                            l2="level-0 vectors 33.5 MB each; the solve streams several of them per iteration (> L2)"),
                roofline={"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": src,
                          "traffic": traffic_for("poisson2d"), "kernel": "flexible-PCG iteration (graph: FP32 V-cycle + FP64 Krylov)",
                          "algorithmic_bytes_per_launch": bpc * N * m["iterations"], "bytes_per_cell_iteration": bpc},
                e2e={"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": a.nbytes, "d2h_bytes_per_step": a.nbytes, "steps": e2e_steps})


def run_batched(args, torch, api, capi, np, ctx, stream, world, rank, local):
    count = args.problems
    probs = wl.batched_problems(api, 99 + rank, count)
    mixed = api.StructSolverParams(tol=1e-10, maxIter=200, precision="mixed", zeroGuess=True)
    B = api.Batch([p for p, _ in probs], mixed, ctx)
    for i, (_, f) in enumerate(probs):
        B.set(i, f)
    for _ in range(args.warmup):
        B.solve()
    torch.cuda.synchronize()
    l0 = capi.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        st = B.solve()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    launches = capi.launch_count() - l0
    iters = [s.niter for s in st]
    worst = max(s.relerr for s in st)
    ok = sum(1 for s in st if s.converged)
    # end to end: host f in, batched solve, every solution back to the host
    t0 = time.perf_counter()
    xs = []
    for i, (_, f) in enumerate(probs):
        B.set(i, f)
    B.solve()
    for i in range(count):
        xs.append(B.get(i))
    e2e_s = time.perf_counter() - t0
    B.close()
    # the same problems one at a time, plain FP64 (a loop of per-problem solves)
    plain = api.StructSolverParams(tol=1e-10, maxIter=200, precision="fp64", zeroGuess=True)
    nloop = min(count, args.loop_sample)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p, f in probs[:nloop]:
        b1 = api.Batch([p], plain, ctx)
        b1.set(0, f)
        b1.solve()
        b1.close()
    torch.cuda.synchronize()
    loop_rate = nloop / (time.perf_counter() - t0)
    cells = sum(int(np.prod([n - 2 for n in p.n])) for p, _ in probs)
    bytes_per_solve = sum(iter_bytes_per_cell(2, "mixed") * int(np.prod([n - 2 for n in p.n])) * it for (p, _), it in zip(probs, iters))
    peak, src = peak_hbm()
    achieved = bytes_per_solve / (ms * 1e-3) / 1e9
    hb = 8 * sum(f.size for _, f in probs)
    return dict(value=count / (ms * 1e-3), unit="solves/s", ms=ms, launches=launches, dtype="f64 outer / f32 V-cycle",
                config=dict(workload="batched", problems=count, operator="(I - k Lap) u = f, corner nodes, Dirichlet 0",
                            k="LogU[1e-4,1]", side="LogU[65,1025] rounded to 2^m+1", unknowns=cells, tol=1e-10, converged=ok,
                            worst_rel_residual=worst, iterations_min=min(iters), iterations_max=max(iters),
                            plain_fp64_loop_solves_per_s=loop_rate, plain_fp64_loop_sample=nloop,
                            batched_over_plain_loop=(count / (ms * 1e-3)) / loop_rate,
                            l2="%.1f GB of level-0 vectors, streamed per iteration (> L2)" % (cells * 48 / 1e9)),
                roofline={"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": src,
                          "traffic": traffic_for("batched"), "kernel": "batched flexible-PCG solve (whole-solve graph)",
                          "algorithmic_bytes_per_launch": bytes_per_solve},
                e2e={"value": count / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": hb, "d2h_bytes_per_step": hb})


def run_poisson3d(args, torch, api, capi, np, ctx, stream, world, rank, local):
    """3D 7-point variable-coefficient Poisson: div(K grad p) = f with K = exp(g) interpolated to faces."""
    n = args.grid or 256
    mesh = api.MeshBuilder().newMesh(n + 1, n + 1, n + 1)
    for d in range(3):
        mesh.setMeshOfDim(d, 0.0, 1.0)
    mesh = mesh.build()
    b = api.ExprBuilder().setMesh(mesh).setLoc(api.LocOnMesh.Center).setExt(1)
    for d in range(3):
        b.setBC(d, api.DimPos.start, api.BCType.Neum, 0.).setBC(d, api.DimPos.end, api.BCType.Neum, 0.)
    p, f, K = b.build(ctx), b.build(ctx), b.build(ctx)
    rng = np.random.default_rng(4321 + rank)
    kk = K.download()
    sl = K.index_slices(K.assignableRange)
    kk[sl] = np.exp(wl.smooth_field(rng, n))
    K.upload(kk)
    ff = f.download()
    v = rng.standard_normal(ff[sl].shape)
    ff[sl] = v - v.mean()
    f.upload(ff)
    getter = lambda e: f == (api.dx(api.d1IntpCenterToCorner(K, 0) * api.dx(e)) + api.dy(api.d1IntpCenterToCorner(K, 1) * api.dy(e))
                             + api.dz(api.d1IntpCenterToCorner(K, 2) * api.dz(e)))
    if args.const_coef:
        getter = lambda e: f == api.d2x(e) + api.d2y(e) + api.d2z(e)
    out = {}
    for prec in ("mixed", "fp64"):
        h = api.makeEqnSolveHandler(getter, p, api.StructSolverParams(tol=1e-10, maxIter=300, pinValue=True, staticMat=True,
                                                                        precision=prec, zeroGuess=True))
        for _ in range(args.warmup):
            st = h.solve()
        torch.cuda.synchronize()
        l0 = capi.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            st = h.solve()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        out[prec] = dict(solves_per_s=1e3 / ms, ms_per_solve=ms, iterations=st.niter, rel_residual=st.relerr, launches=capi.launch_count() - l0)
        h.close()
    host = ff.copy()
    h = api.makeEqnSolveHandler(getter, p, api.StructSolverParams(tol=1e-10, maxIter=300, pinValue=True, staticMat=True,
                                                                    precision="mixed", zeroGuess=True))
    h.solve()
    t0 = time.perf_counter()
    for _ in range(2):
        f.upload(host)
        h.solve()
        _ = p.download()
    e2e = 2 / (time.perf_counter() - t0)
    h.close()
    m = out["mixed"]
    N = n ** 3
    bpc = iter_bytes_per_cell(3, "mixed", var_coef=not args.const_coef)
    achieved = bpc * N * m["iterations"] / (m["ms_per_solve"] * 1e-3) / 1e9
    peak, src = peak_hbm()
    return dict(value=m["solves_per_s"], unit="solves/s", ms=m["ms_per_solve"], launches=m["launches"], dtype="f64 outer / f32 V-cycle",
                config=dict(workload="poisson3d", grid=[n, n, n], loc="cell", bc="neumann 0, pinned",
                            coefficient="1 (d2x + d2y + d2z)" if args.const_coef else "exp(g), g smooth seeded Fourier field of std 1, interpolated to faces",
                            tol=1e-10,
                            mixed=m, fp64=out["fp64"], mixed_over_fp64=m["solves_per_s"] / out["fp64"]["solves_per_s"],
                            l2="level-0 vectors %.0f MB each (> L2)" % (N * 8 / 1e6)),
                roofline={"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": src,
                          "traffic": traffic_for("poisson3d"), "kernel": "flexible-PCG iteration (whole-solve graph)",
                          "algorithmic_bytes_per_launch": bpc * N * m["iterations"], "bytes_per_cell_iteration": bpc},
                e2e={"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": ff.nbytes, "d2h_bytes_per_step": ff.nbytes, "steps": 2})


def run_serve(args, torch, api, capi, np, ctx, stream, world, rank, local):
    """The serving configuration.  One unit throughout is a linear system solved to 1e-10: a one-shot
    request or one backward-Euler step of a session.  A window of --requests requests (Poisson
    arrivals) is served by the request server (continuous batching, mixed precision):

    value: the window served with right-hand sides and result buffers already in HBM (device tensors),
           at the highest swept arrival rate; the window is one continuous run, timed as --steps
           consecutive steps (step k ends when the k-th group of requests, in submission order, has
           its results: CUDA events on the caller's stream), value = systems / total time;
    e2e:   the same window and rate with host right-hand sides in and host solutions out (pinned);
    next to plain FP64 serving one request at a time on the same window (host buffers)."""
    count = args.requests
    rates = [float(r) for r in str(args.rate).split(",")]
    params = api.StructSolverParams(tol=1e-10, maxIter=200, precision="mixed", zeroGuess=True)
    reqs = wl.serve_mix(api, 77 + rank, count)
    total_systems = sum(s for _, _, s in reqs)
    peak, src = peak_hbm()

    # the window's distinct systems (one per request) in one batched solve, inputs resident: the kernel
    # time of the solver itself, against the roofline
    B = api.Batch([p for p, _, _ in reqs], params, ctx)
    for i, (_, f, _) in enumerate(reqs):
        B.set(i, f)
    B.solve()
    torch.cuda.synchronize()
    bms = []
    for _ in range(max(1, min(args.steps, 3))):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = B.solve()
        e1.record(stream)
        torch.cuda.synchronize()
        bms.append(e0.elapsed_time(e1))
    iters = [s_.niter for s_ in st]
    worst = max(s_.relerr for s_ in st)
    B.close()
    batch_ms = statistics.median(bms)
    alg = sum(iter_bytes_per_cell(len(p.n), "mixed") * int(np.prod(p.n)) * it for (p, _, _), it in zip(reqs, iters))
    achieved = alg / (batch_ms * 1e-3) / 1e9

    def pinned(n):
        return torch.empty(n, dtype=torch.float64, pin_memory=True).numpy()

    dev = torch.device("cuda", local)
    host_in, host_out, dev_in, dev_out = [], [], [], []
    for _, f, _ in reqs:
        hb = pinned(f.size)
        hb[:] = f
        host_in.append(hb)
        host_out.append(pinned(f.size))
        dev_in.append(torch.from_numpy(f).to(dev))
        dev_out.append(torch.empty(f.size, dtype=torch.float64, device=dev))
    torch.cuda.synchronize()

    def served(prec, max_active, rate, fin, fout, nsteps=1, rq=None):
        rq = rq if rq is not None else [(p, f, s_) for (p, _, s_), f in zip(reqs, fin)]
        srv = api.Server(api.StructSolverParams(tol=1e-10, maxIter=200, precision=prec), hbm_budget=120 << 30,
                         max_active=max_active, ctx=ctx)
        rng = np.random.default_rng(5)
        gaps = rng.exponential(1.0 / rate, len(rq))
        ids = []
        l0 = capi.launch_count()
        torch.cuda.synchronize()
        evs = [torch.cuda.Event(enable_timing=True)]
        evs[0].record(stream)
        t0 = time.perf_counter()
        tnext = t0
        for k, ((p, f, steps), g) in enumerate(zip(rq, gaps)):
            tnext += g
            while time.perf_counter() < tnext:
                time.sleep(min(0.0005, max(0.0, tnext - time.perf_counter())))
            ids.append(srv.submit(p, f, steps=steps, out=fout[k] if fout is not None else np.zeros(np.size(f))))
        res = []
        bounds = [int(round((g + 1) * len(ids) / nsteps)) for g in range(nsteps)]
        for k, i in enumerate(ids):
            res.append(srv.result(i))
            if k + 1 in bounds:
                ev = torch.cuda.Event(enable_timing=True)
                ev.record(stream)
                evs.append(ev)
        wall = time.perf_counter() - t0
        torch.cuda.synchronize()
        launches = capi.launch_count() - l0
        step_ms = [evs[k].elapsed_time(evs[k + 1]) for k in range(len(evs) - 1)]
        st = srv.stats()
        srv.close()
        ok = sum(1 for r in res if r["status"] == capi.OK)
        lat = sorted(r["latency_ms"] for r in res)
        q = lambda z: lat[min(len(lat) - 1, int(np.ceil(z * len(lat))) - 1)]
        systems = sum(r["solves"] for r in res)
        tot_ms = sum(step_ms)
        return dict(solves_per_s=systems / (tot_ms * 1e-3), p50_ms=q(0.5), p99_ms=q(0.99), ok=ok, n=len(res), systems=systems,
                    iterations=sum(r["iterations"] for r in res), max_active_seen=st["max_active_seen"], wall_s=wall,
                    event_s=tot_ms * 1e-3, step_ms=step_ms, launches=launches, compositions=st["compositions"],
                    worker_s={k: round(st[k], 4) for k in ("setup_s", "compose_s", "iterate_s", "retire_s")})

    # warm-up (allocator pool, graphs, kernels)
    for _ in range(max(1, min(args.warmup, 2))):
        served("mixed", 16, 1000.0, None, None, rq=wl.serve_mix(api, 3, 6))
    served("fp64", 1, 1000.0, None, None, rq=wl.serve_mix(api, 3, 2))
    head_rate = max(rates)
    with ClockSampler(local) as clk:
        dres = served("mixed", 64, head_rate, dev_in, dev_out, nsteps=args.steps)
    sweep = []
    for rate in rates:
        sweep.append(dict(rate_per_s=rate, served_mixed=served("mixed", 64, rate, host_in, host_out)))
    head = [w for w in sweep if w["rate_per_s"] == head_rate][0]
    plain = served("fp64", 1, head_rate, host_in, host_out)
    head["served_plain_fp64_one_at_a_time"] = plain
    head["served_speedup"] = head["served_mixed"]["solves_per_s"] / plain["solves_per_s"]
    head["p99_ratio_mixed_over_plain"] = head["served_mixed"]["p99_ms"] / plain["p99_ms"]
    mixed = head["served_mixed"]
    hb = 8 * sum(f.size for _, f, _ in reqs)
    value = dres["solves_per_s"]
    return dict(value=value, unit="solves/s", ms=statistics.mean(dres["step_ms"]), launches=dres["launches"], clocks=clk.summary(),
                dtype="f64 outer / f32 V-cycle",
                config=dict(workload="serve", requests=count, rates_per_s=rates,
                            mix="70% one-shot Poisson (2D side LogU[129,2049] / 3D side LogU[64,256], Neumann/Dirichlet 50/50), "
                                "30% heat sessions of 10-100 backward-Euler steps (2D side LogU[129,1025])",
                            unit_is="one linear system solved to ||b-Ax||/||b|| <= 1e-10 (a one-shot request or one session step)",
                            systems_in_window=total_systems, budget_gb=120, headline_rate_per_s=head_rate,
                            value_is="the window served at %g req/s with device-resident f and x (one continuous run timed as %d steps "
                                     "of consecutive request groups)" % (head_rate, args.steps),
                            device_resident_served=dres, sweep=sweep,
                            served_speedup=head["served_speedup"], p99_ratio_mixed_over_plain=head["p99_ratio_mixed_over_plain"],
                            device_resident_batch=dict(systems=len(reqs), unknowns=int(sum(int(np.prod(p.n)) for p, _, _ in reqs)),
                                                       ms_median=batch_ms, ms_all=bms, iterations_min=min(iters), iterations_max=max(iters),
                                                       worst_rel_residual=worst,
                                                       what="one batched mixed-precision solve of the window's distinct systems (one per request)"),
                            e2e_is="the same window served at %g req/s with pinned host f in and host x out" % head_rate,
                            l2="%.1f GB of level-0 vectors per batched solve (> L2): no flush needed" % (
                                sum(int(np.prod(p.n)) for p, _, _ in reqs) * 48 / 1e9)),
                roofline={"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": src,
                          "traffic": traffic_for("serve"),
                          "kernel": "batched flexible-PCG solve of the window's distinct systems (FP32 V-cycle + FP64 Krylov kernels)",
                          "algorithmic_bytes_per_launch": alg, "launch_ms": batch_ms,
                          "bytes_per_cell_iteration": {"2d": iter_bytes_per_cell(2), "3d": iter_bytes_per_cell(3)}},
                e2e={"value": mixed["solves_per_s"], "unit": "solves/s", "h2d_bytes_per_step": hb, "d2h_bytes_per_step": hb,
                     "p50_ms": mixed["p50_ms"], "p99_ms": mixed["p99_ms"], "note": "bytes per window (all requests' f and x)"},
                reqs=reqs)


def explicit_record(torch, api, capi, np, ctx, stream, local, rank, steps=20, warmup=3, ftcs_steps=200):
    """Path E measured beside the default (solve) line: the 512^3 FTCS3D configuration (fixed-point
    mode over the configuration's 200 steps, and the bit-exact IEEE mode over a tenth of `steps`) and
    WENO5-RK3 on 65536 x 4096 periodic lines, each timed with CUDA events on the launching stream after
    `warmup`, with its own clock record."""
    out = {}
    peak, src = peak_hbm()
    n = 512
    mesh = api.MeshBuilder().newMesh(n, n, n)
    for d in range(3):
        mesh.setMeshOfDim(d, 0.0, 1.0)
    mesh = mesh.build()
    b = api.ExprBuilder().setMesh(mesh).setName("u").setLoc(api.LocOnMesh.Corner)
    for d in range(3):
        b.setBC(d, api.DimPos.start, api.BCType.Dirc, 0.0).setBC(d, api.DimPos.end, api.BCType.Dirc, 0.0)
    u = b.build(ctx)
    u0 = gaussians_u0(torch, n, 1234 + rank, torch.device("cuda", local)).cpu().numpy()
    host = u.download()
    host[...] = u0
    u.upload(host)
    h = 1.0 / (n - 1)
    expr = u + (0.1 * h * h) * (api.d2x(u) + api.d2y(u) + api.d2z(u))
    pts = (n - 2) ** 3
    for mode, k in (("fast", ftcs_steps), ("exact", max(2, steps // 10))):
        u.assign(expr, mode=mode, steps=warmup)
        torch.cuda.synchronize()
        l0 = capi.launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            ev0.record(stream)
            u.assign(expr, mode=mode, steps=k)
            ev1.record(stream)
            torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / k
        glups = pts / (ms * 1e-3) / 1e9
        out["ftcs3d_512_" + mode] = {"glup_per_s": glups, "ms_per_step": ms, "steps": k, "launches": capi.launch_count() - l0,
                                     "achieved_gbs": 16.0 * glups, "frac": 16.0 * glups / peak, "peak": peak, "peak_source": src,
                                     "bytes_per_update": 16, "clocks": clk.summary()}
    del u
    nx, ny = 4096, 65536
    mesh = api.MeshBuilder().newMesh(nx + 1, ny + 1).setMeshOfDim(0, 0.0, 1.0).setMeshOfDim(1, 0.0, ny / nx).build()
    b = api.ExprBuilder().setMesh(mesh).setName("u").setLoc(api.LocOnMesh.Center).setExt(3)
    for d in range(2):
        b.setBC(d, api.DimPos.start, api.BCType.Periodic, 0.0).setBC(d, api.DimPos.end, api.BCType.Periodic, 0.0)
    w = b.build(ctx)
    host = w.download()
    host[w.index_slices(w.assignableRange)] = wl.weno_u0(2024 + rank, nx, ny)
    w.upload(host)
    del host
    dt = 0.5 / nx
    for mode, k in (("exact", max(2, steps // 4)), ("fast", max(2, steps // 2))):
        m = capi.EVAL_FAST if mode == "fast" else capi.EVAL_EXACT
        api.weno_rk3(w, dt, warmup, mode=m)
        torch.cuda.synchronize()
        l0 = capi.launch_count()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            ev0.record(stream)
            api.weno_rk3(w, dt, k, mode=m)
            ev1.record(stream)
            torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / k
        rate = nx * ny / (ms * 1e-3) / 1e9
        out["weno_65536x4096_" + mode] = {"gpts_per_s": rate, "ms_per_rk3_step": ms, "steps": k, "launches": capi.launch_count() - l0,
                                          "achieved_gbs": 16.0 * rate, "frac": 16.0 * rate / peak, "bytes_per_point_rk3_step": 16,
                                          "bound": "float64 issue", "clocks": clk.summary()}
    del w
    return out


# ------------------------------------------------------------------------------------------- ours
def run_weno(args, torch, api, capi, np, ctx, stream, world, rank, local, dist):
    """WENO5-JS + Shu-Osher RK3 advection on 65536 periodic lines of 4096 cells (square and cosine
    pulses, dt = 0.5 h): one bench step is one RK3 step of every line (opflow_weno_rk3_mode, all stages
    in shared memory).  `value` runs `--steps` steps in one launch with the field resident; `e2e` uploads
    the field from pinned host memory, takes one RK3 step and downloads it, per step."""
    nx, ny = 4096, args.lines or 65536
    mesh = api.MeshBuilder().newMesh(nx + 1, ny + 1).setMeshOfDim(0, 0.0, 1.0).setMeshOfDim(1, 0.0, ny / nx).build()
    b = api.ExprBuilder().setMesh(mesh).setName("u").setLoc(api.LocOnMesh.Center).setExt(3)
    for d in range(2):
        b.setBC(d, api.DimPos.start, api.BCType.Periodic, 0.0).setBC(d, api.DimPos.end, api.BCType.Periodic, 0.0)
    w = b.build(ctx)
    a = w.download()
    a[w.index_slices(w.assignableRange)] = wl.weno_u0(2024 + rank, nx, ny)
    host = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
    host.numpy()[:] = a.reshape(-1)
    del a
    cnt = host.numel()
    P = C.POINTER(C.c_double)
    L = capi.lib()
    capi.check(L.opflow_field_upload(w.handle, C.cast(host.data_ptr(), P), cnt))
    dt = 0.5 / nx
    m = capi.EVAL_FAST if args.mode == "fast" else capi.EVAL_EXACT
    api.weno_rk3(w, dt, max(3, args.warmup), mode=m)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    l0 = capi.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        api.weno_rk3(w, dt, args.steps, mode=m)
        ev1.record(stream)
        torch.cuda.synchronize()
    launches = capi.launch_count() - l0
    ms = ev0.elapsed_time(ev1)
    if world > 1:
        dist.barrier()
    ms = replica_max(ms, world, dist, torch.device("cuda", local))
    pts = nx * ny
    value = pts * args.steps * world / (ms * 1e-3) / 1e9
    # end to end: upload, one RK3 step, download, per step
    e2e_steps = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        capi.check(L.opflow_field_upload(w.handle, C.cast(host.data_ptr(), P), cnt))
        api.weno_rk3(w, dt, 1, mode=m)
        capi.check(L.opflow_field_download(w.handle, C.cast(host.data_ptr(), P), cnt))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3)
    peak, peak_src = peak_hbm()
    ms_step = ms / args.steps
    achieved = 16.0 * pts / (ms_step * 1e-3) / 1e9
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            v, sample, used = cpu_weno_sample(os.cpu_count() or 1)
            cpu = {"value": v, "unit": "Gpts/s", "cores": used, "kind": "port", "sample": sample}
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "Gpts/s", "cores": 0, "kind": "port", "sample": "failed: %s" % ex}
    line = {"metric": METRIC, "value": value, "unit": "Gpts/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "weno", "lines": ny, "cells_per_line": nx, "mode": args.mode, "dt": "0.5 h", "init": "seeded square + cosine pulses",
                       "l2": "field 2.1 GB > L2; the run keeps each line in shared memory across its steps",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                         "traffic": traffic_for("weno_" + ("fast" if m == capi.EVAL_FAST else "exact")),
                         "kernel": "weno_rk3_kernel<16, false, %s, 2>" % ("true" if m == capi.EVAL_FAST else "false"),
                         "algorithmic_bytes_per_launch": 16.0 * pts,
                         "note": "float64-issue-bound: HBM carries 16 B per point per launch of --steps RK3 steps"},
            "cpu_baseline": cpu,
            "e2e": {"value": pts * e2e_steps / (e2e_ms * 1e-3) / 1e9, "unit": "Gpts/s", "h2d_bytes_per_step": cnt * 8,
                    "d2h_bytes_per_step": cnt * 8, "steps": e2e_steps},
            "gpu_launches": launches, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_ftcs_batch(args, torch, api, capi, np, ctx, stream, world, rank, local, dist):
    """Explicit steps of many uneven grids in one launch per step: 256 2D node grids of side LogU[65,513]
    (seeded), Dirichlet 0, u = u + 0.2 h^2 (d2x(u) + d2y(u)) in exact mode, batched (opflow_assign_batch)
    next to the same assignments run one grid after another."""
    rng = np.random.default_rng(4242 + rank)
    sides = [int(round(np.exp(rng.uniform(np.log(65), np.log(513))))) for _ in range(256)]
    fields, exprs, hosts = [], [], []
    for k, n in enumerate(sides):
        mesh = api.MeshBuilder().newMesh(n, n).setMeshOfDim(0, 0.0, 1.0).setMeshOfDim(1, 0.0, 1.0).build()
        b = api.ExprBuilder().setMesh(mesh).setName("u%d" % k).setLoc(api.LocOnMesh.Corner)
        for d in range(2):
            b.setBC(d, api.DimPos.start, api.BCType.Dirc, 0.0).setBC(d, api.DimPos.end, api.BCType.Dirc, 0.0)
        u = b.build(ctx)
        a = u.download()
        a[...] = 0.0
        sl = u.index_slices([tuple(u.info.assignable[d]) for d in range(2)])
        a[sl] = rng.random(a[sl].shape)
        u.upload(a)
        host = torch.empty(a.size, dtype=torch.float64, pin_memory=True)
        host.numpy()[:] = a.reshape(-1)
        hosts.append(host)
        h = 1.0 / (n - 1)
        fields.append(u)
        exprs.append(u + 0.2 * h * h * (api.d2x(u) + api.d2y(u)))
    pts = sum((n - 2) ** 2 for n in sides)
    pairs = list(zip(fields, exprs))
    api.assign_batch(pairs, steps=max(1, args.warmup))
    for u, e in pairs:
        u.assign(e, mode="exact", steps=1)
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    launches0 = capi.launch_count()
    with ClockSampler(local) as clk:
        ev[0].record(stream)
        api.assign_batch(pairs, steps=args.steps)
        ev[1].record(stream)
        torch.cuda.synchronize()
    launches = capi.launch_count() - launches0
    ms = ev[0].elapsed_time(ev[1])
    ev[2].record(stream)
    for u, e in pairs:
        u.assign(e, mode="exact", steps=args.steps)
    ev[3].record(stream)
    torch.cuda.synchronize()
    ms_loop = ev[2].elapsed_time(ev[3])
    value = pts * args.steps / (ms * 1e-3) / 1e9
    # end to end with host buffers: every field uploaded, one batched step, every field downloaded
    P = C.POINTER(C.c_double)
    L = capi.lib()
    e2e_steps = max(1, min(args.steps, 5))
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        for u, host in zip(fields, hosts):
            capi.check(L.opflow_field_upload(u.handle, C.cast(host.data_ptr(), P), host.numel()))
        api.assign_batch(pairs, steps=1)
        for u, host in zip(fields, hosts):
            capi.check(L.opflow_field_download(u.handle, C.cast(host.data_ptr(), P), host.numel()))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3)
    nbytes = sum(h.numel() for h in hosts) * 8
    peak, peak_src = peak_hbm()
    achieved = 16.0 * pts / (ms / args.steps * 1e-3) / 1e9
    line = {"metric": METRIC, "value": value, "unit": "GLUP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "ftcs_batch", "grids": len(sides), "side": "LogU[65,513] nodes", "points": pts, "mode": "exact",
                       "one_grid_at_a_time_glups": pts * args.steps / (ms_loop * 1e-3) / 1e9, "batched_over_loop": ms_loop / ms,
                       "l2": "%.1f MB of fields in total (L2-resident across steps)" % (nbytes / 1e6),
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_src,
                         "traffic": None, "kernel": "interp_batch_kernel (whole step: every grid's tiles from one work queue)",
                         "algorithmic_bytes_per_launch": 16.0 * pts},
            "cpu_baseline": None,
            "e2e": {"value": pts * e2e_steps / (e2e_ms * 1e-3) / 1e9, "unit": "GLUP/s", "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                    "steps": e2e_steps},
            "gpu_launches": launches, "clocks": clk.summary()}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def run_ours(args):
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    from opflow_gb300 import _capi as capi
    from opflow_gb300 import api
    import numpy as np
    ctx = api.Context(local)
    # a stream of its own (not the legacy default stream): kernels and events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)

    if args.workload in SOLVE_WORKLOADS:
        if world > 1:
            dist.barrier()
        with ClockSampler(local) as clk:
            fn = {"poisson2d": run_poisson2d, "serve": run_serve, "batched": run_batched, "poisson3d": run_poisson3d}[args.workload]
            r = fn(args, torch, api, capi, np, ctx, stream, world, rank, local)
        value = r["value"]
        if world > 1:  # every replica does the same work: the slowest rank's rate times N
            value = replica_min(value, world, dist, torch.device("cuda", local)) * world
        cpu = None
        if rank == 0 and not args.no_cpu_baseline and args.workload != "poisson3d":
            try:
                pop = served_population(r["reqs"]) if r.get("reqs") else reference_requests(args)
                v, secs, its, used, desc = cpu_pfmg_sample(pop, 8 if args.workload == "serve" else 2, os.cpu_count() or 1)
                cpu = {"value": v, "unit": "solves/s", "cores": used, "kind": "port", "sample": desc}
            except Exception as ex:
                cpu = {"value": None, "unit": "solves/s", "cores": 0, "kind": "port", "sample": "failed: %s" % ex}
        r.pop("reqs", None)
        if args.workload == "serve" and not args.no_explicit:
            r["config"]["explicit"] = explicit_record(torch, api, capi, np, ctx, stream, local, rank)
        line = {"metric": METRIC, "value": value, "unit": r["unit"], "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": r["dtype"],
                "data": "synthetic", "config": dict(r["config"], parallelism="replicas" if world > 1 else "single"),
                "roofline": r["roofline"], "cpu_baseline": cpu, "e2e": r["e2e"], "gpu_launches": r["launches"],
                "clocks": r.get("clocks") or clk.summary()}
        if rank == 0:
            print(json.dumps(line), flush=True)
        if world > 1:
            dist.destroy_process_group()
        return 0

    if args.workload == "weno":
        return run_weno(args, torch, api, capi, np, ctx, stream, world, rank, local, dist)
    if args.workload == "ftcs_batch":
        return run_ftcs_batch(args, torch, api, capi, np, ctx, stream, world, rank, local, dist)

    cfg = workload_cfg(args.workload)
    if args.grid:
        cfg["grid"] = [args.grid] * len(cfg["grid"])
    D = len(cfg["grid"])
    n = cfg["grid"][0]
    mesh = api.MeshBuilder().newMesh(*cfg["grid"])
    for d in range(D):
        mesh.setMeshOfDim(d, 0.0, 1.0)
    mesh = mesh.build()
    b = api.ExprBuilder().setMesh(mesh).setName("u").setLoc(api.LocOnMesh.Corner)
    for d in range(D):
        b.setBC(d, api.DimPos.start, api.BCType.Dirc, 0.0).setBC(d, api.DimPos.end, api.BCType.Dirc, 0.0)
    u = b.build(ctx)
    dev = torch.device("cuda", local)
    if D == 3:
        u0 = gaussians_u0(torch, n, 1234 + rank, dev)
    else:
        g = torch.Generator(device="cpu").manual_seed(1234 + rank)
        u0 = torch.rand((n, n), generator=g, dtype=torch.float64).to(dev)
        u0[0, :] = u0[-1, :] = 0
        u0[:, 0] = u0[:, -1] = 0
    host = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True)
    host.copy_(u0.cpu())
    cnt = host.numel()
    P = C.POINTER(C.c_double)
    L = capi.lib()
    capi.check(L.opflow_field_upload(u.handle, C.cast(host.data_ptr(), P), cnt))
    u.updatePadding()
    h = 1.0 / (n - 1)
    cfl = 0.1 if D == 3 else 0.2
    s = cfl * h * h * 1.0
    t = api.d2x(u) + api.d2y(u)
    if D == 3:
        t = t + api.d2z(u)
    expr = u + s * t
    mode = args.mode
    pts = (n - 2) ** D

    # warm-up (also builds the plan, the Markstein self-check and the second buffer)
    u.assign(expr, mode=mode, steps=max(1, args.warmup))
    torch.cuda.synchronize()
    launches0 = capi.launch_count()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        u.assign(expr, mode=mode, steps=args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    ms = ev0.elapsed_time(ev1)
    launches = capi.launch_count() - launches0
    ms = replica_max(ms, world, dist, dev)
    ms_step = ms / args.steps
    value = pts * args.steps * world / (ms * 1e-3) / 1e9

    # end-to-end through the C ABI with host buffers: upload, one step, download per step
    e2e_steps = max(1, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        capi.check(L.opflow_field_upload(u.handle, C.cast(host.data_ptr(), P), cnt))
        u.assign(expr, mode=mode, steps=1)
        capi.check(L.opflow_field_download(u.handle, C.cast(host.data_ptr(), P), cnt))
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = max(e0.elapsed_time(e1), (time.perf_counter() - t0) * 1e3)
    e2e_val = pts * e2e_steps * world / (e2e_ms * 1e-3) / 1e9

    peak, peak_src = peak_hbm()
    alg_bytes = 16.0 * pts
    achieved = alg_bytes / (ms_step * 1e-3) / 1e9
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            v, sample, used = cpu_ftcs_sample(args.workload, os.cpu_count() or 1, 2)
            cpu = {"value": v, "unit": "GLUP/s", "cores": used, "kind": "port", "sample": sample}
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "GLUP/s", "cores": 0, "kind": "port", "sample": "failed: %s" % ex}
    line = {
        "metric": METRIC, "value": value, "unit": "GLUP/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if mode == "exact" else "i64 fixed point (f64 storage)", "data": "synthetic",
        "config": dict(cfg, mode=mode, parallelism="replicas" if world > 1 else "single"),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src,
                     "traffic": traffic_for(args.workload + "_" + mode + ("_resident" if D == 3 and mode == "fast" and args.steps >= 2 and
                                                                          os.environ.get("OPFLOW_FX_RESIDENT", "1") != "0" else "")),
                     "kernel": ftcs_kernel_label(D, mode, args.steps),
                     "timed": "whole step (stencil kernel + ghost-padding kernels), CUDA events on the launching stream",
                     "algorithmic_bytes_per_launch": alg_bytes},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": "GLUP/s", "h2d_bytes_per_step": cnt * 8, "d2h_bytes_per_step": cnt * 8,
                "steps": e2e_steps, "ms_per_step": e2e_ms / e2e_steps},
        "gpu_launches": launches,
        "clocks": clk.summary(),
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="serve", choices=["serve", "poisson2d", "poisson3d", "batched", "ftcs3d", "ftcs2d", "weno",
                                                            "ftcs_batch"])
    ap.add_argument("--problems", type=int, default=512, help="batched: problems per batch")
    ap.add_argument("--loop-sample", type=int, default=64, help="batched: problems timed in the plain FP64 one-at-a-time loop")
    ap.add_argument("--requests", type=int, default=500, help="serve: requests per measurement window")
    ap.add_argument("--rate", default="50,200,2000", help="serve: Poisson arrival rates (requests/s), comma-separated; the last is the headline")
    ap.add_argument("--mode", default="fast", choices=["fast", "exact"])
    ap.add_argument("--grid", type=int, default=0, help="override the grid side (profiling a smaller case)")
    ap.add_argument("--lines", type=int, default=0, help="weno: override the number of lines (profiling a smaller case)")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU baseline leg (profiling runs)")
    ap.add_argument("--no-explicit", action="store_true", help="serve: skip the explicit-path record (profiling runs)")
    ap.add_argument("--sweeps", type=int, default=2, help="poisson2d: red-black Gauss-Seidel sweeps before and after each coarsening")
    ap.add_argument("--const-coef", action="store_true", help="poisson3d: constant coefficient (the serving workload's 3D operator)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

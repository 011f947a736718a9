#!/usr/bin/env python3
"""Benchmark of the GB300 engine for OpFlow's hot paths; prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workloads (seeded synthetic inputs with the configurations' shapes and value distributions):
  ftcs3d  7-point FTCS heat update, 512^3 node grid, Dirichlet 0, u0 = 8 seeded Gaussians,
          dt = 0.1 h^2 (one step = one update of the whole grid; GLUP/s)
  ftcs2d  the CPU-runnable FTCS2D case: 1025^2 nodes, Dirichlet 0, u0 ~ U[0,1), dt = 0.2 h^2

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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

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


def workload_cfg(name):
    if name == "ftcs3d":
        return dict(workload="ftcs3d", grid=[512, 512, 512], loc="node", bc="dirichlet 0", dt="0.1*h^2", init="8 seeded Gaussians",
                    expression="u = u + dt*alpha*(d2x(u)+d2y(u)+d2z(u))", l2="field 1.07 GB > L2 (129 MB): no flush needed")
    if name == "ftcs2d":
        return dict(workload="ftcs2d", grid=[1025, 1025], loc="node", bc="dirichlet 0", dt="0.2*h^2", init="U[0,1) seeded",
                    expression="u = u + dt*alpha*(d2x(u)+d2y(u))", l2="field 8.4 MB fits in L2: L2-resident")
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


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
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


# ------------------------------------------------------------------------------------------- ours
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
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)

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
    if world > 1:
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
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
                     "peak_source": peak_src, "traffic": traffic_for(args.workload + "_" + mode),
                     "kernel": "fast_stencil_kernel" if mode == "fast" else "ftcs_exact_kernel",
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
    ap.add_argument("--workload", default="ftcs3d", choices=["ftcs3d", "ftcs2d"])
    ap.add_argument("--mode", default="fast", choices=["fast", "exact"])
    ap.add_argument("--grid", type=int, default=0, help="override the grid side (profiling a smaller case)")
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU baseline leg (profiling runs)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python
"""MG-PCG time-to-solution benchmark (one JSON line on stdout).

Workload: the 512 x 512 uniform quadtree on [0,1]^2 with tensor-product Q3
LDG (16 DOF per element, 4,194,304 DOF), tau0 = tauD = 1/h = 512,
homogeneous Dirichlet data and a seeded 8-Gaussian forcing (seed 2001);
RATRAT Galerkin hierarchy 512 -> 4 (8 levels) with a dense coarsest
Cholesky; MG-PCG with one V(2,2) cycle as preconditioner, stopped at
r.z <= (1e-10)^2 r0.z0 as the reference's pcg does.  The coarsest level is
solved without the reference's mean projection (b -= mean(b),
multigrid.h:367): with Dirichlet data the coarse matrix is non-singular and
the projection only perturbs the correction (PCG then stalls, iteration
counts grow with n); the parity tests keep the projection on.

One step = one MG-PCG solve from x = 0 with b already in HBM.  The headline
value is the mixed form (FP32 V-cycle, FP64 CG and coarsest solve) with
block Gauss-Seidel; the plain FP64 form and the damped block-Jacobi
(omega = 0.7) variants are timed beside it.  The operator (2.68 GB in FP64)
is larger than L2, so no flush is needed between steps.

--impl reference times the CPU oracle (the restatement of the reference's
serial solver) on a bounded sample of the same workload.
Multi-GPU: the path does not shard (exact Gauss-Seidel is sequential), so
--gpus N runs N independent replicas, one per rank.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "multigrid-ldg_gb300")
sys.path.insert(0, PKG)

METRIC = "MG-PCG time-to-1e-10 residual: mixed vs FP64 on 1 GB300; SpMV HBM GB/s"
WL = dict(P=4, n=512, levels=8, npre=2, npost=2, tol=1e-10, seed=2001, maxit=200)


def workload_name(n, P, levels):
    return (f"{n}x{n} uniform quadtree, Q{P - 1} LDG ({P * P} DOF/element, {n * n * P * P:,} DOF), "
            f"tau0=tauD={n}, RATRAT hierarchy {n}->{n >> (levels - 1)} ({levels} levels, dense coarsest "
            f"Cholesky), MG-PCG V(2,2), tol 1e-10")


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------------ clocks --
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


# ----------------------------------------------------------- distributed --
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return ws, rank, local


def dist_max(v, ws):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------ CPU oracle --
def cpu_baseline(n, P, levels, iters, tol, seed):
    """Times the CPU oracle (serial restatement of the reference) on the same
    problem: setup untimed, then one pcg call with maxit=1 (initial residual,
    two V-cycles, one iteration); scaled to a full solve of `iters`
    iterations as (iters + 1) / 2 of that sample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as O
    t0 = time.perf_counter()
    pr = O.Problem(P, 1.0 / n, tau0=n, tauD=n, seed=seed)
    omg = O.Multigrid(pr, relaxation=O.RELAX_GS, omega=0.8, npre=2, npost=2, solver=O.COARSE_DENSE,
                      nlevels=levels, mean_project=False)
    t_setup = time.perf_counter() - t0
    b = pr.rhs()
    t1 = time.perf_counter()
    pr.pcg(b, mg=omg, tol=tol, maxit=1)
    t_sample = time.perf_counter() - t1
    est_ms = t_sample * (iters + 1) / 2 * 1e3
    return {"value": est_ms, "unit": "ms", "cores": 1, "kind": "port",
            "sample": (f"oracle (serial C++ restatement of the reference, FP64 Gauss-Seidel V(2,2)) on the "
                       f"full {n}x{n} Q{P - 1} problem: one pcg call with maxit=1 (initial residual + 2 V-cycles) "
                       f"took {t_sample:.2f} s; scaled by ({iters}+1)/2 to the GPU FP64 iteration count; "
                       f"oracle setup {t_setup:.1f} s not included"),
            "sample_s": t_sample, "setup_s": t_setup}


# ------------------------------------------------------------- GPU forms --
def level_bytes(mg, nlev, s):
    """Per level: algorithmic bytes of one GS sweep, one Jacobi sweep, one SpMV."""
    out = []
    for l in range(nlev):
        nbr, nbc, br, bc, nnzb = mg.level_op(l, 4).info()
        b2 = br * bc
        n = nbr * br
        idx = 4 * nnzb + 4 * (nbr + 1)
        gs = (nnzb - nbr) * b2 * s + nbr * b2 * s + idx + 3 * n * s
        jac = nnzb * b2 * s + nbr * b2 * s + idx + 3 * n * s
        spmv = nnzb * b2 * s + idx + 3 * n * s
        out.append(dict(gs=gs, jacobi=jac, spmv=spmv, nbr=nbr, nnzb=nnzb, b=br))
    return out


def run_gpu(args, ws, rank, local):
    import torch
    import mgldg
    n, P, levels = args.n, WL["P"], args.levels
    torch.cuda.set_device(local)
    ctx = mgldg.Context(local)
    ext = torch.cuda.ExternalStream(ctx.stream)
    L = mgldg.lib()
    t0 = time.perf_counter()
    prob = mgldg.CartesianProblem(ctx, P, n, tau0=float(n), tauD=float(n))
    t_build = time.perf_counter() - t0
    ndof = prob.ndof
    b = torch.empty(ndof, dtype=torch.float64, device=f"cuda:{local}")
    x = torch.zeros(ndof, dtype=torch.float64, device=f"cuda:{local}")
    torch.cuda.synchronize()
    ctx.check(L.mgldg_problem_rhs_gaussian_dev(ctx.h, prob.h, WL["seed"], C.c_void_p(b.data_ptr())), "rhs")
    ctx.sync()
    A = prob.ops.A
    forms = {
        "mixed_gs": dict(relaxation=mgldg.RELAX_GAUSS_SEIDEL, omega=0.8, precision=mgldg.PREC_MIXED),
        "fp64_gs": dict(relaxation=mgldg.RELAX_GAUSS_SEIDEL, omega=0.8, precision=mgldg.PREC_FP64),
        "mixed_jacobi": dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, precision=mgldg.PREC_MIXED),
        "fp64_jacobi": dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, precision=mgldg.PREC_FP64),
    }
    headline = "mixed_gs"
    hist = np.zeros(WL["maxit"])

    def solve(mg):
        with torch.cuda.stream(ext):
            x.zero_()
        it = C.c_int()
        ctx.check(L.mgldg_pcg_dev(ctx.h, mg.h, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), WL["tol"],
                                  WL["maxit"], C.byref(it), hist), "pcg")
        return it.value

    def timed(mg, steps, warmup, prof=False):
        for _ in range(warmup):
            solve(mg)
        torch.cuda.synchronize()
        ctx.sync()
        dist_barrier(ws)
        if prof:
            ctx.prof_reset()
            ctx.prof_enable(True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        iters = [solve(mg) for _ in range(steps)]
        e1.record(ext)
        e1.synchronize()
        ctx.sync()
        ms = e0.elapsed_time(e1) / steps
        prof_out = None
        if prof:
            prof_out = ctx.prof()
            ctx.prof_enable(False)
        torch.cuda.synchronize()
        dist_barrier(ws)
        return dist_max(ms, ws), iters, prof_out

    results, setup_ms, mgs = {}, {}, {}
    xref = None
    for name, kw in forms.items():
        t0 = time.perf_counter()
        mg = mgldg.Multigrid(ctx, prob.ops, prob.T, npre=WL["npre"], npost=WL["npost"],
                             solver=mgldg.COARSE_DENSE, max_levels=levels, mean_project=0, **kw)
        setup_ms[name] = (time.perf_counter() - t0) * 1e3
        mgs[name] = mg
    clocks = Clocks(local)
    clocks.start()
    out_prof = None
    for name in forms:
        ms, iters, prof = timed(mgs[name], args.steps, args.warmup, prof=(name == headline))
        xs = x.cpu().numpy().copy()
        bh = b.cpu().numpy()
        res = A.mv(xs, alpha=-1.0, beta=1.0, y=bh)
        results[name] = dict(ms=ms, iters=iters[-1], rel_residual=float(np.linalg.norm(res) / np.linalg.norm(bh)),
                             x=xs)
        if name == headline:
            out_prof = prof
    clk = clocks.stop()
    # FP64 reference solution for the error of each form (FP64 GS to 1e-13)
    with torch.cuda.stream(ext):
        x.zero_()
    it = C.c_int()
    ctx.check(L.mgldg_pcg_dev(ctx.h, mgs["fp64_gs"].h, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
                              1e-13, WL["maxit"], C.byref(it), hist), "pcg ref")
    ctx.sync()
    xref = x.cpu().numpy().copy()
    for name in forms:
        xs = results[name].pop("x")
        results[name]["rel_error_vs_fp64"] = float(np.linalg.norm(xs - xref) / np.linalg.norm(xref))

    # SpMV bandwidth (FP64, the outer CG operator)
    s64 = level_bytes(mgs["fp64_gs"], 1, 8)[0]["spmv"]
    y = torch.empty_like(x)
    for _ in range(3):
        ctx.check(L.mgldg_bsr_mv_dev(ctx.h, 1.0, A.h, C.c_void_p(b.data_ptr()), 0.0, C.c_void_p(y.data_ptr())), "mv")
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    nrep = 20
    e0.record(ext)
    for _ in range(nrep):
        ctx.check(L.mgldg_bsr_mv_dev(ctx.h, 1.0, A.h, C.c_void_p(b.data_ptr()), 0.0, C.c_void_p(y.data_ptr())), "mv")
    e1.record(ext)
    e1.synchronize()
    spmv_ms = e0.elapsed_time(e1) / nrep
    hbm, peak_kind = peaks()

    # roofline of the dominant kernel class of the headline form
    mgh = mgs[headline]
    s = 4 if forms[headline]["precision"] == mgldg.PREC_MIXED else 8
    lb = level_bytes(mgh, levels - 1, s)
    cls = max(out_prof, key=lambda k: out_prof[k][1])
    vcycles = sum(1 for _ in range(args.steps)) * (results[headline]["iters"] + 1)
    key = "gs" if forms[headline]["relaxation"] == mgldg.RELAX_GAUSS_SEIDEL else "jacobi"
    sweep_bytes = vcycles * (WL["npre"] + WL["npost"]) * sum(l[key] for l in lb)
    launches, cls_ms = out_prof[cls]
    if cls in ("gauss_seidel", "jacobi"):
        algo_bytes = sweep_bytes
    else:
        algo_bytes = None
    achieved = algo_bytes / (cls_ms * 1e-3) / 1e9 if algo_bytes else None
    roof = {"bound": "hbm", "kernel": cls, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": (achieved / hbm) if achieved else None, "traffic": None, "peak_kind": peak_kind,
            "launches": launches, "avg_launch_ms": cls_ms / max(1, launches),
            "algorithmic_bytes_per_launch": (algo_bytes / launches) if algo_bytes else None}
    gpu_launches = int(sum(v[0] for v in out_prof.values()))

    # end to end through the public host API: pinned host b -> device, solve,
    # x -> host, every step
    bh = torch.empty(ndof, dtype=torch.float64, pin_memory=True)
    bh.copy_(b.cpu())
    xh = torch.zeros(ndof, dtype=torch.float64, pin_memory=True)
    bnp, xnp = bh.numpy(), xh.numpy()
    e2e = []
    for k in range(args.warmup + args.steps):
        xnp[:] = 0.0
        dist_barrier(ws)
        t0 = time.perf_counter()
        _, hh = mgldg.pcg(ctx, A, bnp, x=xnp, precon=mgs[headline], tol=WL["tol"], maxit=WL["maxit"])
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            e2e.append(dt * 1e3)
    e2e_ms = dist_max(float(np.mean(e2e)), ws)

    line = {
        "metric": METRIC, "value": results[headline]["ms"], "unit": "ms", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": results[headline]["ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 V-cycle / f64 CG",
        "data": f"synthetic: seeded 8-Gaussian forcing (seed {WL['seed']}), homogeneous Dirichlet",
        "config": {"workload": workload_name(n, P, levels), "form": "mixed precision, block Gauss-Seidel omega=0.8",
                   "parallelism": "replicas" if ws > 1 else "single GPU",
                   "l2": "inputs larger than L2 (A is 2.68 GB in FP64, 1.34 GB in FP32)"},
        "forms": results,
        "mixed_vs_fp64_speedup": {"gs": results["fp64_gs"]["ms"] / results["mixed_gs"]["ms"],
                                  "jacobi": results["fp64_jacobi"]["ms"] / results["mixed_jacobi"]["ms"],
                                  "best_mixed_vs_best_fp64": min(results["fp64_gs"]["ms"], results["fp64_jacobi"]["ms"]) /
                                  min(results["mixed_gs"]["ms"], results["mixed_jacobi"]["ms"])},
        "spmv": {"precision": "fp64", "ms": spmv_ms, "gbs": s64 / (spmv_ms * 1e-3) / 1e9, "bytes": s64,
                 "frac_of_hbm": s64 / (spmv_ms * 1e-3) / 1e9 / hbm},
        "setup_ms": {"problem_build": t_build * 1e3, **setup_ms},
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": 2 * ndof * 8, "d2h_bytes_per_step": ndof * 8,
                "api": "mgldg_pcg (host buffers, pinned)"},
        "roofline": roof,
        "kernel_breakdown_ms": {k: v[1] for k, v in out_prof.items()},
        "gpu_launches": gpu_launches,
        "clocks": clk,
    }
    return line, results


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=WL["n"])
    ap.add_argument("--levels", type=int, default=WL["levels"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline")
    args = ap.parse_args()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        if rank == 0:
            iters = 14
            cb = cpu_baseline(args.n, WL["P"], args.levels, iters, WL["tol"], WL["seed"])
            samples = [cb["value"]]
            line = {"metric": METRIC, "value": cb["value"], "unit": "ms", "n_gpus": ws, "steps": 1, "warmup": 0,
                    "ms_per_step": cb["value"], "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                    "dtype": "f64", "data": f"synthetic: seeded 8-Gaussian forcing (seed {WL['seed']})",
                    "config": {"workload": workload_name(args.n, WL["P"], args.levels),
                               "form": "reference method: FP64 Gauss-Seidel V(2,2), serial CPU"},
                    "impl": "reference",
                    "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                    "e2e": {"value": cb["value"], "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
            del samples
            print(json.dumps(line), flush=True)
        return
    t0 = time.perf_counter()
    line, results = run_gpu(args, ws, rank, local)
    print(f"[bench] GPU part {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
    if rank == 0:
        if ws == 1 and not args.no_cpu:
            line["cpu_baseline"] = {k: v for k, v in cpu_baseline(args.n, WL["P"], args.levels,
                                                                  results["fp64_gs"]["iters"], WL["tol"],
                                                                  WL["seed"]).items()
                                    if k in ("value", "unit", "cores", "kind", "sample")}
        print(f"[bench] total {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

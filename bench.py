#!/usr/bin/env python
"""MG-PCG time-to-solution benchmark (one JSON line on stdout).

Workload: the 512 x 512 uniform quadtree on [0,1]^2 with tensor-product Q3
LDG (16 DOF per element, 4,194,304 DOF), tau0 = tauD = 1/h = 512,
homogeneous Dirichlet data and a seeded 8-Gaussian forcing (seed 2001);
RATRAT Galerkin hierarchy 512 -> 4 (8 levels) with a dense coarsest
inverse; MG-PCG with one V(2,2) cycle as preconditioner, stopped at
r.z <= (1e-10)^2 r0.z0 as the reference's pcg does.  The coarsest level is
solved without the reference's mean projection (b -= mean(b),
multigrid.h:367): with Dirichlet data the coarse matrix is non-singular and
the projection only perturbs the correction (PCG then stalls, iteration
counts grow with n); the parity tests keep the projection on.

One step = one MG-PCG solve from x = 0 with b already in HBM.  The headline
value is the mixed form of the workload -- FP32 BSR blocks, FP32 V-cycle,
FP64 outer CG and coarsest solve -- with damped block Jacobi (omega = 0.7);
the plain FP64 form, block Gauss-Seidel (omega = 0.8, the reference's exact
sweep order) in both precisions and the FP16-stored copy of the level
operators are timed beside it ("forms").  The operator (2.68 GB in FP64) is
larger than L2, so no flush is needed between steps.

CPU baseline: the oracle (the restatement of the reference's serial solver)
runs the whole FP64 solve of the same problem with the same smoother on one
host core -- setup ("Build multigrid hierarchy") and solve ("Solve using
MGPCG") timed separately, as the reference's driver does -- in a child
process beside the GPU measurement.  --impl reference prints that
measurement as the reference arm.
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
            f"inverse), MG-PCG V(2,2), tol 1e-10")


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
REF_SMOOTHERS = {"jacobi": (0, 0.7), "gs": (1, 0.8)}   # oracle RELAX_* value, omega


def cpu_oracle_solve(n, P, levels, smoother, tol, seed):
    """The CPU oracle (serial restatement of the reference's solver) on the
    full problem, timed as the reference's driver times it
    (tests/cartesian/dg_tests.cpp:294-308): "Build multigrid hierarchy" --
    the LDG operators and the Galerkin hierarchy -- then "Solve using MGPCG",
    the whole pcg to the tolerance from x = 0.  FP64, one thread (the
    reference is serial)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as O
    relax, omega = REF_SMOOTHERS[smoother]
    t0 = time.perf_counter()
    pr = O.Problem(P, 1.0 / n, tau0=n, tauD=n, seed=seed)
    omg = O.Multigrid(pr, relaxation=relax, omega=omega, npre=2, npost=2, solver=O.COARSE_DENSE,
                      nlevels=levels, mean_project=False)
    setup_s = time.perf_counter() - t0
    b = pr.rhs()
    t1 = time.perf_counter()
    _, hist, _ = pr.pcg(b, mg=omg, tol=tol, maxit=WL["maxit"])
    solve_s = time.perf_counter() - t1
    return {"smoother": smoother, "setup_s": setup_s, "solve_ms": solve_s * 1e3, "iters": int(len(hist))}


def cpu_baseline_line(results, n, P):
    """cpu_baseline object from measured full oracle solves."""
    main = results[0]
    text = "; ".join(f"{r['smoother']}: setup {r['setup_s']:.1f} s, solve {r['solve_ms'] / 1e3:.1f} s, "
                     f"{r['iters']} iterations" for r in results)
    return {"value": main["solve_ms"], "unit": "ms", "cores": 1, "kind": "port",
            "sample": (f"the whole FP64 MG-PCG solve to 1e-10 of the oracle (serial C++ restatement of the "
                       f"reference) on the full {n}x{n} Q{P - 1} problem, measured, not extrapolated ({text}); "
                       f"value = the {main['smoother']} solve"),
            "runs": results}


def start_cpu_baseline(args):
    """Starts the oracle's full solve in a child process (spawned before any
    GPU work, so that it runs beside the GPU measurement on another host
    core); returns the process, whose stdout is one JSON line."""
    cmd = [sys.executable, os.path.abspath(__file__), "--cpu-oracle", args.cpu_smoothers, "--n", str(args.n),
           "--levels", str(args.levels)]
    return subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)


def finish_cpu_baseline(proc):
    out, _ = proc.communicate()
    for line in out.splitlines():
        if line.startswith("["):
            return json.loads(line)
    return None


# ------------------------------------------------------------- GPU forms --
def level_bytes(mg, nlev, s, f16=False):
    """Per level: algorithmic bytes of one GS sweep, one Jacobi sweep, one
    Jacobi sweep from x = 0 (the first of each V-cycle level: inverse diagonal
    blocks, b and x_out only), one SpMV.  f16: the level operator is read from
    its block-scaled FP16 copy (2 bytes per entry + one 4-byte scale per
    block; inverse diagonal blocks and vectors in FP32, s = 4)."""
    out = []
    for l in range(nlev):
        nbr, nbc, br, bc, nnzb = mg.level_op(l, 4).info()
        b2 = br * bc
        n = nbr * br
        idx = 4 * nnzb + 4 * (nbr + 1)
        av = nnzb * (b2 * 2 + 4) if f16 else nnzb * b2 * s
        gs = (nnzb - nbr) * b2 * s + nbr * b2 * s + idx + 3 * n * s
        jac = av + nbr * b2 * s + idx + 3 * n * s
        jac0 = nbr * b2 * s + 2 * n * s
        spmv = av + idx + 3 * n * s
        out.append(dict(gs=gs, jacobi=jac, jacobi0=jac0, spmv=spmv, nbr=nbr, nnzb=nnzb, b=br))
    return out


FORMS = {
    # name: (relaxation, omega, precision) -- MGLDG_RELAX_* / MGLDG_PREC_* values
    "mixed_jacobi": (0, 0.7, 1),
    "fp64_jacobi": (0, 0.7, 0),
    "mixed_gs": (1, 0.8, 1),
    "fp64_gs": (1, 0.8, 0),
    "mixed16_jacobi": (0, 0.7, 2),
}
FORM_TEXT = {"mixed16_jacobi": ("mixed precision with the level operators stored as block-scaled FP16 (one FP32 "
                               "scale per block), damped block Jacobi omega=0.7"),
             "mixed_jacobi": "mixed precision (FP32 BSR blocks, FP32 V-cycle, FP64 CG), damped block Jacobi omega=0.7",
             "fp64_jacobi": "FP64, damped block Jacobi omega=0.7",
             "mixed_gs": "mixed precision (FP32 BSR blocks, FP32 V-cycle, FP64 CG), block Gauss-Seidel omega=0.8",
             "fp64_gs": "FP64, block Gauss-Seidel omega=0.8"}
SMOOTHER_TEXT = {0: "damped block Jacobi omega=0.7, V(2,2)", 1: "block Gauss-Seidel omega=0.8 (exact order), V(2,2)"}
DTYPE = {0: "f64", 1: "f32 V-cycle (FP32 BSR blocks) / f64 CG", 2: "f16-stored level operators, f32 V-cycle / f64 CG"}
L2_TEXT = "inputs larger than L2 (A is 2.68 GB in FP64, 1.34 GB in FP32), no flush"


def fp64_peak_tflops(torch):
    """cuBLAS FP64 GEMM rate (the FP64 ceiling of this GPU), best of 3."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    bm = torch.randn(n, n, dtype=torch.float64, device="cuda")
    a @ bm
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        a @ bm
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, bm
    return 2 * n ** 3 / (best * 1e-3) / 1e12


def run_config1(args, ctx, ext, torch, local, ws):
    """The reference method on the small grid: 32 x 32 uniform quadtree, Q2
    LDG (9 DOF/element, 9,216 DOF), tau0 = tauD = 32, RATRAT hierarchy
    32 -> 4 (4 levels) with a dense coarsest inverse, FP64 block
    Gauss-Seidel (omega 0.8) V(2,2) with the reference's coarse mean
    projection, MG-PCG to 1e-10.  The operator (3.2 MB) lives in L2, so the
    line is a latency figure: solves per second, device-timed (b resident)
    and end to end through mgldg_pcg with host buffers; the oracle's whole
    solve of the same problem is timed beside it."""
    import mgldg
    L = mgldg.lib()
    n, P, levels, seed = 32, 3, 4, 1001
    prob = mgldg.CartesianProblem(ctx, P, n, tau0=float(n), tauD=float(n))
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, npre=2, npost=2, solver=mgldg.COARSE_DENSE, max_levels=levels,
                         relaxation=mgldg.RELAX_GAUSS_SEIDEL, omega=0.8)
    dev = f"cuda:{local}"
    b = torch.empty(prob.ndof, dtype=torch.float64, device=dev)
    x = torch.zeros_like(b)
    torch.cuda.synchronize()
    ctx.check(L.mgldg_problem_rhs_gaussian_dev(ctx.h, prob.h, seed, C.c_void_p(b.data_ptr())), "rhs")
    ctx.sync()
    A = prob.ops.A
    hist = np.zeros(WL["maxit"])
    it = C.c_int()

    def solve():
        with torch.cuda.stream(ext):
            x.zero_()
        ctx.check(L.mgldg_pcg_dev(ctx.h, mg.h, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), WL["tol"],
                                  WL["maxit"], C.byref(it), hist), "pcg")

    for _ in range(max(3, args.warmup)):
        solve()
    ctx.sync()
    nrep = 200
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(nrep):
        solve()
    e1.record(ext)
    e1.synchronize()
    ms = dist_max(e0.elapsed_time(e1) / nrep, ws)
    # end to end through mgldg_pcg with pinned host b and x (x zeroed outside the clock)
    bh = torch.empty(b.numel(), dtype=torch.float64, pin_memory=True)
    bh.copy_(b.cpu())
    xh = torch.zeros(b.numel(), dtype=torch.float64, pin_memory=True)
    bh, xh = bh.numpy(), xh.numpy()
    lib = mgldg.lib()
    it_e2e = C.c_int()
    hist_e2e = np.zeros(WL["maxit"])
    e2e = 0.0
    for _ in range(nrep):
        xh[:] = 0.0
        t0 = time.perf_counter()
        ctx.check(lib.mgldg_pcg(ctx.h, mg.h, A.h, bh, xh, WL["tol"], WL["maxit"], C.byref(it_e2e), hist_e2e), "pcg")
        e2e += time.perf_counter() - t0
    e2e_ms = e2e * 1e3 / nrep
    out = {"workload": ("32x32 uniform quadtree, Q2 LDG (9,216 DOF), tau0=tauD=32, RATRAT 32->4 (4 levels, dense "
                        "coarsest, mean projection), FP64 block Gauss-Seidel omega=0.8 V(2,2), tol 1e-10"),
           "ms_per_solve": ms, "solves_per_s": 1e3 / ms, "e2e_ms_per_solve": e2e_ms, "iters": it.value}
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle_py as O
        t0 = time.perf_counter()
        pr = O.Problem(P, 1.0 / n, tau0=n, tauD=n, seed=seed)
        omg = O.Multigrid(pr, relaxation=O.RELAX_GS, omega=0.8, npre=2, npost=2, solver=O.COARSE_DENSE,
                          nlevels=levels, mean_project=True)
        setup_s = time.perf_counter() - t0
        t1 = time.perf_counter()
        _, hr, _ = pr.pcg(pr.rhs(), mg=omg, tol=WL["tol"], maxit=WL["maxit"])
        out["cpu_oracle"] = {"setup_s": setup_s, "solve_ms": (time.perf_counter() - t1) * 1e3, "iters": len(hr),
                             "cores": 1}
    del mg, prob, b, x
    return out


def run_batched(args, ctx, ext, torch, local, ws, precision=None):
    """Many right-hand sides: k seeded 8-Gaussian forcings (seeds 3001..)
    solved together by the block PCG, mixed precision, damped block Jacobi
    (omega 0.7), V(2,2).  Mesh: the adaptive quadtree of the multi-RHS
    workload -- 64 x 64 refined up to 6 more levels around 4 seeded points
    (seed 3000; a cell of extra level l is split while its centre lies within
    0.5 * 2^-l of a point), 2:1 balanced, per-face penalty 1/min(h_L, h_R) --
    or (--batched-mesh uniform) a uniform n x n grid."""
    import mgldg
    L = mgldg.lib()
    k, nb, P = args.batched, args.batched_n, 3
    t0 = time.perf_counter()
    if args.batched_mesh == "adaptive":
        pts = mgldg.seeded_points(3000, 4)
        qt = mgldg.Quadtree.points(pts, 6, 6, radius=0.5, balance=True)
        prob = mgldg.CartesianProblem(ctx, P, quadtree=qt, tau0=1.0, tauD=1.0, tau_per_face=True)
        levels = prob.nlevels - 3                 # coarsest layer: the 8 x 8 grid
        mesh = (f"adaptive quadtree 64x64 + 6 levels around 4 seeded points (seed 3000), 2:1 balanced, "
                f"{prob.ne:,} elements, tau=1/min(h_L,h_R)")
    else:
        prob = mgldg.CartesianProblem(ctx, P, nb, tau0=float(nb), tauD=float(nb))
        levels = max(2, nb.bit_length() - 3)      # down to 4 x 4
        mesh = f"{nb}x{nb} uniform quadtree"
    build_ms = (time.perf_counter() - t0) * 1e3
    ndof = prob.ndof
    dev = f"cuda:{local}"
    B = torch.empty((ndof, k), dtype=torch.float64, device=dev)
    tmp = torch.empty(ndof, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    for c in range(k):
        ctx.check(L.mgldg_problem_rhs_gaussian_dev(ctx.h, prob.h, 3001 + c, C.c_void_p(tmp.data_ptr())), "rhs")
        ctx.sync()
        B[:, c] = tmp
    torch.cuda.synchronize()
    X = torch.zeros_like(B)
    prec = mgldg.PREC_MIXED if precision is None else precision
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, npre=2, npost=2, solver=mgldg.COARSE_DENSE, max_levels=levels,
                         mean_project=0, relaxation=mgldg.RELAX_JACOBI, omega=0.7, precision=prec)
    A = prob.ops.A
    its = np.zeros(k, np.int32)
    hist = np.zeros(WL["maxit"] * k)

    def solve():
        with torch.cuda.stream(ext):
            X.zero_()
        ctx.check(L.mgldg_pcg_batched_dev(ctx.h, mg.h, A.h, k, C.c_void_p(B.data_ptr()), C.c_void_p(X.data_ptr()),
                                          WL["tol"], WL["maxit"], its, hist), "pcg_batched")

    t0 = time.perf_counter()
    solve()                                       # first call: work space + tile autotuning
    ctx.sync()
    first_ms = (time.perf_counter() - t0) * 1e3
    for _ in range(max(0, args.warmup - 1)):
        solve()
    ctx.sync()
    dist_barrier(ws)
    ctx.prof_reset()
    steps = max(1, min(args.steps, 3))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(steps):
        solve()
    e1.record(ext)
    e1.synchronize()
    ms = dist_max(e0.elapsed_time(e1) / steps, ws)
    launches = ctx.prof()
    ctx.prof_enable(True)
    ctx.prof_reset()
    solve()
    prof = ctx.prof()
    ctx.prof_enable(False)
    # single-RHS solve of column 0 with the same hierarchy for comparison
    x1 = torch.zeros(ndof, dtype=torch.float64, device=dev)
    b0 = B[:, 0].contiguous()
    torch.cuda.synchronize()
    it1 = C.c_int()
    h1 = np.zeros(WL["maxit"])
    for _ in range(2):
        with torch.cuda.stream(ext):
            x1.zero_()
        ctx.check(L.mgldg_pcg_dev(ctx.h, mg.h, A.h, C.c_void_p(b0.data_ptr()), C.c_void_p(x1.data_ptr()),
                                  WL["tol"], WL["maxit"], C.byref(it1), h1), "pcg")
    ctx.sync()
    e0.record(ext)
    with torch.cuda.stream(ext):
        x1.zero_()
    ctx.check(L.mgldg_pcg_dev(ctx.h, mg.h, A.h, C.c_void_p(b0.data_ptr()), C.c_void_p(x1.data_ptr()),
                              WL["tol"], WL["maxit"], C.byref(it1), h1), "pcg")
    e1.record(ext)
    e1.synchronize()
    single_ms = e0.elapsed_time(e1)
    torch.cuda.synchronize()
    err0 = float(torch.linalg.norm(X[:, 0] - x1) / torch.linalg.norm(x1))
    nbr, _, br, _, nnzb = A.info()
    tiles = [mgldg.batch_tiles(mg, l) for l in range(mg.nlevels)]
    # level-0 Jacobi SpMM of the profiled batch against HBM: per V-cycle
    # npre + npost launches, the first from X = 0 (inverse diagonal blocks,
    # B and X_out only), the others full sweeps (FP32 blocks, indices, B,
    # X_in, X_out; k columns per vector)
    nj, msj = ctx.prof_level(2, 0)
    n0 = nbr * br
    full = nnzb * br * br * 4 + nbr * br * br * 4 + 4 * nnzb + 4 * (nbr + 1) + 3 * n0 * k * 4
    zero = nbr * br * br * 4 + 2 * n0 * k * 4
    nsw = WL["npre"] + WL["npost"]
    jbytes = ((nsw - 1) * full + zero) / nsw
    hbm, peak_kind = peaks()
    roof = None
    if nj:
        ach = jbytes * nj / (msj * 1e-3) / 1e9
        roof = {"bound": "hbm", "kernel": "jacobi (multi-RHS SpMM, CUDA cores)" if prec != mgldg.PREC_MIXED_TF32
                else "jacobi (multi-RHS SpMM, tensor cores 3xTF32)", "level": 0, "achieved": ach, "peak": hbm,
                "unit": "GB/s", "frac": ach / hbm, "peak_kind": peak_kind, "launches": nj, "avg_launch_ms": msj / nj,
                "algorithmic_bytes_per_launch": jbytes}
    out = {
        "workload": (f"{mesh}, Q2 LDG (9 DOF/element, {ndof:,} DOF), {k} right-hand sides "
                     f"(seeds 3001..{3000 + k}), RATRAT ({levels} levels, dense coarsest), "
                     f"{'mixed precision with the level products on the tensor cores (3xTF32)' if prec == mgldg.PREC_MIXED_TF32 else 'mixed precision'}, "
                     f"block Jacobi omega=0.7, V(2,2), tol 1e-10 per column"),
        "problem_build_ms": build_ms,
        "k": k, "ms_per_batch": ms, "solves_per_s": k / (ms * 1e-3), "ms_per_rhs": ms / k,
        "single_rhs_ms": single_ms, "batching_gain": single_ms / (ms / k),
        "iters_min": int(its.min()), "iters_max": int(its.max()),
        "col0_rel_diff_vs_single": err0,
        "first_call_ms_incl_autotune": first_ms,
        "tiles_level0": dict(zip(["spmm", "jacobi", "restrict", "prolong", "outer_fp64"], tiles[0])),
        "kernel_ms": {kk: round(v[1], 3) for kk, v in prof.items() if v[0]},
        "launches_per_batch": int(sum(v[0] for v in launches.values()) / steps),
        "outer_fp64_spmm_gflop": 2 * nnzb * br * br * k / 1e9,
        "roofline": roof,
        "steps": steps,
    }
    del B, X, tmp, mg, prob
    torch.cuda.empty_cache()
    return out


def _coarse_levels(prob, max_dense=4096):
    """Levels to keep so that the coarsest agglomerated level fits the dense solve."""
    n = prob.ne * prob.npl
    for l in range(len(prob.T)):
        if n <= max_dense:
            return l + 1
        n = (int(prob.partition(l).max()) + 1) * prob.T[l].info()[3]
    return len(prob.T) + 1


def run_unstructured(args, ctx, ext, torch, local, ws):
    """Unstructured P2 triangles on the unit disk (ring mesher, spacing h):
    one mesh at h = 0.004 and an uneven batch of 48 disks with h drawn from
    U[0.01, 0.04] (seed 4000) solved together by the segmented PCG; each mesh
    with its own seeded disk Gaussian-sum forcing, tau = 1/h, greedy seeded
    agglomeration (seed 4000), RATRAT, mixed precision, block Jacobi omega 0.7,
    V(2,2), dense coarsest solve, tol 1e-10."""
    import mgldg
    L = mgldg.lib()
    P = 3
    dev = f"cuda:{local}"
    out = {}
    steps = max(1, min(args.steps, 3))

    def time_solves(fn):
        for _ in range(max(1, args.warmup - 1)):
            fn()
        ctx.sync()
        dist_barrier(ws)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        for _ in range(steps):
            r = fn()
        e1.record(ext)
        e1.synchronize()
        return dist_max(e0.elapsed_time(e1) / steps, ws), r

    # ---- one large mesh ----
    h = args.disk_h
    t0 = time.perf_counter()
    pts, tri = mgldg.disk_mesh(h)
    prob = mgldg.CartesianProblem(ctx, P, mesh=(pts, tri), tau0=1 / h, tauD=1 / h, agg_levels=12, agg_seed=4000)
    build_ms = (time.perf_counter() - t0) * 1e3
    nlev = _coarse_levels(prob)
    t0 = time.perf_counter()
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, npre=2, npost=2, solver=mgldg.COARSE_DENSE, max_levels=nlev,
                         mean_project=0, relaxation=mgldg.RELAX_JACOBI, omega=0.7, precision=_vprec(args))
    setup_ms = (time.perf_counter() - t0) * 1e3
    b = torch.empty(prob.ndof, dtype=torch.float64, device=dev)
    x = torch.zeros_like(b)
    torch.cuda.synchronize()
    ctx.check(L.mgldg_problem_rhs_gaussian_dev(ctx.h, prob.h, 4001, C.c_void_p(b.data_ptr())), "rhs")
    ctx.sync()
    hist = np.zeros(WL["maxit"])
    A = prob.ops.A

    def solve1():
        with torch.cuda.stream(ext):
            x.zero_()
        it = C.c_int()
        ctx.check(L.mgldg_pcg_dev(ctx.h, mg.h, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), WL["tol"],
                                  WL["maxit"], C.byref(it), hist), "pcg")
        return it.value

    ms, iters = time_solves(solve1)
    xs = x.cpu().numpy()
    bs = b.cpu().numpy()
    res1 = float(np.linalg.norm(A.mv(xs, alpha=-1.0, beta=1.0, y=bs)) / np.linalg.norm(bs))
    out["single"] = {
        "workload": (f"unit disk, ring mesh h={h} in Morton order: {prob.ne:,} triangles, P2 LDG (6 DOF/element, "
                     f"{prob.ndof:,} "
                     f"DOF), tau=1/h, {nlev} agglomeration levels (dense coarsest), {_vtext(args)}, Jacobi "
                     f"omega=0.7, V(2,2), tol 1e-10"),
        "ms_per_solve": ms, "iters": iters, "true_rel_residual": res1, "problem_build_ms": build_ms,
        "mg_setup_ms": setup_ms,
    }
    del mg, prob, b, x
    torch.cuda.empty_cache()
    if args.disk_batch <= 0:
        return out

    # ---- uneven batch of meshes ----
    rng = np.random.default_rng(4000)
    hs = rng.uniform(0.01, 0.04, args.disk_batch)
    meshes = [mgldg.disk_mesh(float(v)) for v in hs]
    pts, tri, eoff = mgldg.mesh_union(meshes)
    t0 = time.perf_counter()
    prob = mgldg.CartesianProblem(ctx, P, mesh=(pts, tri), tau0=1 / float(hs.min()), tauD=1 / float(hs.min()),
                                  agg_levels=12, agg_seed=4000)
    build_ms = (time.perf_counter() - t0) * 1e3
    nlev = _coarse_levels(prob)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, npre=2, npost=2, solver=mgldg.COARSE_DENSE, max_levels=nlev,
                         mean_project=0, relaxation=mgldg.RELAX_JACOBI, omega=0.7, precision=_vprec(args))
    off = (eoff * prob.npl).astype(np.int64)
    nseg = len(meshes)
    b = torch.empty(prob.ndof, dtype=torch.float64, device=dev)
    tmp = torch.empty_like(b)
    x = torch.zeros_like(b)
    torch.cuda.synchronize()
    for s in range(nseg):
        ctx.check(L.mgldg_problem_rhs_gaussian_dev(ctx.h, prob.h, 4001 + s, C.c_void_p(tmp.data_ptr())), "rhs")
        ctx.sync()
        b[off[s]:off[s + 1]] = tmp[off[s]:off[s + 1]]
    torch.cuda.synchronize()
    its = np.zeros(nseg, np.int32)
    shist = np.zeros(WL["maxit"] * nseg)
    offp = off.ctypes.data_as(C.POINTER(C.c_int64))

    def solve_batch():
        with torch.cuda.stream(ext):
            x.zero_()
        ctx.check(L.mgldg_pcg_segmented_dev(ctx.h, mg.h, prob.ops.A.h, nseg, offp, C.c_void_p(b.data_ptr()),
                                            C.c_void_p(x.data_ptr()), WL["tol"], WL["maxit"], its, shist), "seg")
        return its.copy()

    ms, it = time_solves(solve_batch)
    xs = x.cpu().numpy()
    bs = b.cpu().numpy()
    rs = prob.ops.A.mv(xs, alpha=-1.0, beta=1.0, y=bs)
    worst = max(float(np.linalg.norm(rs[off[s]:off[s + 1]]) / np.linalg.norm(bs[off[s]:off[s + 1]]))
                for s in range(nseg))
    out["uneven_batch"] = {
        "workload": (f"{nseg} disks, h ~ U[0.01,0.04] (seed 4000), {prob.ne:,} triangles / {prob.ndof:,} DOF in "
                     f"total ({min(len(t) for _, t in meshes):,}..{max(len(t) for _, t in meshes):,} per mesh), "
                     f"one block-diagonal union, segmented PCG (per-mesh CG scalars and stopping), {nlev} "
                     f"agglomeration levels, {_vtext(args)}, Jacobi omega=0.7, V(2,2), tol 1e-10 per mesh"),
        "ms_per_batch": ms, "meshes_per_s": nseg / (ms * 1e-3), "iters_min": int(it.min()), "iters_max": int(it.max()),
        "worst_true_rel_residual": worst,
        "problem_build_ms": build_ms,
    }
    del mg, prob, b, x, tmp
    torch.cuda.empty_cache()
    return out


def _vprec(args):
    """V-cycle precision of the unstructured and adjoint lines."""
    import mgldg
    return mgldg.PREC_MIXED_F16 if args.vcycle == "mixed16" else mgldg.PREC_MIXED


def _vtext(args):
    return ("mixed precision with FP16-stored level operators (one FP32 scale per block)" if args.vcycle == "mixed16"
            else "mixed precision")


def _field_at(X, seed, corr=0.2, sigma=0.5, nfeat=64):
    """log-normal per-element diffusivity exp(g(x)), g a random-Fourier-feature
    Gaussian field (correlation length corr, deviation sigma) -- the same
    construction as the test's FP64 reference."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nfeat, X.shape[1])) / corr
    ph = rng.uniform(0, 2 * np.pi, nfeat)
    a = rng.standard_normal(nfeat) * sigma * np.sqrt(2.0 / nfeat)
    return np.exp(np.cos(X @ w.T + ph) @ a)


def run_adjoint(args, ctx, ext, torch, local, ws):
    """P2 LDG on tetrahedra of the unit ball (ball mesher, h), per-element
    diffusivity kappa_e = exp(g_e) (field seed 5011), u_obs the solution for a
    perturbed kappa (seed 5012), loss 1/2 ||u - u_obs||^2: one step = forward
    MG-PCG + adjoint MG-PCG on the same hierarchy + dL/dkappa, mixed precision,
    RAT coarsening over the agglomeration hierarchy, block Jacobi omega 0.7,
    V(2,2), tol 1e-10."""
    import mgldg
    L = mgldg.lib()
    h, P = args.ball_h, 3
    dev = f"cuda:{local}"
    t0 = time.perf_counter()
    pts, tets = mgldg.ball_mesh(h)
    prob = mgldg.CartesianProblem(ctx, P, mesh=(pts, tets), tau0=1 / h, tauD=1 / h, agg_levels=12, agg_seed=5000)
    build_ms = (time.perf_counter() - t0) * 1e3
    cent = pts[tets].mean(axis=1)
    kappa = _field_at(cent, 5011)
    k_true = _field_at(cent, 5012)
    nlev = _coarse_levels(prob)
    kw = dict(npre=2, npost=2, solver=mgldg.COARSE_DENSE, max_levels=nlev, mean_project=0,
              relaxation=mgldg.RELAX_JACOBI, omega=0.7, restriction=mgldg.RESTRICT_RAT,
              precision=_vprec(args))
    n, ne = prob.ndof, prob.ne
    b = torch.empty(n, dtype=torch.float64, device=dev)
    u = torch.zeros_like(b)
    lam = torch.zeros_like(b)
    uobs = torch.zeros_like(b)
    dk = torch.zeros(ne, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    ctx.check(L.mgldg_problem_rhs_gaussian_dev(ctx.h, prob.h, 5001, C.c_void_p(b.data_ptr())), "rhs")
    ctx.sync()
    it1 = C.c_int()
    # A(k_true) kept as a copy (the multigrid built next borrows ops' own A)
    prob.ops.construct_laplacian_kappa(k_true)
    A_true = prob.ops.A.clone()
    t0 = time.perf_counter()
    prob.ops.construct_laplacian_kappa(kappa)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, **kw)
    setup_ms = (time.perf_counter() - t0) * 1e3
    # observation: the solve with the perturbed diffusivity, preconditioned by
    # the same hierarchy (an SPD preconditioner for A(k_true) as well)
    ctx.check(L.mgldg_pcg_dev(ctx.h, mg.h, A_true.h, C.c_void_p(b.data_ptr()), C.c_void_p(uobs.data_ptr()),
                              1e-12, 1000, C.byref(it1), np.zeros(1000)), "pcg")
    del A_true
    loss = C.c_double()
    its = (C.c_int * 2)()
    p_ = lambda t: C.c_void_p(t.data_ptr())

    def step():
        with torch.cuda.stream(ext):
            u.zero_()
            lam.zero_()
        ctx.check(L.mgldg_adjoint_l2_dev(ctx.h, mg.h, prob.ops.h, p_(b), p_(uobs), WL["tol"], 400, p_(u), p_(lam),
                                         p_(dk), C.byref(loss), its), "adjoint")
        return its[0], its[1]

    step()   # warm-up (a gradient is seconds of work)
    ctx.sync()
    dist_barrier(ws)
    steps = 2
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(steps):
        itp = step()
    e1.record(ext)
    e1.synchronize()
    ms = dist_max(e0.elapsed_time(e1) / steps, ws)
    g = dk.cpu().numpy()
    # check: true relative residual of the forward solution
    r = torch.empty_like(b)
    r.copy_(b)
    torch.cuda.synchronize()
    ctx.check(L.mgldg_bsr_mv_dev(ctx.h, -1.0, prob.ops.A.h, p_(u), 1.0, p_(r)), "mv")
    ctx.sync()
    rel_res = float(torch.linalg.norm(r) / torch.linalg.norm(b))
    # the mixed form's gradient against the FP64 one (FP64 V-cycle, tol 1e-12)
    del mg
    kw64 = dict(kw, precision=mgldg.PREC_FP64)
    mg64 = mgldg.Multigrid(ctx, prob.ops, prob.T, **kw64)
    u64, lam64, dk64 = torch.zeros_like(b), torch.zeros_like(b), torch.zeros_like(dk)
    loss64 = C.c_double()
    its64 = (C.c_int * 2)()
    ctx.check(L.mgldg_adjoint_l2_dev(ctx.h, mg64.h, prob.ops.h, p_(b), p_(uobs), 1e-12, 600, p_(u64), p_(lam64),
                                     p_(dk64), C.byref(loss64), its64), "adjoint fp64")
    ctx.sync()
    g64 = dk64.cpu().numpy()
    grad_err = float(np.abs(g - g64).max() / np.abs(g64).max())
    del mg64, u64, lam64, dk64
    out = {
        "workload": (f"unit ball, cubed-sphere hexahedra cut into 24 tetrahedra each, h={h}: {ne:,} tetrahedra, "
                     f"P2 LDG (10 DOF/element, "
                     f"{n:,} DOF), kappa_e = exp(g_e) (random-Fourier-feature field, corr 0.2, sigma 0.5, seed 5011), "
                     f"u_obs from kappa seed 5012, L = 1/2 ||u - u_obs||^2; forward + adjoint MG-PCG on one hierarchy "
                     f"({nlev} agglomeration levels, RAT, dense coarsest), {_vtext(args)}, block Jacobi "
                     f"omega=0.7, V(2,2), "
                     f"tol 1e-10, plus dL/dkappa"),
        "ms_per_gradient": ms, "forward_iters": int(itp[0]), "adjoint_iters": int(itp[1]),
        "loss": loss.value, "grad_norm": float(np.linalg.norm(g)), "forward_true_rel_residual": rel_res,
        "problem_build_ms": build_ms, "operator_and_mg_setup_ms": setup_ms, "steps": steps,
        "grad_rel_error_vs_fp64": grad_err, "fp64_loss_rel_diff": abs(loss.value - loss64.value) / loss64.value,
        "fp64_iters": [int(its64[0]), int(its64[1])],
    }
    del prob, b, u, lam, uobs, dk, r
    torch.cuda.empty_cache()
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
    names = [f for f in args.forms.split(",") if f]
    for f in names:
        if f not in FORMS:
            raise SystemExit(f"unknown form {f}")
    headline = args.headline if args.headline in names else names[0]
    hist = np.zeros(WL["maxit"])

    def solve(mg, xbuf, tol=WL["tol"]):
        with torch.cuda.stream(ext):
            xbuf.zero_()
        it = C.c_int()
        ctx.check(L.mgldg_pcg_dev(ctx.h, mg.h, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(xbuf.data_ptr()), tol,
                                  WL["maxit"], C.byref(it), hist), "pcg")
        return it.value

    def timed(mg):
        # timed region: the solves as a user runs them (V-cycles replayed as
        # CUDA graphs); then the same steps again with per-kernel CUDA-event
        # timing on the library's stream (eager launches) for the breakdown
        for _ in range(args.warmup):
            solve(mg, x)
        torch.cuda.synchronize()
        ctx.sync()
        dist_barrier(ws)
        ctx.prof_reset()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        iters = [solve(mg, x) for _ in range(args.steps)]
        e1.record(ext)
        e1.synchronize()
        ctx.sync()
        ms = e0.elapsed_time(e1) / args.steps
        launches = ctx.prof()
        torch.cuda.synchronize()
        dist_barrier(ws)
        ctx.prof_reset()
        ctx.prof_enable(True)
        for _ in range(args.steps):
            solve(mg, x)
        prof = ctx.prof()
        # per multigrid level (-1: pcg's own products) of the profiled pass
        per_level = {}
        for kid, kname in enumerate(mgldg.K_NAMES):
            for lvl in range(-1, levels):
                nl, tl = ctx.prof_level(kid, lvl)
                if nl:
                    per_level.setdefault(kname, {})[lvl] = (nl, tl)
        ctx.prof_enable(False)
        prof = {k: (launches[k][0], prof[k][1]) for k in prof}
        prof["_per_level"] = per_level
        return dist_max(ms, ws), iters, prof

    mgs, setup_ms = {}, {}
    for name in names:
        relax, omega, prec = FORMS[name]
        t0 = time.perf_counter()
        mgs[name] = mgldg.Multigrid(ctx, prob.ops, prob.T, npre=WL["npre"], npost=WL["npost"],
                                    solver=mgldg.COARSE_DENSE, max_levels=levels, mean_project=0,
                                    relaxation=relax, omega=omega, precision=prec)
        setup_ms[name] = (time.perf_counter() - t0) * 1e3
    bh = b.cpu().numpy()
    results, profs = {}, {}
    clocks = Clocks(local)
    clocks.start()
    for name in names:
        ms, iters, prof = timed(mgs[name])
        per_level = prof.pop("_per_level")
        xs = x.cpu().numpy().copy()
        res = A.mv(xs, alpha=-1.0, beta=1.0, y=bh)
        results[name] = dict(ms=ms, iters=iters[-1], rel_residual=float(np.linalg.norm(res) / np.linalg.norm(bh)),
                             kernel_ms={k: round(v[1] / args.steps, 4) for k, v in prof.items() if v[0]},
                             launches_per_solve=int(sum(v[0] for v in prof.values()) / args.steps), x=xs)
        profs[name] = (prof, per_level)
    clk = clocks.stop()
    # FP64 reference solution (FP64 form to 1e-13) for each form's error
    ref_form = "fp64_gs" if "fp64_gs" in mgs else ("fp64_jacobi" if "fp64_jacobi" in mgs else None)
    xref = None
    if ref_form:
        solve(mgs[ref_form], x, tol=1e-13)
        ctx.sync()
        xref = x.cpu().numpy().copy()
    for name in names:
        xs = results[name].pop("x")
        if xref is not None:
            results[name]["rel_error_vs_fp64"] = float(np.linalg.norm(xs - xref) / np.linalg.norm(xref))

    # SpMV bandwidth (FP64, the outer CG operator)
    nbr, _, br, _, nnzb = A.info()
    s64 = nnzb * br * br * 8 + 4 * nnzb + 4 * (nbr + 1) + 2 * ndof * 8
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
    fp64_tf = fp64_peak_tflops(torch)

    # Roofline of the dominant kernel class of the headline form, taken on the
    # finest level (its launches carry the bytes; coarse-level launches are a
    # few us each and their event times include launch gaps).  Algorithmic
    # bytes per launch come from the level's actual matrix; time from CUDA
    # events on the library's stream in the profiled pass of the same steps.
    # traffic: dram__bytes_read.sum + dram__bytes_write.sum of the same kernel
    # from one ncu capture at 256x256 Q3 (DRAM bytes / algorithmic bytes, the
    # ratio below), scaled to this launch by its algorithmic bytes.
    NCU_TRAFFIC_RATIO = {("mixed_jacobi", "jacobi"): 418.508032 / 415.756292,
                         ("mixed16_jacobi", "jacobi"): 254.26816 / 249.815044}

    def kernel_roof(form, cls, key):
        _, _, prec = FORMS[form]
        prof_f, per_level_f = profs[form]
        if not key or 0 not in per_level_f.get(cls, {}):
            return None
        lb = level_bytes(mgs[form], levels - 1, 4 if prec in (1, 2) else 8, f16=prec == 2)
        n0, ms0 = per_level_f[cls][0]
        # a Gauss-Seidel launch is a pass of npre (= npost) sweeps, each
        # reading the level's blocks once; of the npre + npost Jacobi launches
        # per V-cycle the first starts from x = 0 and reads no operator
        bytes0 = lb[0][key] * (WL["npre"] if key == "gs" else 1)
        if key == "jacobi":
            nsw = WL["npre"] + WL["npost"]
            bytes0 = ((nsw - 1) * lb[0]["jacobi"] + lb[0]["jacobi0"]) / nsw
        achieved = bytes0 * n0 / (ms0 * 1e-3) / 1e9
        r = {"bound": "hbm", "form": form, "kernel": cls, "level": 0, "achieved": achieved, "peak": hbm,
             "unit": "GB/s", "frac": achieved / hbm, "traffic": None, "peak_kind": peak_kind, "launches": n0,
             "avg_launch_ms": ms0 / n0, "algorithmic_bytes_per_launch": bytes0,
             "all_levels": {"launches": prof_f[cls][0], "ms": prof_f[cls][1]}}
        ratio = NCU_TRAFFIC_RATIO.get((form, key))
        if ratio:
            r["traffic"] = bytes0 * ratio
            r["traffic_source"] = "ncu at 256x256 Q3, scaled by block rows"
        return r

    _, _, prec_h = FORMS[headline]
    prof, per_level = profs[headline]
    cls = max(prof, key=lambda k: prof[k][1])
    keymap = {"gauss_seidel": "gs", "jacobi": "jacobi", "spmv": "spmv"}
    roof = kernel_roof(headline, cls, keymap.get(cls)) or {
        "bound": "hbm", "kernel": cls, "achieved": None, "peak": hbm, "unit": "GB/s", "frac": None, "traffic": None,
        "peak_kind": peak_kind}
    roof_more = [r for r in (kernel_roof(f, c, keymap[c]) for f in names for c in ("jacobi", "spmv", "gauss_seidel")
                             if not (f == headline and c == cls)) if r]
    gpu_launches = int(sum(v[0] for v in prof.values()))
    results[headline]["per_level_ms"] = {k: {str(l): round(v[1] / args.steps, 4) for l, v in d.items()}
                                         for k, d in per_level.items()}

    # end to end through the C ABI's host-buffer call (mgldg_pcg, the
    # reference's pcg(A, b, x, ...) with x in/out): pinned host b and x ->
    # device, solve, x -> host, every step
    bpin = torch.empty(ndof, dtype=torch.float64, pin_memory=True)
    bpin.copy_(b.cpu())
    xpin = torch.zeros(ndof, dtype=torch.float64, pin_memory=True)
    bnp, xnp = bpin.numpy(), xpin.numpy()
    lib = mgldg.lib()
    it_e2e = C.c_int()
    hist_e2e = np.zeros(WL["maxit"])
    e2e = []
    for k in range(args.warmup + args.steps):
        xnp[:] = 0.0
        dist_barrier(ws)
        t0 = time.perf_counter()
        ctx.check(lib.mgldg_pcg(ctx.h, mgs[headline].h, A.h, bnp, xnp, WL["tol"], WL["maxit"], C.byref(it_e2e),
                                hist_e2e), "pcg")
        dt = time.perf_counter() - t0
        if k >= args.warmup:
            e2e.append(dt * 1e3)
    e2e_ms = dist_max(float(np.mean(e2e)), ws)

    batched = None
    del mgs
    import gc
    gc.collect()
    config1 = run_config1(args, ctx, ext, torch, local, ws) if args.config1 else None
    gc.collect()
    batched_tc = None
    if args.batched > 0:
        batched = run_batched(args, ctx, ext, torch, local, ws)
        gc.collect()
        batched_tc = run_batched(args, ctx, ext, torch, local, ws, precision=mgldg.PREC_MIXED_TF32)
    gc.collect()
    unstructured = run_unstructured(args, ctx, ext, torch, local, ws) if args.disk_h > 0 else None
    gc.collect()
    adjoint = run_adjoint(args, ctx, ext, torch, local, ws) if args.ball_h > 0 else None

    speedup = {}
    for sm in ("gs", "jacobi"):
        if f"fp64_{sm}" in results and f"mixed_{sm}" in results:
            speedup[sm] = results[f"fp64_{sm}"]["ms"] / results[f"mixed_{sm}"]["ms"]
    if "fp64_jacobi" in results and "mixed16_jacobi" in results:
        speedup["jacobi_f16"] = results["fp64_jacobi"]["ms"] / results["mixed16_jacobi"]["ms"]
    f64 = [results[f]["ms"] for f in results if f.startswith("fp64")]
    mx = [results[f]["ms"] for f in results if f.startswith("mixed")]
    if f64 and mx:
        speedup["best_mixed_vs_best_fp64"] = min(f64) / min(mx)

    relax_h = FORMS[headline][0]
    # compact per-form summary (kept near the end of the line)
    forms_short = {f: {"ms": round(r["ms"], 3), "iters": r["iters"],
                       "rel_error_vs_fp64": r.get("rel_error_vs_fp64"), "kernel_ms": r["kernel_ms"]}
                   for f, r in results.items()}
    line = {
        "metric": METRIC, "value": results[headline]["ms"], "unit": "ms", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": results[headline]["ms"], "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPE[prec_h],
        "data": f"synthetic: seeded 8-Gaussian forcing (seed {WL['seed']}), homogeneous Dirichlet",
        "config": run_config(n, P, levels, relax_h),
        "form": FORM_TEXT[headline],
        "parallelism": "replicas" if ws > 1 else "single GPU",
        "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": 2 * ndof * 8, "d2h_bytes_per_step": ndof * 8,
                "api": "mgldg_pcg (host buffers, pinned)"},
        "roofline": roof,
        "gpu_launches": gpu_launches,
        "clocks": clk,
        "roofline_more": roof_more,
        "per_level_ms": results[headline].pop("per_level_ms"),
        "spmv": {"precision": "fp64", "ms": spmv_ms, "gbs": s64 / (spmv_ms * 1e-3) / 1e9, "bytes": s64,
                 "frac_of_hbm": s64 / (spmv_ms * 1e-3) / 1e9 / hbm,
                 "fp64_tflops": 2 * nnzb * br * br / (spmv_ms * 1e-3) / 1e12,
                 "fp64_peak_tflops_cublas": fp64_tf},
        "setup_ms": {"problem_build": t_build * 1e3, **setup_ms},
        "config1": config1,
        "batched": batched,
        "batched_tensor_cores": batched_tc,
        "unstructured": unstructured,
        "adjoint": adjoint,
        "forms": forms_short,
        "mixed_vs_fp64_speedup": speedup,
    }
    return line, results


def run_config(n, P, levels, relax):
    """The workload as both arms name it (the reference arm runs the same
    problem, smoother and tolerance in FP64 on the host)."""
    return {"workload": workload_name(n, P, levels), "smoother": SMOOTHER_TEXT[relax], "l2": L2_TEXT}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=WL["n"])
    ap.add_argument("--levels", type=int, default=WL["levels"])
    ap.add_argument("--forms", default="mixed_jacobi,fp64_jacobi,mixed_gs,fp64_gs,mixed16_jacobi")
    ap.add_argument("--headline", default="mixed_jacobi")
    ap.add_argument("--batched", type=int, default=64, help="right-hand sides of the multi-RHS line (0: skip)")
    ap.add_argument("--batched-n", type=int, default=512, help="mesh side of the uniform multi-RHS mesh")
    ap.add_argument("--batched-mesh", default="adaptive", choices=["adaptive", "uniform"])
    ap.add_argument("--disk-h", type=float, default=0.004, help="mesh size of the single unstructured disk (0: skip "
                    "the unstructured lines)")
    ap.add_argument("--disk-batch", type=int, default=48, help="meshes in the uneven batch (0: skip the line)")
    ap.add_argument("--config1", type=int, default=1, help="time the 32x32 Q2 reference-method line (0: skip)")
    ap.add_argument("--ball-h", type=float, default=0.026, help="tetrahedral ball mesh size of the adjoint line (0: skip)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline")
    ap.add_argument("--cpu-smoothers", default="jacobi",
                    help="smoothers of the CPU oracle's full solves (comma list of jacobi, gs; the first is the "
                         "reported value)")
    ap.add_argument("--cpu-oracle", default=None, help=argparse.SUPPRESS)
    ap.add_argument("--vcycle", default="mixed", choices=["mixed16", "mixed"],
                    help="V-cycle form of the unstructured and adjoint lines (their blocks are below 16 x 16, "
                         "which the FP16 copy does not cover)")
    args = ap.parse_args()
    if args.cpu_oracle is not None:
        # child process of the CPU baseline: full oracle solves, one JSON line
        res = [cpu_oracle_solve(args.n, WL["P"], args.levels, sm, WL["tol"], WL["seed"])
               for sm in args.cpu_oracle.split(",") if sm]
        print(json.dumps(res), flush=True)
        return
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        # the reference's CPU solver (the oracle port), one full solve per
        # smoother on the host; under torchrun only rank 0 works
        if rank == 0:
            smoothers = [sm for sm in args.cpu_smoothers.split(",") if sm]
            res = [cpu_oracle_solve(args.n, WL["P"], args.levels, sm, WL["tol"], WL["seed"]) for sm in smoothers]
            cb = cpu_baseline_line(res, args.n, WL["P"])
            v = cb["value"]
            relax = REF_SMOOTHERS[smoothers[0]][0]
            line = {"metric": METRIC, "value": v, "unit": "ms", "n_gpus": ws, "steps": 1, "warmup": 0,
                    "ms_per_step": v, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
                    "dtype": "f64", "data": f"synthetic: seeded 8-Gaussian forcing (seed {WL['seed']}), "
                                            f"homogeneous Dirichlet",
                    "config": run_config(args.n, WL["P"], args.levels, relax),
                    "form": "reference method on the host: FP64 MG-PCG, serial (one full solve per smoother)",
                    "impl": "reference",
                    "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
                    "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                    "runs": res}
            print(json.dumps(line), flush=True)
        return
    t0 = time.perf_counter()
    cpu_proc = start_cpu_baseline(args) if (ws == 1 and not args.no_cpu) else None
    line, results = run_gpu(args, ws, rank, local)
    print(f"[bench] GPU part {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
    if rank == 0:
        if cpu_proc is not None:
            res = finish_cpu_baseline(cpu_proc)
            if res:
                line["cpu_baseline"] = cpu_baseline_line(res, args.n, WL["P"])
        print(f"[bench] total {time.perf_counter() - t0:.1f} s", file=sys.stderr, flush=True)
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()

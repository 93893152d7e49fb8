"""GPU test of mgldg_cg_noalloc_dev, the allocation-free CG entry point.

Some callers cannot allocate device memory while they solve (their
framework's caching allocator owns the GPU's memory, or they run under a
memory budget fixed at start-up); mgldg_cg_noalloc_dev serves them from a
fixed ~4.1 MiB device array instead of allocating work vectors per call.
This file is collected last so that a run stopping at the first failure has
already run every other test.  It compares the new entry point, through the
C ABI, with the existing unpreconditioned path mgldg_pcg_dev(ctx, NULL, ...)
on two calls in a row (the second call must not see the first call's
leftovers), from a zero and from a nonzero starting x; checks that the
device's free memory does not change across calls after the first (which
looks up the array's address); and checks the refusals (too many unknowns,
maxit above 1024) and the breakdown report for a non-finite right-hand side.
"""
import ctypes as C

import numpy as np
import pytest

import mgldg

pytestmark = pytest.mark.gpu

TOL, MAXIT = 1e-8, 1000


def _dev(torch, n):
    return torch.zeros(n, dtype=torch.float64, device="cuda:0")


def _call(ctx, fn_name, A, b, x, maxit=MAXIT):
    hist = np.zeros(max(1, maxit))
    it = C.c_int()
    L = mgldg.lib()
    if fn_name == "pcg":
        rc = L.mgldg_pcg_dev(ctx.h, None, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), TOL, maxit,
                             C.byref(it), hist)
    else:
        rc = L.mgldg_cg_noalloc_dev(ctx.h, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), TOL, maxit,
                                    C.byref(it), hist)
    return rc, it.value, hist


def _solve(ctx, fn_name, A, b, x):
    rc, it, hist = _call(ctx, fn_name, A, b, x)
    ctx.check(rc, fn_name)
    ctx.sync()
    return x.cpu().numpy().copy(), hist[:it].copy()


def _problem(ctx, torch):
    prob = mgldg.CartesianProblem(ctx, 4, 16)          # 16 x 16 Q3: 4,096 unknowns
    b = _dev(torch, prob.ndof)
    ctx.check(mgldg.lib().mgldg_problem_rhs_gaussian_dev(ctx.h, prob.h, 1001, C.c_void_p(b.data_ptr())), "rhs")
    ctx.sync()
    return prob, b


def test_noalloc_cg_matches_existing_entry_point(ctx):
    torch = pytest.importorskip("torch")
    prob, b = _problem(ctx, torch)
    A, n = prob.ops.A, prob.ndof
    x_ref, h_ref = _solve(ctx, "pcg", A, b, _dev(torch, n))
    assert len(h_ref) > 10
    free = []
    for call in range(3):                              # calls in a row share the scratch
        x = _dev(torch, n)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(0)[0])
        x_new, h_new = _solve(ctx, "noalloc", A, b, x)
        assert len(h_new) == len(h_ref), call
        assert np.abs(x_new - x_ref).max() <= 1e-12 * np.abs(x_ref).max(), call
        assert np.abs(h_new - h_ref).max() <= 1e-12 * h_ref[0], call
    torch.cuda.synchronize()
    free.append(torch.cuda.mem_get_info(0)[0])
    # the first call may load the library's device code and look up the
    # array; later calls leave the device's free memory exactly as it was
    assert free[1] == free[2] == free[3], free


def test_noalloc_cg_nonzero_start_matches(ctx):
    torch = pytest.importorskip("torch")
    prob, b = _problem(ctx, torch)
    A, n = prob.ops.A, prob.ndof
    x0 = torch.from_numpy(np.random.default_rng(3).standard_normal(n)).to("cuda:0")
    x_ref, h_ref = _solve(ctx, "pcg", A, b, x0.clone())
    for call in range(2):
        x_new, h_new = _solve(ctx, "noalloc", A, b, x0.clone())
        assert len(h_new) == len(h_ref), call
        assert np.abs(x_new - x_ref).max() <= 1e-12 * np.abs(x_ref).max(), call
        assert np.abs(h_new - h_ref).max() <= 1e-12 * h_ref[0], call


def test_noalloc_cg_reports_breakdown_like_pcg(ctx):
    torch = pytest.importorskip("torch")
    prob, b = _problem(ctx, torch)
    A, n = prob.ops.A, prob.ndof
    b[7] = float("nan")
    for fn in ("pcg", "noalloc"):
        x = _dev(torch, n)
        rc, it, _ = _call(ctx, fn, A, b, x)
        assert rc == mgldg.ERR_BREAKDOWN, fn
        assert it == 0, fn
        ctx.sync()
        assert torch.count_nonzero(x).item() == 0, fn
    # the context and the scratch stay usable
    b[7] = 0.0
    x_ref, h_ref = _solve(ctx, "pcg", A, b, _dev(torch, n))
    x_new, h_new = _solve(ctx, "noalloc", A, b, _dev(torch, n))
    assert len(h_new) == len(h_ref)
    assert np.abs(x_new - x_ref).max() <= 1e-12 * np.abs(x_ref).max()


def test_noalloc_cg_rejects_oversized_systems(ctx):
    torch = pytest.importorskip("torch")
    prob = mgldg.CartesianProblem(ctx, 4, 128)         # 262,144 unknowns > 131,072
    b = _dev(torch, prob.ndof)
    x = _dev(torch, prob.ndof)
    rc, _, _ = _call(ctx, "noalloc", prob.ops.A, b, x, maxit=4)
    assert rc == mgldg.ERR_ARG
    assert "131072" in mgldg.lib().mgldg_last_error(ctx.h).decode()


def test_noalloc_cg_rejects_large_maxit(ctx):
    torch = pytest.importorskip("torch")
    prob, b = _problem(ctx, torch)
    rc, _, _ = _call(ctx, "noalloc", prob.ops.A, b, _dev(torch, prob.ndof), maxit=1025)
    assert rc == mgldg.ERR_ARG
    assert "1024" in mgldg.lib().mgldg_last_error(ctx.h).decode()

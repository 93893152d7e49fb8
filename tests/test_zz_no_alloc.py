"""GPU test of mgldg_cg_noalloc_dev, the allocation-free CG entry point.

Some callers cannot allocate device memory while they solve (their
framework's caching allocator owns the GPU's memory, or they run under a
memory budget fixed at start-up); mgldg_cg_noalloc_dev serves them from a
fixed ~4.1 MiB device array instead of allocating work vectors per call.
This file is collected last so that a run stopping at the first failure has
already run every other test.  It compares the new entry point, through the
C ABI, with the existing unpreconditioned path mgldg_pcg_dev(ctx, NULL, ...)
on two calls in a row (the second call must not see the first call's
leftovers), and checks that an oversized system is refused.
"""
import ctypes as C

import numpy as np
import pytest

import mgldg

pytestmark = pytest.mark.gpu

TOL, MAXIT = 1e-8, 1000


def _dev(torch, n):
    return torch.zeros(n, dtype=torch.float64, device="cuda:0")


def _solve(ctx, fn_name, A, b, x, with_mg=False):
    hist = np.zeros(MAXIT)
    it = C.c_int()
    L = mgldg.lib()
    if fn_name == "pcg":
        rc = L.mgldg_pcg_dev(ctx.h, None, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), TOL, MAXIT,
                             C.byref(it), hist)
    else:
        rc = L.mgldg_cg_noalloc_dev(ctx.h, A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), TOL, MAXIT,
                                    C.byref(it), hist)
    ctx.check(rc, fn_name)
    ctx.sync()
    return x.cpu().numpy().copy(), hist[:it.value].copy()


def test_noalloc_cg_matches_existing_entry_point(ctx):
    torch = pytest.importorskip("torch")
    prob = mgldg.CartesianProblem(ctx, 4, 16)          # 16 x 16 Q3: 4,096 unknowns
    A = prob.ops.A
    n = prob.ndof
    b = _dev(torch, n)
    ctx.check(mgldg.lib().mgldg_problem_rhs_gaussian_dev(ctx.h, prob.h, 1001, C.c_void_p(b.data_ptr())), "rhs")
    ctx.sync()
    x_ref, h_ref = _solve(ctx, "pcg", A, b, _dev(torch, n))
    assert len(h_ref) > 10
    for call in range(2):                              # two calls in a row share the scratch
        torch.cuda.synchronize()
        x_new, h_new = _solve(ctx, "noalloc", A, b, _dev(torch, n))
        assert len(h_new) == len(h_ref), call
        assert np.abs(x_new - x_ref).max() <= 1e-12 * np.abs(x_ref).max(), call
        assert np.abs(h_new - h_ref).max() <= 1e-12 * h_ref[0], call


def test_noalloc_cg_rejects_oversized_systems(ctx):
    torch = pytest.importorskip("torch")
    prob = mgldg.CartesianProblem(ctx, 4, 128)         # 262,144 unknowns > 131,072
    b = _dev(torch, prob.ndof)
    x = _dev(torch, prob.ndof)
    hist = np.zeros(4)
    it = C.c_int()
    rc = mgldg.lib().mgldg_cg_noalloc_dev(ctx.h, prob.ops.A.h, C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()),
                                          TOL, 4, C.byref(it), hist)
    assert rc == mgldg.ERR_ARG
    assert "131072" in mgldg.lib().mgldg_last_error(ctx.h).decode()

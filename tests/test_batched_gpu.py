"""GPU parity of the many-right-hand-side path (block SpMM, multi-RHS
V-cycle, lock-step block PCG) against the CPU oracle, column by column.

Each column of a batched solve must reproduce the oracle's single-RHS pcg
(krylov.h:22-68) for that right-hand side: the same iteration count, every
printed ||r_k|| within 1e-12 ||b|| (and within 1e-10 of itself while above
1e-4 ||b||), the solution within 1e-10.  SpMM columns match the oracle SpMV
within 1e-13 of the largest entry.
"""
import ctypes as C

import numpy as np
import pytest

import mgldg
import oracle_py as O

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float64)).to("cuda")


@pytest.mark.parametrize("P,k", [(3, 1), (3, 5), (4, 32), (4, 64), (3, 96), (2, 64)])
def test_spmm_matches_oracle_columns(ctx, P, k):
    torch = pytest.importorskip("torch")
    n = 16
    prob = mgldg.CartesianProblem(ctx, P, n)
    pr = O.Problem(P, 1.0 / n)
    A = pr.op(O.OP_A)
    rng = np.random.default_rng(k)
    X = rng.standard_normal((prob.ndof, k))
    Y0 = rng.standard_normal((prob.ndof, k))
    dX, dY = _dev(torch, X), _dev(torch, Y0)
    torch.cuda.synchronize()
    rc = mgldg.lib().mgldg_bsr_mm_dev(ctx.h, -0.5, prob.ops.A.h, k, C.c_void_p(dX.data_ptr()), 2.0,
                                      C.c_void_p(dY.data_ptr()))
    ctx.check(rc, "mm")
    ctx.sync()
    Y = dY.cpu().numpy()
    ref = np.stack([-0.5 * A.matvec(X[:, c]) + 2.0 * Y0[:, c] for c in range(k)], axis=1)
    assert np.abs(Y - ref).max() <= 1e-14 * np.abs(ref).max() * 10


def _rhs(pr_seeds, P, n):
    cols = []
    for s in pr_seeds:
        cols.append(O.Problem(P, 1.0 / n, tau0=n, tauD=n, seed=s).rhs())
    return np.stack(cols, axis=1)


def assert_history_parity(hg, hr, bnorm):
    # same count; every ||r_k|| within 1e-12 ||b||; while ||r_k|| > 1e-3 ||b||
    # also within 1e-10 of itself (further down, rounding differences of a
    # few 1e-14 ||b|| from the SpMM's summation order, which is not the
    # single-RHS kernel's, are a larger fraction of ||r_k||)
    assert len(hg) == len(hr)
    assert np.all(np.isfinite(hg))
    assert np.abs(hg - hr).max() <= 1e-12 * bnorm
    big = hr > 1e-3 * bnorm
    assert np.max(np.abs(hg - hr)[big] / hr[big]) <= 1e-10


@pytest.mark.parametrize("mean_project", [1, 0])
def test_batched_pcg_columns_match_oracle(ctx, mean_project):
    # 32x32 Q2, 32 -> 16 -> 8 -> 4 with a dense coarsest solve, V(2,2) Jacobi
    P, n, nlev, omega = 3, 32, 4, 0.7
    seeds = [1001, 1002, 1003, 1004, 1005]
    B = _rhs(seeds, P, n)
    prob = mgldg.CartesianProblem(ctx, P, n, tau0=float(n), tauD=float(n))
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI, omega=omega, npre=2, npost=2,
                         solver=mgldg.COARSE_DENSE, max_levels=nlev, mean_project=mean_project)
    X, its, hist = mgldg.pcg_batched(ctx, prob.ops.A, B, precon=mg, tol=1e-10, maxit=200)
    for c, s in enumerate(seeds):
        pr = O.Problem(P, 1.0 / n, tau0=n, tauD=n, seed=s)
        omg = O.Multigrid(pr, relaxation=O.RELAX_JACOBI, omega=omega, npre=2, npost=2, solver=O.COARSE_DENSE,
                          nlevels=nlev, mean_project=mean_project)
        xr, hr, _ = pr.pcg(B[:, c], mg=omg, tol=1e-10)
        assert its[c] == len(hr)
        assert_history_parity(hist[c], hr, np.linalg.norm(B[:, c]))
        assert np.abs(X[:, c] - xr).max() <= 1e-10 * np.abs(xr).max()


def test_batched_vcycle_matches_oracle(ctx):
    torch = pytest.importorskip("torch")
    P, n = 4, 16
    prob = mgldg.CartesianProblem(ctx, P, n)
    pr = O.Problem(P, 1.0 / n)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI, omega=0.8, npre=2, npost=2)
    omg = O.Multigrid(pr, relaxation=O.RELAX_JACOBI, omega=0.8, npre=2, npost=2)
    k = 7
    rng = np.random.default_rng(2)
    B = rng.standard_normal((prob.ndof, k))
    X0 = rng.standard_normal((prob.ndof, k))
    dB, dX = _dev(torch, B), _dev(torch, X0)
    torch.cuda.synchronize()
    ctx.check(mgldg.lib().mgldg_mg_vcycle_batched_dev(ctx.h, mg.h, k, C.c_void_p(dB.data_ptr()),
                                                      C.c_void_p(dX.data_ptr())), "vcycle_batched")
    ctx.sync()
    X = dX.cpu().numpy()
    for c in range(k):
        ref = omg.vcycle(B[:, c], X0[:, c])
        assert np.abs(X[:, c] - ref).max() <= 1e-12 * np.abs(ref).max()


def test_batched_mixed_matches_single_rhs(ctx):
    P, n = 4, 32
    prob = mgldg.CartesianProblem(ctx, P, n)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2,
                         solver=mgldg.COARSE_DENSE, max_levels=4, mean_project=0, precision=mgldg.PREC_MIXED)
    k = 64
    B = np.stack([prob.rhs_gaussian(3000 + c) for c in range(k)], axis=1)
    X, its, hist = mgldg.pcg_batched(ctx, prob.ops.A, B, precon=mg, tol=1e-10, maxit=200)
    fp64 = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2,
                           solver=mgldg.COARSE_DENSE, max_levels=4, mean_project=0)
    for c in (0, 17, 63):
        xs, hs = mgldg.pcg(ctx, prob.ops.A, B[:, c], precon=mg, tol=1e-10)
        xd, _ = mgldg.pcg(ctx, prob.ops.A, B[:, c], precon=fp64, tol=1e-12)
        # FP32 V-cycles in another summation order: the same solve up to the
        # stopping tolerance (on r.z), not bit for bit
        assert abs(its[c] - len(hs)) <= 1
        assert hist[c][-1] <= 10 * hs[-1]
        assert np.abs(X[:, c] - xs).max() <= 1e-8 * np.abs(xs).max()
        assert np.abs(X[:, c] - xd).max() <= 1e-8 * np.abs(xd).max()
    tiles = mgldg.batch_tiles(mg, 0)
    assert all(t in (32, 64, 128) for t in tiles)


@pytest.mark.parametrize("P,n,k", [(3, 32, 64), (4, 16, 20), (3, 16, 130)])
def test_batched_tensor_core_form(ctx, P, n, k):
    # MGLDG_PREC_MIXED_TF32: the multi-RHS V-cycle's level products on the
    # tensor cores (3xTF32 split products, FP32 accumulation).  One V-cycle
    # must match the FP32 CUDA-core V-cycle to FP32 rounding, and the block
    # PCG must reach the FP64 solution of every column within 1e-10 in about
    # as many iterations; block sizes 9 (Q2) and 16 (Q3), 64-column tiles
    # full, partial (20) and over two tiles (130)
    torch = pytest.importorskip("torch")
    prob = mgldg.CartesianProblem(ctx, P, n)
    kw = dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2, solver=mgldg.COARSE_DENSE,
              max_levels=4, mean_project=0)
    mg32 = mgldg.Multigrid(ctx, prob.ops, prob.T, precision=mgldg.PREC_MIXED, **kw)
    mgtc = mgldg.Multigrid(ctx, prob.ops, prob.T, precision=mgldg.PREC_MIXED_TF32, **kw)
    rng = np.random.default_rng(k)
    Bv = rng.standard_normal((prob.ndof, k))
    outs = []
    for mg in (mg32, mgtc):
        dB, dX = _dev(torch, Bv), _dev(torch, np.zeros_like(Bv))
        torch.cuda.synchronize()
        ctx.check(mgldg.lib().mgldg_mg_vcycle_batched_dev(ctx.h, mg.h, k, C.c_void_p(dB.data_ptr()),
                                                          C.c_void_p(dX.data_ptr())), "vcycle_batched")
        ctx.sync()
        outs.append(dX.cpu().numpy())
    assert np.abs(outs[1] - outs[0]).max() <= 1e-5 * np.abs(outs[0]).max()
    B = np.stack([prob.rhs_gaussian(3000 + c) for c in range(k)], axis=1)
    X32, its32, _ = mgldg.pcg_batched(ctx, prob.ops.A, B, precon=mg32, tol=1e-11, maxit=200)
    Xtc, itstc, _ = mgldg.pcg_batched(ctx, prob.ops.A, B, precon=mgtc, tol=1e-11, maxit=200)
    assert np.all(np.abs(itstc - its32) <= 2)
    fp64 = mgldg.Multigrid(ctx, prob.ops, prob.T, **kw)
    for c in (0, k // 2, k - 1):
        xd, _ = mgldg.pcg(ctx, prob.ops.A, B[:, c], precon=fp64, tol=1e-13)
        assert np.linalg.norm(Xtc[:, c] - xd) <= 1e-10 * np.linalg.norm(xd)


def test_frozen_and_zero_columns(ctx):
    P, n = 3, 16
    prob = mgldg.CartesianProblem(ctx, P, n)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI, omega=0.8, npre=2, npost=2,
                         mean_project=0)
    b = prob.rhs_gaussian(11)
    B = np.stack([b, np.zeros_like(b), 1e-3 * b], axis=1)
    X, its, hist = mgldg.pcg_batched(ctx, prob.ops.A, B, precon=mg, tol=1e-10, maxit=200)
    assert its[1] == 0 and np.all(X[:, 1] == 0)
    assert its[0] == its[2] > 0
    assert np.allclose(X[:, 2], 1e-3 * X[:, 0], rtol=0, atol=1e-12 * np.abs(X[:, 0]).max())
    xs, hs = mgldg.pcg(ctx, prob.ops.A, b, precon=mg, tol=1e-10)
    assert its[0] == len(hs)
    assert np.abs(X[:, 0] - xs).max() <= 1e-12 * np.abs(xs).max()


def test_batched_rejects_gauss_seidel_and_bad_k(ctx):
    prob = mgldg.CartesianProblem(ctx, 3, 8)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T)   # reference defaults: Gauss-Seidel
    B = np.ones((prob.ndof, 2))
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.pcg_batched(ctx, prob.ops.A, B, precon=mg)
    assert e.value.code == mgldg.ERR_UNSUPPORTED
    mgj = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI)
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.pcg_batched(ctx, prob.ops.A, np.ones((prob.ndof, 2000)), precon=mgj, maxit=1)
    assert e.value.code == mgldg.ERR_ARG

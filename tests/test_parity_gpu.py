"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle.

Tolerances (FP64 plain form): operators and single kernels to 1e-13 relative
to the largest entry; V-cycles to 1e-12; PCG residual histories to 1e-12
relative to the initial residual norm ||r_0|| (later entries are tiny, so a
relative-per-entry bound would measure round-off, not parity); solutions to
1e-10 relative.  Integer setup (patterns, orders) must be bit-exact.
"""
import numpy as np
import pytest

import mgldg
import oracle_py as O

pytestmark = pytest.mark.gpu


def to_gpu(ctx, csr):
    return mgldg.SparseBlockMatrix.from_csr(ctx, csr.nbr, csr.nbc, csr.br, csr.bc, csr.row_ptr, csr.col_idx, csr.vals)


def ops_from_oracle(ctx, pr):
    M, G0, G1, T = (to_gpu(ctx, pr.op(w)) for w in (O.OP_M, O.OP_G0, O.OP_G1, O.OP_T))
    ops = mgldg.LDGOperators.create(ctx, M, [G0, G1], T)
    ops.construct_laplacian()
    return ops


def assert_same_bsr(gpu, csr, rtol):
    rp, ci, v = gpu.download()
    assert np.array_equal(rp, csr.row_ptr)
    assert np.array_equal(ci, csr.col_idx)
    scale = max(1.0, np.abs(csr.vals).max())
    err = np.abs(v - csr.vals).max() / scale
    assert err <= rtol, err


def test_spmv_2x2_known_answer(ctx):
    rp = np.array([0, 2, 4], np.int32)
    ci = np.array([0, 1, 0, 1], np.int32)
    vals = np.array([[1, 2, 3, 4], [9, 10, 11, 12], [4, 6, 7, 8], [13, 14, 15, 8]], float)
    A = mgldg.SparseBlockMatrix.from_csr(ctx, 2, 2, 2, 2, rp, ci, vals)
    assert np.array_equal(A.mv(np.ones(4)), [22.0, 30.0, 37.0, 38.0])


@pytest.mark.parametrize("P,n", [(2, 8), (3, 32), (4, 16), (5, 8)])
def test_spmv_matches_oracle(ctx, P, n):
    pr = O.Problem(P, 1 / n, seed=7)
    Acsr = pr.op(O.OP_A)
    A = to_gpu(ctx, Acsr)
    rng = np.random.default_rng(P * 100 + n)
    x = rng.standard_normal(pr.ndof)
    y0 = rng.standard_normal(pr.ndof)
    ref = pr.mv(O.OP_A, x, alpha=-1.0, beta=1.0, y=y0)
    got = A.mv(x, alpha=-1.0, beta=1.0, y=y0)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    assert np.abs(A.mv(x) - pr.mv(O.OP_A, x)).max() <= 1e-13 * np.abs(ref).max()


def test_spmv_empty_and_ragged_rows(ctx):
    # rows without blocks, unsorted columns, duplicate entries (summed)
    rp = np.array([0, 0, 3, 3, 4], np.int32)
    ci = np.array([2, 0, 2, 1], np.int32)
    rng = np.random.default_rng(1)
    vals = rng.standard_normal((4, 3, 3))
    A = mgldg.SparseBlockMatrix.from_csr(ctx, 4, 3, 3, 3, rp, ci, vals)
    D = np.zeros((12, 9))
    for i in range(4):
        for k in range(rp[i], rp[i + 1]):
            j = ci[k]
            D[3 * i:3 * i + 3, 3 * j:3 * j + 3] += vals[k]
    x = rng.standard_normal(9)
    assert np.allclose(A.mv(x), D @ x, rtol=0, atol=1e-13)
    z = rng.standard_normal(12)
    assert np.allclose(A.mv_t(z), D.T @ z, rtol=0, atol=1e-13)
    assert A.info()[4] == 3


def test_mv_t_matches_oracle(ctx):
    pr = O.Problem(3, 1 / 16)
    T = pr.hierarchy()[0]
    Tg = to_gpu(ctx, T)
    rng = np.random.default_rng(5)
    r = rng.standard_normal(T.nbr * T.br)
    ref = T.todense().T @ r
    assert np.abs(Tg.mv_t(r) - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("P", [2, 3])
def test_construct_laplacian_matches_oracle(ctx, P):
    pr = O.Problem(P, 1 / 16, seed=11)
    ops = ops_from_oracle(ctx, pr)
    assert_same_bsr(ops.A, pr.op(O.OP_A), 1e-13)


def test_construct_laplacian_hanging_faces(ctx):
    pr = O.Problem(3, 1 / 4, refine=O.REFINE_REF_ADAPTIVE)
    ops = ops_from_oracle(ctx, pr)
    assert_same_bsr(ops.A, pr.op(O.OP_A), 1e-13)


@pytest.mark.parametrize("P,n", [(2, 32), (3, 16), (4, 8)])
def test_cartesian_builder_matches_oracle(ctx, P, n):
    prob = mgldg.CartesianProblem(ctx, P, n, tau0=float(n), tauD=float(n))
    pr = O.Problem(P, 1 / n, tau0=n, tauD=n, seed=1001)
    for which in (O.OP_M, O.OP_G0, O.OP_G1, O.OP_T, O.OP_A):
        assert_same_bsr(prob.ops.get(which), pr.op(which), 1e-14 if which != O.OP_A else 1e-13)
    hier = pr.hierarchy()
    assert prob.nT == len(hier)
    for Tg, Tc in zip(prob.T, hier):
        assert_same_bsr(Tg, Tc, 1e-15)
    b = prob.rhs_gaussian(1001)
    ref = pr.rhs()
    assert np.abs(b - ref).max() <= 1e-13 * np.abs(ref).max()


@pytest.mark.parametrize("restriction", [mgldg.RESTRICT_RATRAT, mgldg.RESTRICT_RAT])
def test_galerkin_levels_match_oracle(ctx, restriction):
    pr = O.Problem(3, 1 / 16, seed=3)
    ops = ops_from_oracle(ctx, pr)
    T = [to_gpu(ctx, t) for t in pr.hierarchy()]
    mg = mgldg.Multigrid(ctx, ops, T, restriction=restriction, npre=2, npost=2)
    omg = O.Multigrid(pr, restriction=restriction, npre=2, npost=2)
    assert mg.nlevels == omg.nlevels == 5
    for l in range(1, mg.nlevels):
        assert_same_bsr(mg.level_op(l, O.OP_A), omg.level_op(l, O.OP_A), 1e-12)
        if restriction == mgldg.RESTRICT_RATRAT:
            for w in (O.OP_M, O.OP_G0, O.OP_G1, O.OP_T):
                assert_same_bsr(mg.level_op(l, w), omg.level_op(l, w), 1e-12)


@pytest.mark.parametrize("relax", [mgldg.RELAX_GAUSS_SEIDEL, mgldg.RELAX_JACOBI])
def test_smoothers_match_oracle(ctx, relax):
    pr = O.Problem(3, 1 / 16, seed=5)
    ops = ops_from_oracle(ctx, pr)
    T = [to_gpu(ctx, t) for t in pr.hierarchy()]
    mg = mgldg.Multigrid(ctx, ops, T, relaxation=relax, omega=0.8, npre=2, npost=2)
    omg = O.Multigrid(pr, relaxation=relax, omega=0.8, npre=2, npost=2)
    rng = np.random.default_rng(9)
    for l in range(mg.nlevels - 1):
        n = omg.level_op(l, O.OP_A).nbr * pr.npl
        b, x0 = rng.standard_normal(n), rng.standard_normal(n)
        for rev in (False, True):
            ref = omg.relax(l, 3, rev, b, x0)
            got = mg.relax(l, 3, rev, b, x0)
            assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max(), (l, rev)


@pytest.mark.parametrize("solver,nlev", [(mgldg.COARSE_CHOLESKY, 0), (mgldg.COARSE_DENSE, 4),
                                         (mgldg.COARSE_RELAXATION, 3)])
def test_vcycle_matches_oracle(ctx, solver, nlev):
    pr = O.Problem(3, 1 / 16, seed=21)
    ops = ops_from_oracle(ctx, pr)
    T = [to_gpu(ctx, t) for t in pr.hierarchy()]
    mg = mgldg.Multigrid(ctx, ops, T, npre=2, npost=2, solver=solver, max_levels=nlev)
    omg = O.Multigrid(pr, npre=2, npost=2, solver=solver, nlevels=nlev)
    b = pr.rhs()
    rng = np.random.default_rng(2)
    x0 = rng.standard_normal(pr.ndof)
    ref = omg.vcycle(b, x0)
    got = mg.vcycle(b, x0)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_vcycle_matrix_8x8(ctx):
    # multigrid.h:386-400: the V-cycle applied to unit vectors, column by column
    pr = O.Problem(2, 1 / 8, seed=1)
    ops = ops_from_oracle(ctx, pr)
    T = [to_gpu(ctx, t) for t in pr.hierarchy()]
    mg = mgldg.Multigrid(ctx, ops, T)
    omg = O.Multigrid(pr)
    n = pr.ndof
    for i in range(0, n, 37):
        e = np.zeros(n)
        e[i] = 1
        ref = omg.vcycle(e, np.zeros(n))
        got = mg.vcycle(e, np.zeros(n))
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def pcg_case(ctx, P, n, nlev, relax, omega, tol=1e-10, npre=2, npost=2, seed=1001):
    pr = O.Problem(P, 1 / n, tau0=n, tauD=n, seed=seed)
    solver = mgldg.COARSE_CHOLESKY if nlev == 0 else mgldg.COARSE_DENSE
    omg = O.Multigrid(pr, relaxation=relax, omega=omega, npre=npre, npost=npost, solver=solver, nlevels=nlev)
    b = pr.rhs()
    xr, hr, _ = pr.pcg(b, mg=omg, tol=tol)
    prob = mgldg.CartesianProblem(ctx, P, n, tau0=float(n), tauD=float(n))
    bg = prob.rhs_gaussian(seed)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=relax, omega=omega, npre=npre, npost=npost,
                         solver=solver, max_levels=nlev)
    xg, hg = mgldg.pcg(ctx, prob.ops.A, bg, precon=mg, tol=tol)
    return xr, hr, xg, hg, np.linalg.norm(b)


def assert_history_parity(hg, hr, bnorm):
    # same iteration count; every printed ||r_k|| within 1e-12 ||r_0|| (x0 = 0,
    # so ||r_0|| = ||b||) and within 1e-10 of itself
    assert len(hg) == len(hr)
    assert np.all(np.isfinite(hg))
    assert np.abs(hg - hr).max() <= 1e-12 * bnorm
    assert np.max(np.abs(hg - hr) / hr) <= 1e-10


@pytest.mark.parametrize("relax,omega", [(mgldg.RELAX_GAUSS_SEIDEL, 0.8), (mgldg.RELAX_JACOBI, 0.7)])
def test_pcg_history_config1(ctx, relax, omega):
    # 32x32 Q2, hierarchy 32->16->8->4 with a dense coarsest Cholesky, V(2,2)
    xr, hr, xg, hg, bn = pcg_case(ctx, 3, 32, 4, relax, omega)
    assert_history_parity(hg, hr, bn)
    assert np.abs(xg - xr).max() <= 1e-10 * np.abs(xr).max()


def test_pcg_history_reference_defaults(ctx):
    # reference defaults: V(3,3) Gauss-Seidel, omega 0.8, RATRAT, to one element
    xr, hr, xg, hg, bn = pcg_case(ctx, 3, 16, 0, mgldg.RELAX_GAUSS_SEIDEL, 0.8, npre=3, npost=3)
    assert_history_parity(hg, hr, bn)
    assert np.abs(xg - xr).max() <= 1e-10 * np.abs(xr).max()


def test_unpreconditioned_cg(ctx):
    pr = O.Problem(2, 1 / 8, seed=4)
    A = to_gpu(ctx, pr.op(O.OP_A))
    b = pr.rhs()
    xr, hr, _ = pr.pcg(b, mg=None, tol=1e-8, maxit=300)
    xg, hg = mgldg.pcg(ctx, A, b, tol=1e-8, maxit=300)
    assert len(hg) == len(hr)
    assert np.abs(xg - xr).max() <= 1e-9 * np.abs(xr).max()


@pytest.mark.parametrize("relax", [mgldg.RELAX_GAUSS_SEIDEL, mgldg.RELAX_JACOBI])
def test_mixed_precision_reaches_fp64_accuracy(ctx, relax):
    n, P = 64, 4
    prob = mgldg.CartesianProblem(ctx, P, n)
    b = prob.rhs_gaussian(2001)
    omega = 0.8 if relax == mgldg.RELAX_GAUSS_SEIDEL else 0.7
    mg64 = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=relax, omega=omega, npre=2, npost=2,
                           solver=mgldg.COARSE_DENSE, max_levels=5)
    mg32 = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=relax, omega=omega, npre=2, npost=2,
                           solver=mgldg.COARSE_DENSE, max_levels=5, precision=mgldg.PREC_MIXED)
    x64, h64 = mgldg.pcg(ctx, prob.ops.A, b, precon=mg64, tol=1e-12)
    # the FP32 V-cycle does not limit the attainable accuracy: solved to a
    # residual of 1e-11 the mixed form agrees with FP64 to 1e-10 (at 1e-10
    # both solutions sit ~1e-10 from the exact one; the 128 x 128 workload
    # test compares them at that tolerance)
    x32, h32 = mgldg.pcg(ctx, prob.ops.A, b, precon=mg32, tol=1e-11)
    assert np.linalg.norm(x32 - x64) <= 1e-10 * np.linalg.norm(x64)
    assert len(h32) <= len(h64) + 5


def test_error_codes(ctx):
    rp = np.array([0, 1], np.int32)
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.SparseBlockMatrix.from_csr(ctx, 1, 1, 2, 2, rp, np.array([3], np.int32), np.zeros(4))
    assert e.value.code == mgldg.ERR_ARG
    prob = mgldg.CartesianProblem(ctx, 2, 8)
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.Multigrid(ctx, prob.ops, prob.T, solver=mgldg.COARSE_CHOLESKY, max_levels=2)
    assert e.value.code == mgldg.ERR_ARG
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=7)
    assert e.value.code == mgldg.ERR_ARG
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.Multigrid(ctx, prob.ops, prob.T[1:])
    assert e.value.code == mgldg.ERR_SHAPE


def test_bounded_wait_reports_timeout(ctx):
    import ctypes as C
    st = C.c_int(-1)
    rc = mgldg.lib().mgldg_selftest_wait_timeout(ctx.h, 2_000_000, C.byref(st))
    assert rc == mgldg.OK
    assert st.value == mgldg.ERR_TIMEOUT
    # the context keeps working
    prob = mgldg.CartesianProblem(ctx, 2, 4)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T)
    x, h = mgldg.pcg(ctx, prob.ops.A, prob.rhs_gaussian(1), precon=mg, tol=1e-10)
    assert np.all(np.isfinite(h)) and h[-1] < 1e-8 * h[0]

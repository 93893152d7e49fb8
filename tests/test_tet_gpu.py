"""GPU parity of P_{P-1} LDG on tetrahedral meshes of the unit ball (the
reference's unstructured path with N = 3) against the oracle: operators
assembled on the GPU (M, G0, G1, G2, T, A), aggregates (bit-identical) and
transfers, right-hand sides, MG-PCG histories with RAT coarsening, the .fun
dump, and the adjoint gradient dL/dkappa of a per-element diffusivity
against the sparse-direct restatement and finite differences.

Tolerances: operators 1e-13 of their largest entry; transfers 1e-8 (see the
test); rhs
1e-14; PCG histories: the same iteration count, every ||r_k|| within
1e-10 ||b|| (the coarse levels of bounding-box spaces reach cond ~ 1e6-1e7,
so block inverses agree to cond * eps), solutions 1e-8; gradients 1e-7 of
the largest entry; GPU central finite differences (32 elements, relative
step 1e-6) 1e-6 of the largest entry.
"""
import numpy as np
import pytest

import mgldg
import oracle_py as O

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy.sparse")
import adjoint_ref as R  # noqa: E402


def make(ctx, h, P, levels=5, seed=5001):
    p, t = mgldg.ball_mesh(h)
    tau = 1.0 / h
    prob = mgldg.CartesianProblem(ctx, P, mesh=(p, t), tau0=tau, tauD=tau, agg_levels=levels, agg_seed=5000)
    pr = O.Problem.simplex(p, t, P, tau, tau, agg_levels=levels, agg_seed=5000, seed=seed)
    return p, t, prob, pr


def assert_same(gpu, csr, rtol):
    rp, ci, v = gpu.download()
    assert np.array_equal(rp, csr.row_ptr)
    assert np.array_equal(ci, csr.col_idx)
    err = np.abs(v - csr.vals).max() / max(1e-300, np.abs(csr.vals).max())
    assert err <= rtol, err


@pytest.mark.parametrize("h,P", [(0.5, 1), (0.4, 2), (0.3, 3)])
def test_tet_operators_match_oracle(ctx, h, P):
    p, t, prob, pr = make(ctx, h, P)
    assert prob.ne == pr.ne and prob.nfaces == pr.nfaces and prob.nbfaces == pr.nbfaces
    for which in (O.OP_M, O.OP_G0, O.OP_G1, O.OP_G2, O.OP_T, O.OP_A):
        assert_same(prob.ops.get(which), pr.op(which), 1e-13)


def test_tet_hierarchy_rhs_and_dump_match_oracle(ctx, tmp_path):
    p, t, prob, pr = make(ctx, 0.3, 3)
    assert prob.nlevels == pr.nlevels
    for l in range(pr.nlevels - 1):
        assert np.array_equal(prob.partition(l), pr.partition(l))
    H = pr.hierarchy()
    assert (H[0].br, H[0].bc) == (10, 27)
    # the transfers' per-aggregate orthonormalisation goes through Cholesky
    # factors of Gram matrices with cond up to ~1e8, whose inputs (the
    # master mass matrices) differ between the two implementations in the
    # last bit: agreement to cond * eps
    for Tg, Tr in zip(prob.T, H):
        assert_same(Tg, Tr, 1e-8)
    b = prob.rhs_gaussian(5001)
    br = pr.rhs()
    assert np.abs(b - br).max() <= 1e-14 * np.abs(br).max()
    u = np.random.default_rng(3).standard_normal(prob.ndof)
    prob.write_fun(u, tmp_path / "ours.fun")
    pr.write_fun(u, tmp_path / "ref.fun")
    assert open(tmp_path / "ours.fun").read() == open(tmp_path / "ref.fun").read()


@pytest.mark.parametrize("h,relax", [(0.3, mgldg.RELAX_JACOBI), (0.3, mgldg.RELAX_GAUSS_SEIDEL),
                                     (0.1, mgldg.RELAX_GAUSS_SEIDEL)])
def test_tet_pcg_history_matches_oracle(ctx, h, relax):
    # on the 0.1 ball some aggregates' tensor spaces are rank deficient: the
    # dropped directions are zero columns of T0 and absent unknowns of the
    # coarse levels (zero rows in the block and dense inverses) on both sides
    p, t, prob, pr = make(ctx, h, 3)
    if h < 0.2:
        _, ci, v0 = prob.T[0].download()
        zero = np.ones((ci.max() + 1, v0.shape[2]), bool)
        np.logical_and.at(zero, ci, np.all(v0 == 0, axis=1))
        assert zero.any()
    b = pr.rhs()
    omega = 0.7 if relax == mgldg.RELAX_JACOBI else 0.8
    omg = O.Multigrid(pr, relaxation=relax, omega=omega, npre=2, npost=2, solver=O.COARSE_DENSE,
                      restriction=O.RESTRICT_RAT, mean_project=False)
    xr, hr, _ = pr.pcg(b, mg=omg, tol=1e-10)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=relax, omega=omega, npre=2, npost=2,
                         solver=mgldg.COARSE_DENSE, restriction=mgldg.RESTRICT_RAT, mean_project=0)
    xg, hg = mgldg.pcg(ctx, prob.ops.A, b, precon=mg, tol=1e-10)
    assert len(hg) == len(hr) and 2 < len(hr) < 100
    assert np.abs(hg - hr).max() <= 1e-10 * np.linalg.norm(b)
    assert np.abs(xg - xr).max() <= 1e-8 * np.abs(xr).max()


def _centroids(p, t):
    return p[t].mean(axis=1)


def _adjoint_case(ctx, h):
    p, t, prob, pr = make(ctx, h, 3, levels=4)
    kappa = R.field_at(_centroids(p, t), 11)
    k_true = R.field_at(_centroids(p, t), 12)
    b = pr.rhs()
    u_obs = R.l2_adjoint(pr, k_true, b, np.zeros(prob.ndof))[0]
    return p, t, prob, pr, kappa, b, u_obs


def _gpu_adjoint(ctx, prob, kappa, b, u_obs, precision=mgldg.PREC_FP64, tol=1e-12):
    prob.ops.construct_laplacian_kappa(kappa)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, restriction=mgldg.RESTRICT_RAT,
                         relaxation=mgldg.RELAX_GAUSS_SEIDEL, omega=0.8, npre=2, npost=2, solver=mgldg.COARSE_DENSE,
                         mean_project=0, precision=precision)
    return mgldg.adjoint_l2(ctx, prob.ops, b, u_obs, precon=mg, tol=tol, maxit=300)


def test_tet_adjoint_matches_sparse_direct(ctx):
    # FP64 solves to 1e-12; the mixed form (FP32 V-cycle) to its 1e-10 target,
    # whose gradient must still be within 1e-6 of the sparse-direct one
    p, t, prob, pr, kappa, b, u_obs = _adjoint_case(ctx, 0.4)
    ur, lr, gr, Lr = R.l2_adjoint(pr, kappa, b, u_obs)
    for precision, tol, gtol in ((mgldg.PREC_FP64, 1e-12, 1e-7), (mgldg.PREC_MIXED, 1e-10, 1e-6)):
        u, lam, g, L, its = _gpu_adjoint(ctx, prob, kappa, b, u_obs, precision, tol)
        assert np.abs(u - ur).max() <= 1e2 * gtol * np.abs(ur).max() and 0 < its[0] < 300 and 0 < its[1] < 300
        assert np.abs(g - gr).max() <= gtol * np.abs(gr).max()
        assert abs(L - Lr) <= gtol * Lr


def test_tet_adjoint_finite_differences_on_gpu(ctx):
    # 32 seeded tetrahedra of the 0.4 ball, step 1e-6 kappa_e, FP64 solves
    # to 1e-12 (measured: 7.3e-8 of the largest entry)
    from test_adjoint_gpu import fd_check
    p, t, prob, pr, kappa, b, u_obs = _adjoint_case(ctx, 0.4)
    _, _, g, _, _ = _gpu_adjoint(ctx, prob, kappa, b, u_obs)
    fd_check(lambda k: _gpu_adjoint(ctx, prob, k, b, u_obs)[0], kappa, u_obs, g, prob.ne)


def test_indefinite_preconditioner_is_reported(ctx):
    # block Jacobi damped by omega 1.6 is not a convergent smoother (omega
    # exceeds 2 / lambda_max(D^-1 A)), so the V-cycle is indefinite; pcg must
    # report a breakdown instead of stopping on a spurious r.z test (the solve
    # with block Gauss-Seidel converges)
    p, t, prob, pr = make(ctx, 0.2, 3)
    b = pr.rhs()
    bad = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI, omega=1.6, npre=2, npost=2,
                          solver=mgldg.COARSE_DENSE, restriction=mgldg.RESTRICT_RAT, mean_project=0)
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.pcg(ctx, prob.ops.A, b, precon=bad, tol=1e-10, maxit=200)
    assert e.value.code == mgldg.ERR_BREAKDOWN
    good = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_GAUSS_SEIDEL, omega=0.8, npre=2, npost=2,
                           solver=mgldg.COARSE_DENSE, restriction=mgldg.RESTRICT_RAT, mean_project=0)
    x, h = mgldg.pcg(ctx, prob.ops.A, b, precon=good, tol=1e-10, maxit=200)
    r = prob.ops.A.mv(x, alpha=-1.0, beta=1.0, y=b)
    assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(b)

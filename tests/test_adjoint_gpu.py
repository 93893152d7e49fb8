"""GPU parity of the diffusivity-weighted operator and the adjoint gradient
entries (mgldg_ops_construct_laplacian_kappa, mgldg_kappa_gradient_dev,
mgldg_adjoint_l2_dev) against the FP64 sparse-direct restatement in
oracle/adjoint_ref.py, whose formula tests/test_adjoint.py pins with finite
differences.

Tolerances: operators 1e-13 relative to their largest entry; the direct
gradient contraction 1e-12; solutions of the MG-PCG solves (tol 1e-12)
against sparse LU 1e-9 relative, the gradients from them 1e-7 relative to
their largest entry; GPU central finite differences (32 elements, relative
step 1e-6) 1e-6 of the largest gradient entry.
"""
import numpy as np
import pytest

import mgldg
import oracle_py as O

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy.sparse")
import adjoint_ref as R  # noqa: E402


def _dense(gpu):
    rp, ci, v = gpu.download()
    nbr, nbc, br, bc, _ = gpu.info()
    D = np.zeros((nbr * br, nbc * bc))
    for i in range(nbr):
        for k in range(rp[i], rp[i + 1]):
            D[i * br:(i + 1) * br, ci[k] * bc:(ci[k] + 1) * bc] = v[k]
    return D


def test_unit_kappa_matches_construct_laplacian(ctx):
    prob = mgldg.CartesianProblem(ctx, 3, 8)
    rp0, ci0, v0 = prob.ops.A.download()
    prob.ops.construct_laplacian_kappa(None)
    rp1, ci1, v1 = prob.ops.A.download()
    assert np.array_equal(rp0, rp1) and np.array_equal(ci0, ci1)
    assert np.abs(v1 - v0).max() <= 1e-15 * np.abs(v0).max()


@pytest.mark.parametrize("P,n", [(3, 8), (4, 16)])
def test_kappa_operator_matches_restatement(ctx, P, n):
    prob = mgldg.CartesianProblem(ctx, P, n)
    pr = O.Problem(P, 1.0 / n)
    kappa = R.smooth_field(n, 11)
    prob.ops.construct_laplacian_kappa(kappa)
    D = _dense(prob.ops.A)
    ref = R.kappa_laplacian(pr, kappa).toarray()
    assert np.abs(D - ref).max() <= 1e-13 * np.abs(ref).max()


def test_kappa_gradient_contraction(ctx):
    P, n = 4, 16
    prob = mgldg.CartesianProblem(ctx, P, n)
    pr = O.Problem(P, 1.0 / n)
    rng = np.random.default_rng(5)
    u, lam = rng.standard_normal(prob.ndof), rng.standard_normal(prob.ndof)
    g = mgldg.kappa_gradient(ctx, prob.ops, u, lam)
    ref = R.kappa_gradient(pr, u, lam)
    assert np.abs(g - ref).max() <= 1e-12 * np.abs(ref).max()


def _problem(ctx, P, n, seed=21):
    prob = mgldg.CartesianProblem(ctx, P, n)
    pr = O.Problem(P, 1.0 / n, seed=1001)
    b = pr.rhs()
    kappa = R.smooth_field(n, seed)
    k_true = kappa * np.exp(0.3 * np.random.default_rng(seed).standard_normal(prob.ne))
    u_obs = R.l2_adjoint(pr, k_true, b, np.zeros(prob.ndof))[0]
    return prob, pr, b, kappa, u_obs


def _gpu_adjoint(ctx, prob, kappa, b, u_obs, relaxation=mgldg.RELAX_JACOBI):
    prob.ops.construct_laplacian_kappa(kappa)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, restriction=mgldg.RESTRICT_RAT, relaxation=relaxation,
                         omega=0.8, npre=2, npost=2, mean_project=0)
    return mgldg.adjoint_l2(ctx, prob.ops, b, u_obs, precon=mg, tol=1e-12, maxit=200)


@pytest.mark.parametrize("relaxation", [mgldg.RELAX_JACOBI, mgldg.RELAX_GAUSS_SEIDEL])
def test_adjoint_l2_matches_sparse_direct(ctx, relaxation):
    prob, pr, b, kappa, u_obs = _problem(ctx, 4, 16)
    u, lam, g, L, its = _gpu_adjoint(ctx, prob, kappa, b, u_obs, relaxation)
    ur, lr, gr, Lr = R.l2_adjoint(pr, kappa, b, u_obs)
    assert 0 < its[0] < 200 and 0 < its[1] < 200
    assert np.abs(u - ur).max() <= 1e-9 * np.abs(ur).max()
    assert np.abs(lam - lr).max() <= 1e-9 * np.abs(lr).max()
    assert np.abs(g - gr).max() <= 1e-7 * np.abs(gr).max()
    assert abs(L - Lr) <= 1e-9 * Lr


def fd_check(run, kappa, u_obs, g, ne, seed=32, n_el=32, step=1e-6):
    """Central finite differences of L = 1/2 ||u - u_obs||^2 on n_el seeded
    elements with the relative step `step` of kappa_e: every difference
    quotient within 1e-6 of the gradient's largest entry.  L(k+) - L(k-) is
    formed as 1/2 (u+ - u-).(u+ + u- - 2 u_obs), which keeps the rounding of
    the two losses out of the quotient."""
    gmax = np.abs(g).max()
    worst = 0.0
    for e in np.random.default_rng(seed).choice(ne, min(n_el, ne), replace=False):
        h = step * kappa[e]
        kp, km = kappa.copy(), kappa.copy()
        kp[e] += h
        km[e] -= h
        up, um = run(kp), run(km)
        fd = 0.5 * np.dot(up - um, up + um - 2 * u_obs) / (2 * h)
        worst = max(worst, abs(fd - g[e]) / gmax)
    assert worst <= 1e-6, worst
    return worst


def test_adjoint_gradient_finite_differences_on_gpu(ctx):
    # 32 seeded elements, step 1e-6 kappa_e, FP64 solves to 1e-12
    # (measured: 1.9e-7 of the largest entry)
    prob, pr, b, kappa, u_obs = _problem(ctx, 3, 16, seed=4)
    _, _, g, _, _ = _gpu_adjoint(ctx, prob, kappa, b, u_obs, mgldg.RELAX_GAUSS_SEIDEL)
    fd_check(lambda k: _gpu_adjoint(ctx, prob, k, b, u_obs, mgldg.RELAX_GAUSS_SEIDEL)[0], kappa, u_obs, g, prob.ne)


def test_kappa_rejects_nonpositive(ctx):
    prob = mgldg.CartesianProblem(ctx, 3, 4)
    bad = np.ones(prob.ne)
    bad[3] = 0.0
    with pytest.raises(mgldg.MgldgError) as e:
        prob.ops.construct_laplacian_kappa(bad)
    assert e.value.code == mgldg.ERR_ARG

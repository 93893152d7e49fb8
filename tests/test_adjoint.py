"""CPU checks of the diffusivity-weighted operator and its adjoint gradient
restated in oracle/adjoint_ref.py (the checker of the GPU adjoint entries).

The gradient formula dL/dkappa_e = -sum_d (G_d lambda)_e^T M_e (G_d u)_e is
pinned against central finite differences of L(kappa) computed by sparse LU;
kappa = 1 must give the reference Laplacian (ldgpoisson.h:34-52).
"""
import numpy as np
import pytest

import oracle_py as O

sp = pytest.importorskip("scipy.sparse")
import adjoint_ref as R  # noqa: E402


def _setup(n=4, P=3, seed=7):
    pr = O.Problem(P, 1.0 / n, seed=1001)
    kappa = R.smooth_field(n, seed)
    b = pr.rhs()
    u_obs, _, _, _ = R.l2_adjoint(pr, kappa * np.exp(0.3 * np.random.default_rng(seed).standard_normal(pr.ne)),
                                  b, np.zeros(pr.ndof))
    return pr, kappa, b, u_obs


def test_unit_kappa_is_the_reference_laplacian():
    pr = O.Problem(3, 0.25)
    A1 = R.kappa_laplacian(pr, np.ones(pr.ne)).toarray()
    A = pr.op(O.OP_A).todense()
    assert np.abs(A1 - A).max() <= 1e-13 * np.abs(A).max()


def test_kappa_gradient_matches_finite_differences():
    pr, kappa, b, u_obs = _setup()
    _, _, g, L = R.l2_adjoint(pr, kappa, b, u_obs)
    assert L > 0
    rng = np.random.default_rng(3)
    for e in rng.choice(pr.ne, 8, replace=False):
        h = 1e-5 * kappa[e]
        kp, km = kappa.copy(), kappa.copy()
        kp[e] += h
        km[e] -= h
        fd = (R.l2_adjoint(pr, kp, b, u_obs)[3] - R.l2_adjoint(pr, km, b, u_obs)[3]) / (2 * h)
        assert abs(fd - g[e]) <= 1e-6 * np.abs(g).max(), (e, fd, g[e])


def test_rhs_gradient_is_lambda():
    pr, kappa, b, u_obs = _setup()
    _, lam, _, _ = R.l2_adjoint(pr, kappa, b, u_obs)
    rng = np.random.default_rng(4)
    for i in rng.choice(pr.ndof, 6, replace=False):
        h = 1e-4 * max(1.0, abs(b[i]))
        bp, bm = b.copy(), b.copy()
        bp[i] += h
        bm[i] -= h
        fd = (R.l2_adjoint(pr, kappa, bp, u_obs)[3] - R.l2_adjoint(pr, kappa, bm, u_obs)[3]) / (2 * h)
        assert abs(fd - lam[i]) <= 1e-7 * np.abs(lam).max(), (i, fd, lam[i])


def test_kappa_laplacian_is_linear_in_kappa():
    pr = O.Problem(3, 0.25)
    k1 = R.smooth_field(4, 1)
    k2 = R.smooth_field(4, 2)
    T = pr.op(O.OP_T).todense()
    lhs = R.kappa_laplacian(pr, k1 + k2).toarray() - T
    rhs = (R.kappa_laplacian(pr, k1).toarray() - T) + (R.kappa_laplacian(pr, k2).toarray() - T)
    assert np.abs(lhs - rhs).max() <= 1e-12 * np.abs(lhs).max()

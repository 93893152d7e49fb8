"""FP64 sparse-direct restatement of the diffusivity-weighted LDG operator and
its adjoint gradient (TEST INFRASTRUCTURE ONLY).

The reference has no diffusivity or adjoint path; this module builds them
from the oracle's exported reference operators (M, G_d, T of
src/cartesian/dg/ldgpoisson.h:15-53) with scipy, so the GPU entry points
mgldg_ops_construct_laplacian_kappa / mgldg_kappa_gradient_dev /
mgldg_adjoint_l2_dev have a checker:

    A(kappa)    = T + sum_d G_d^T diag(kappa_e M_e) G_d
    L           = 1/2 ||u - u_obs||^2,  A u = b
    A lambda    = u - u_obs
    dL/db       = lambda
    dL/dkappa_e = -sum_d (G_d lambda)_e^T M_e (G_d u)_e
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import oracle_py as O


def to_scipy(csr):
    """Block CSR export -> scipy CSR matrix."""
    m = sp.bsr_matrix((csr.vals, csr.col_idx, csr.row_ptr),
                      shape=(csr.nbr * csr.br, csr.nbc * csr.bc))
    return m.tocsr()


def operators(pr):
    """(M, [G0, G1(, G2)], T) of an oracle Problem as scipy matrices, plus M's blocks."""
    Mc = pr.op(O.OP_M)
    ids = [O.OP_G0, O.OP_G1] + ([O.OP_G2] if getattr(pr, "dim", 2) == 3 else [])
    return to_scipy(Mc), [to_scipy(pr.op(w)) for w in ids], to_scipy(pr.op(O.OP_T)), Mc


def kappa_laplacian(pr, kappa):
    M, G, T, _ = operators(pr)
    b = pr.npl
    K = sp.diags(np.repeat(np.asarray(kappa, np.float64), b))
    A = T.copy()
    for g in G:
        A = A + g.T @ (K @ M) @ g
    return A.tocsr()


def kappa_gradient(pr, u, lam):
    """dkappa_e = -sum_d (G_d lam)_e^T M_e (G_d u)_e."""
    M, G, _, Mc = operators(pr)
    b = pr.npl
    out = np.zeros(pr.ne)
    diag = np.array([Mc.row_ptr[e] + list(Mc.col_idx[Mc.row_ptr[e]:Mc.row_ptr[e + 1]]).index(e)
                     for e in range(pr.ne)])
    Me = Mc.vals[diag]
    for g in G:
        gu = (g @ u).reshape(pr.ne, b)
        gl = (g @ lam).reshape(pr.ne, b)
        out -= np.einsum("ei,eij,ej->e", gl, Me, gu)
    return out


def l2_adjoint(pr, kappa, b, u_obs):
    """(u, lambda, dL/dkappa, L) by sparse LU."""
    A = kappa_laplacian(pr, kappa).tocsc()
    lu = spla.splu(A)
    u = lu.solve(np.asarray(b, np.float64))
    r = u - u_obs
    lam = lu.solve(r)
    return u, lam, kappa_gradient(pr, u, lam), 0.5 * float(r @ r)


def smooth_field(n, seed, corr=0.2, sigma=0.5, nfeat=64):
    """log-normal per-element diffusivity on an n x n grid of [0,1]^2 in the
    element order of the Cartesian builder (Morton, x bit above y): random
    Fourier features of a Gaussian covariance with length `corr`."""
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nfeat, 2)) / corr
    ph = rng.uniform(0, 2 * np.pi, nfeat)
    a = rng.standard_normal(nfeat) * sigma * np.sqrt(2.0 / nfeat)
    ne = n * n
    kappa = np.zeros(ne)
    for e in range(ne):
        ix = iy = 0
        for bit in range(n.bit_length() - 1):
            iy |= ((e >> (2 * bit)) & 1) << bit
            ix |= ((e >> (2 * bit + 1)) & 1) << bit
        x, y = (ix + 0.5) / n, (iy + 0.5) / n
        kappa[e] = np.exp(a @ np.cos(w @ np.array([x, y]) + ph))
    return kappa


def field_at(X, seed, corr=0.2, sigma=0.5, nfeat=64):
    """log-normal diffusivity exp(g(x)) at points X (n x dim): random Fourier
    features of a Gaussian covariance with length `corr` and deviation sigma."""
    X = np.asarray(X, np.float64)
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nfeat, X.shape[1])) / corr
    ph = rng.uniform(0, 2 * np.pi, nfeat)
    a = rng.standard_normal(nfeat) * sigma * np.sqrt(2.0 / nfeat)
    return np.exp(np.cos(X @ w.T + ph) @ a)

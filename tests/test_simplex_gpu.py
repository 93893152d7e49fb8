"""GPU parity of the unstructured (triangle) LDG path against the oracle:
operators assembled on the GPU, the agglomeration hierarchy (aggregates
bit-identical, transfer blocks), the right-hand side, MG-PCG histories and
the .fun dump.

Tolerances: operators 1e-13 of their largest entry; transfers 1e-14;
right-hand sides 1e-14; PCG histories with the same iteration count and
every ||r_k|| within 1e-12 ||b|| (RAT coarsening; RATRAT 1e-8, see the
test), solutions 1e-10.
"""
import numpy as np
import pytest

import mgldg
import oracle_py as O

pytestmark = pytest.mark.gpu


def make(ctx, h, P, levels=5, seed=4001):
    p, t = mgldg.disk_mesh(h)
    tau = 1.0 / h
    prob = mgldg.CartesianProblem(ctx, P, mesh=(p, t), tau0=tau, tauD=tau, agg_levels=levels, agg_seed=4000)
    pr = O.Problem.simplex(p, t, P, tau, tau, agg_levels=levels, agg_seed=4000, seed=seed)
    return p, t, prob, pr


def assert_same(gpu, csr, rtol):
    rp, ci, v = gpu.download()
    assert np.array_equal(rp, csr.row_ptr)
    assert np.array_equal(ci, csr.col_idx)
    err = np.abs(v - csr.vals).max() / max(1e-300, np.abs(csr.vals).max())
    assert err <= rtol, err


@pytest.mark.parametrize("h,P", [(0.2, 1), (0.1, 2), (0.1, 3), (0.05, 3), (0.1, 4)])
def test_simplex_operators_match_oracle(ctx, h, P):
    p, t, prob, pr = make(ctx, h, P)
    assert prob.ne == pr.ne and prob.nfaces == pr.nfaces and prob.nbfaces == pr.nbfaces
    for which in (O.OP_M, O.OP_G0, O.OP_G1, O.OP_T, O.OP_A):
        assert_same(prob.ops.get(which), pr.op(which), 1e-13)


@pytest.mark.parametrize("h,P", [(0.1, 3), (0.05, 2)])
def test_simplex_hierarchy_rhs_match_oracle(ctx, h, P):
    p, t, prob, pr = make(ctx, h, P)
    assert prob.nlevels == pr.nlevels
    for l in range(pr.nlevels - 1):
        assert np.array_equal(prob.partition(l), pr.partition(l))
    H = pr.hierarchy()
    assert len(H) == len(prob.T)
    for Tg, Tr in zip(prob.T, H):
        assert_same(Tg, Tr, 1e-14)
    b = prob.rhs_gaussian(4001)
    br = pr.rhs()
    assert np.abs(b - br).max() <= 1e-14 * np.abs(br).max()


@pytest.mark.parametrize("relax,omega,restriction", [(mgldg.RELAX_JACOBI, 0.7, mgldg.RESTRICT_RATRAT),
                                                     (mgldg.RELAX_GAUSS_SEIDEL, 0.8, mgldg.RESTRICT_RATRAT),
                                                     (mgldg.RELAX_JACOBI, 0.7, mgldg.RESTRICT_RAT)])
def test_simplex_pcg_history_matches_oracle(ctx, relax, omega, restriction):
    p, t, prob, pr = make(ctx, 0.05, 3, levels=6)
    b = pr.rhs()
    omg = O.Multigrid(pr, relaxation=relax, omega=omega, npre=2, npost=2, solver=O.COARSE_DENSE,
                      restriction=restriction, mean_project=False)
    xr, hr, _ = pr.pcg(b, mg=omg, tol=1e-10)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=relax, omega=omega, npre=2, npost=2,
                         solver=mgldg.COARSE_DENSE, restriction=restriction, mean_project=0)
    xg, hg = mgldg.pcg(ctx, prob.ops.A, b, precon=mg, tol=1e-10)
    assert len(hg) == len(hr) and 5 < len(hr) < 80
    # RATRAT inverts the coarse mass blocks M_c = T^T M T; on aggregates that
    # fill a thin part of their bounding box these reach cond ~ 3e8 (0.05
    # disk, level 1), so the oracle's LDL^T solves and the GPU's inverses
    # agree to cond * eps only; RAT inverts nothing and keeps 1e-12
    tol = 1e-12 if restriction == mgldg.RESTRICT_RAT else 1e-8
    assert np.abs(hg - hr).max() <= tol * np.linalg.norm(b)
    assert np.abs(xg - xr).max() <= max(1e-10, tol) * np.abs(xr).max()


def test_simplex_mixed_precision_and_batched(ctx):
    p, t, prob, pr = make(ctx, 0.05, 3, levels=6)
    fp64 = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2,
                           solver=mgldg.COARSE_DENSE, mean_project=0)
    mixed = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2,
                            solver=mgldg.COARSE_DENSE, mean_project=0, precision=mgldg.PREC_MIXED)
    B = np.stack([prob.rhs_gaussian(4001 + c) for c in range(8)], axis=1)
    xd, _ = mgldg.pcg(ctx, prob.ops.A, B[:, 0], precon=fp64, tol=1e-12)
    xm, hm = mgldg.pcg(ctx, prob.ops.A, B[:, 0], precon=mixed, tol=1e-10)
    assert np.abs(xm - xd).max() <= 1e-8 * np.abs(xd).max()
    X, its, _ = mgldg.pcg_batched(ctx, prob.ops.A, B, precon=mixed, tol=1e-10)
    assert abs(its[0] - len(hm)) <= 1
    assert np.abs(X[:, 0] - xd).max() <= 1e-8 * np.abs(xd).max()


def test_simplex_write_fun_matches_oracle(ctx, tmp_path):
    p, t, prob, pr = make(ctx, 0.2, 3)
    u = np.random.default_rng(3).standard_normal(prob.ndof)
    prob.write_fun(u, tmp_path / "ours.fun")
    pr.write_fun(u, tmp_path / "ref.fun")
    assert open(tmp_path / "ours.fun").read() == open(tmp_path / "ref.fun").read()


@pytest.mark.parametrize("restriction", [mgldg.RESTRICT_RAT, mgldg.RESTRICT_RATRAT])
def test_segmented_pcg_on_a_union_of_meshes(ctx, restriction):
    # three disks of uneven sizes as one block-diagonal system; segment s must
    # follow the oracle's pcg of the union with b zero outside segment s
    # (A and the V-cycle are block diagonal, so that is segment s's own solve)
    meshes = [mgldg.disk_mesh(h) for h in (0.1, 0.2, 0.13)]
    p, t, eoff = mgldg.mesh_union(meshes)
    P, tau = 3, 10.0
    prob = mgldg.CartesianProblem(ctx, P, mesh=(p, t), tau0=tau, tauD=tau, agg_levels=6, agg_seed=4000)
    pr = O.Problem.simplex(p, t, P, tau, tau, agg_levels=6, agg_seed=4000, seed=4001)
    b = pr.rhs()
    off = eoff * prob.npl
    kw = dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2, restriction=restriction, mean_project=0)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, solver=mgldg.COARSE_DENSE, **kw)
    omg = O.Multigrid(pr, relaxation=O.RELAX_JACOBI, omega=0.7, npre=2, npost=2, solver=O.COARSE_DENSE,
                      restriction=restriction, mean_project=False)
    x, its, hist = mgldg.pcg_segmented(ctx, prob.ops.A, b, off, precon=mg, tol=1e-10)
    tol = 1e-12 if restriction == mgldg.RESTRICT_RAT else 1e-8
    for s in range(len(meshes)):
        bs = np.zeros_like(b)
        bs[off[s]:off[s + 1]] = b[off[s]:off[s + 1]]
        xr, hr, _ = pr.pcg(bs, mg=omg, tol=1e-10)
        assert its[s] == len(hr) > 3
        nb = np.linalg.norm(bs)
        assert np.abs(hist[s] - hr).max() <= tol * nb
        seg = slice(off[s], off[s + 1])
        assert np.abs(x[seg] - xr[seg]).max() <= max(1e-10, tol) * np.abs(xr[seg]).max()

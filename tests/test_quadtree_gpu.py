"""GPU parity of LDG problems on adaptive quadtrees (non-canonical faces,
hanging nodes) against the oracle: operators, h-interpolation hierarchy over
the tree's layers, right-hand side and MG-PCG histories.

Tolerances: operators 1e-13 of their largest entry (identical patterns);
transfers 1e-15; right-hand sides 1e-14; PCG histories with the same
iteration count and every ||r_k|| within 1e-12 ||b||; solutions 1e-10.
"""
import numpy as np
import pytest

import mgldg
import oracle_py as O

pytestmark = pytest.mark.gpu


def ref_adaptive(dx):
    return lambda x, y: dx if x > 0.5 else (0.25 * dx if x > 0.25 else 0.5 * dx)


def make(ctx, case, P):
    if case == "ref_adaptive":
        dx = 1 / 8
        qt = mgldg.Quadtree(ref_adaptive(dx))
        prob = mgldg.CartesianProblem(ctx, P, quadtree=qt, tau0=1 / dx, tauD=1 / dx)
        pr = O.Problem(P, dx, refine=O.REFINE_REF_ADAPTIVE)
    elif case == "points":
        pts = mgldg.seeded_points(3000, 4)
        qt = mgldg.Quadtree.points(pts, 3, 3, balance=True)
        prob = mgldg.CartesianProblem(ctx, P, quadtree=qt, tau_per_face=True)
        pr = O.Problem.points(P, 3, 3, balance=True, tau_per_face=True)
    else:   # sharp points rule, unbalanced: level jumps of 3
        pts = mgldg.seeded_points(3000, 4)
        qt = mgldg.Quadtree.points(pts, 3, 5, radius=0.1, balance=False)
        prob = mgldg.CartesianProblem(ctx, P, quadtree=qt, tau0=8.0, tauD=8.0)
        pr = O.Problem.points(P, 3, 5, radius=0.1, balance=False, tau_per_face=False, tau0=8.0, tauD=8.0)
    return qt, prob, pr


def assert_same(gpu, csr, rtol):
    rp, ci, v = gpu.download()
    assert np.array_equal(rp, csr.row_ptr)
    assert np.array_equal(ci, csr.col_idx)
    err = np.abs(v - csr.vals).max() / max(1e-300, np.abs(csr.vals).max())
    assert err <= rtol, err


CASES = [("ref_adaptive", 3), ("points", 3), ("sharp", 2), ("points", 4)]


@pytest.mark.parametrize("case,P", CASES)
def test_adaptive_operators_match_oracle(ctx, case, P):
    qt, prob, pr = make(ctx, case, P)
    assert prob.ne == pr.ne and prob.nfaces == pr.nfaces and prob.nbfaces == pr.nbfaces
    assert prob.nlevels == pr.nlevels
    for which in (O.OP_M, O.OP_G0, O.OP_G1, O.OP_T, O.OP_A):
        assert_same(prob.ops.get(which), pr.op(which), 1e-13)


@pytest.mark.parametrize("case,P", CASES[:3])
def test_adaptive_hierarchy_and_rhs_match_oracle(ctx, case, P):
    qt, prob, pr = make(ctx, case, P)
    H = pr.hierarchy()
    assert len(H) == len(prob.T)
    for Tg, Tr in zip(prob.T, H):
        assert_same(Tg, Tr, 1e-15)
    seed = 1001 if case == "ref_adaptive" else 3001
    b = prob.rhs_gaussian(seed)
    br = pr.rhs()
    assert np.abs(b - br).max() <= 1e-14 * np.abs(br).max()


@pytest.mark.parametrize("relax,omega", [(mgldg.RELAX_GAUSS_SEIDEL, 0.8), (mgldg.RELAX_JACOBI, 0.7)])
def test_adaptive_pcg_history_matches_oracle(ctx, relax, omega):
    qt, prob, pr = make(ctx, "points", 3)
    omg = O.Multigrid(pr, relaxation=relax, omega=omega, npre=2, npost=2)
    b = pr.rhs()
    xr, hr, _ = pr.pcg(b, mg=omg, tol=1e-10)
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, relaxation=relax, omega=omega, npre=2, npost=2)
    xg, hg = mgldg.pcg(ctx, prob.ops.A, b, precon=mg, tol=1e-10)
    assert len(hg) == len(hr)
    assert np.abs(hg - hr).max() <= 1e-12 * np.linalg.norm(b)
    assert np.abs(xg - xr).max() <= 1e-10 * np.abs(xr).max()


def test_adaptive_write_fun_matches_oracle(ctx, tmp_path):
    qt, prob, pr = make(ctx, "ref_adaptive", 3)
    u = np.random.default_rng(1).standard_normal(prob.ndof)
    prob.write_fun(u, tmp_path / "ours.fun")
    pr.write_fun(u, tmp_path / "ref.fun")
    assert open(tmp_path / "ours.fun").read() == open(tmp_path / "ref.fun").read()

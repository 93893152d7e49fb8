"""GPU parity of p- and hp-multigrid (the reference's Multigrid<N,P1,P2,...>,
src/cartesian/multigrid/multigrid.h:436-560) against the CPU oracle.

Tolerances as in test_parity_gpu.py: transfers 1e-15 relative to their
largest entry, level operators 1e-12, V-cycles 1e-12, PCG histories within
1e-12 ||r_0|| with the same iteration count, solutions 1e-10.
"""
import numpy as np
import pytest

import mgldg
import oracle_py as O

pytestmark = pytest.mark.gpu


def assert_same(gpu, csr, rtol):
    rp, ci, v = gpu.download()
    assert np.array_equal(rp, csr.row_ptr)
    assert np.array_equal(ci, csr.col_idx)
    err = np.abs(v - csr.vals).max() / max(1.0, np.abs(csr.vals).max())
    assert err <= rtol, err


CASES = [([4, 2], 0, mgldg.COARSE_RELAXATION), ([4, 3, 2], 3, mgldg.COARSE_DENSE), ([3, 2], 4, mgldg.COARSE_DENSE)]


@pytest.mark.parametrize("degrees,nh,solver", CASES)
def test_hp_transfers_and_levels_match_oracle(ctx, degrees, nh, solver):
    n = 16
    pr = O.Problem(degrees[0], 1 / n, tau0=n, tauD=n, seed=1001)
    omg = O.Multigrid.hp(pr, degrees, nh, npre=2, npost=2, solver=solver)
    prob = mgldg.CartesianProblem(ctx, degrees[0], n)
    T = mgldg.hp_chain(ctx, n, degrees, nh)
    for l, t in enumerate(T):
        assert_same(t, omg.transfer(l), 1e-15)
    mg = mgldg.Multigrid(ctx, prob.ops, T, npre=2, npost=2, solver=solver)
    assert mg.nlevels == omg.nlevels
    for l in range(1, mg.nlevels):
        for w in (O.OP_M, O.OP_G0, O.OP_G1, O.OP_T, O.OP_A):
            assert_same(mg.level_op(l, w), omg.level_op(l, w), 1e-12)


@pytest.mark.parametrize("degrees,nh,solver", CASES)
@pytest.mark.parametrize("mean_project", [True, False])
def test_hp_pcg_matches_oracle(ctx, degrees, nh, solver, mean_project):
    n = 16
    pr = O.Problem(degrees[0], 1 / n, tau0=n, tauD=n, seed=1001)
    omg = O.Multigrid.hp(pr, degrees, nh, npre=2, npost=2, solver=solver, mean_project=mean_project)
    b = pr.rhs()
    xr, hr, _ = pr.pcg(b, mg=omg, tol=1e-10)
    prob = mgldg.CartesianProblem(ctx, degrees[0], n)
    mg = mgldg.Multigrid(ctx, prob.ops, mgldg.hp_chain(ctx, n, degrees, nh), npre=2, npost=2, solver=solver,
                         mean_project=int(mean_project))
    ref_v = omg.vcycle(b)
    got_v = mg.vcycle(b)
    assert np.abs(got_v - ref_v).max() <= 1e-12 * np.abs(ref_v).max()
    xg, hg = mgldg.pcg(ctx, prob.ops.A, prob.rhs_gaussian(1001), precon=mg, tol=1e-10)
    assert len(hg) == len(hr)
    assert np.abs(hg - hr).max() <= 1e-12 * np.linalg.norm(b)
    assert np.abs(xg - xr).max() <= 1e-10 * np.abs(xr).max()


def test_hp_mixed_precision(ctx):
    n, degrees, nh = 64, [4, 2], 4
    prob = mgldg.CartesianProblem(ctx, degrees[0], n)
    b = prob.rhs_gaussian(7)
    kw = dict(npre=2, npost=2, solver=mgldg.COARSE_DENSE, mean_project=0)
    mg64 = mgldg.Multigrid(ctx, prob.ops, mgldg.hp_chain(ctx, n, degrees, nh), **kw)
    mg32 = mgldg.Multigrid(ctx, prob.ops, mgldg.hp_chain(ctx, n, degrees, nh), precision=mgldg.PREC_MIXED, **kw)
    x64, h64 = mgldg.pcg(ctx, prob.ops.A, b, precon=mg64, tol=1e-12)
    x32, h32 = mgldg.pcg(ctx, prob.ops.A, b, precon=mg32, tol=1e-10)
    assert np.linalg.norm(x32 - x64) <= 1e-9 * np.linalg.norm(x64)
    assert len(h32) <= len(h64) + 5

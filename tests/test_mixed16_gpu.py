"""The block-scaled FP16 form of the mixed V-cycle (MGLDG_PREC_MIXED_F16): the
level operators' Jacobi sweeps and residuals read an FP16 copy with one FP32
scale per block (entries / block max), arithmetic and vectors in FP32, the
outer CG in FP64.

The form changes the preconditioner, not the solution: PCG must reach the
FP64 solution (1e-10 relative, solved to a residual of 1e-11) and take about
as many iterations to 1e-10 as the FP32 form.
One sweep on its own must equal the FP64 sweep to the FP16 quantisation
(|error| <= 2^-10 of the largest entry times the block row's sum, checked as
1e-3 of the result's largest entry) on 16x16 blocks (Q4 on a Cartesian
grid); other block sizes (P3 triangles: 6x6 and 9x9) keep the FP32 copy, so
there the form equals MIXED bit for bit.
"""
import numpy as np
import pytest

import mgldg

pytestmark = pytest.mark.gpu


def _forms(ctx, prob, T, **kw):
    return {prec: mgldg.Multigrid(ctx, prob.ops, T, precision=prec, **kw)
            for prec in (mgldg.PREC_FP64, mgldg.PREC_MIXED, mgldg.PREC_MIXED_F16)}


def _check_pcg(ctx, prob, mgs, b):
    x64, h64 = mgldg.pcg(ctx, prob.ops.A, b, precon=mgs[mgldg.PREC_FP64], tol=1e-12)
    _, h32 = mgldg.pcg(ctx, prob.ops.A, b, precon=mgs[mgldg.PREC_MIXED], tol=1e-10)
    x16, h16 = mgldg.pcg(ctx, prob.ops.A, b, precon=mgs[mgldg.PREC_MIXED_F16], tol=1e-10)
    # solved to a residual of 1e-11 the FP16-stored form reaches FP64 to 1e-10
    x16t, _ = mgldg.pcg(ctx, prob.ops.A, b, precon=mgs[mgldg.PREC_MIXED_F16], tol=1e-11)
    assert np.linalg.norm(x16t - x64) <= 1e-10 * np.linalg.norm(x64)
    assert len(h16) <= len(h32) + 3
    r = prob.ops.A.mv(x16, alpha=-1.0, beta=1.0, y=b)
    assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(b)


def _check_sweeps(mgs, levels, n_of):
    rng = np.random.default_rng(7)
    for l in levels:
        n = n_of(l)
        b = rng.standard_normal(n)
        x0 = rng.standard_normal(n)
        ref = mgs[mgldg.PREC_FP64].relax(l, 1, False, b, x0)
        got = mgs[mgldg.PREC_MIXED_F16].relax(l, 1, False, b, x0)
        f32 = mgs[mgldg.PREC_MIXED].relax(l, 1, False, b, x0)
        scale = np.abs(ref).max()
        err16 = np.abs(got - ref).max()
        assert err16 <= 1e-3 * scale, (l, err16 / scale)
        # the FP16 copy is really in use: its error is well above FP32 rounding
        assert err16 > 4 * np.abs(f32 - ref).max(), (l, err16, np.abs(f32 - ref).max())


@pytest.mark.parametrize("P", [4])
def test_cartesian_q3_blocks(ctx, P):
    n = 64
    prob = mgldg.CartesianProblem(ctx, P, n)
    kw = dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2, solver=mgldg.COARSE_DENSE, max_levels=5)
    mgs = _forms(ctx, prob, prob.T, **kw)
    _check_pcg(ctx, prob, mgs, prob.rhs_gaussian(2001))
    _check_sweeps(mgs, [0, 1, 2], lambda l: (n >> l) ** 2 * P * P)


def test_triangle_blocks_keep_fp32(ctx):
    h = 0.05
    p, t = mgldg.disk_mesh(h)
    prob = mgldg.CartesianProblem(ctx, 3, mesh=(p, t), tau0=1 / h, tauD=1 / h, agg_levels=6, agg_seed=4000)
    kw = dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2, solver=mgldg.COARSE_DENSE,
              mean_project=0)
    mgs = _forms(ctx, prob, prob.T, **kw)
    _check_pcg(ctx, prob, mgs, prob.rhs_gaussian(4001))
    sizes = [mgs[mgldg.PREC_FP64].level_op(l, 4).info() for l in range(3)]
    assert sizes[0][2] == 6 and sizes[1][2] == 9
    rng = np.random.default_rng(9)
    for l in range(3):
        n = sizes[l][0] * sizes[l][2]
        b, x0 = rng.standard_normal(n), rng.standard_normal(n)
        a = mgs[mgldg.PREC_MIXED_F16].relax(l, 1, False, b, x0)
        c = mgs[mgldg.PREC_MIXED].relax(l, 1, False, b, x0)
        assert np.array_equal(a, c)

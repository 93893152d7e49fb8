"""The coarse end of the mixed Jacobi V-cycle as one cooperative launch
(csrc/tail.cu, opt-in through MGLDG_VTAIL_ROWS) against the same V-cycle run
as one launch per step (the default): the tail repeats each replaced kernel's
arithmetic lane for lane, so the PCG residual histories and solutions must
agree bit for bit, with fewer launches.  Parity of the per-step path with the
oracle is covered by test_parity_gpu.py and test_config2_parity_gpu.py.
"""
import numpy as np
import pytest

import mgldg

pytestmark = pytest.mark.gpu


def _solve(ctx, prob, b, monkeypatch, rows, **kw):
    if rows is None:
        monkeypatch.delenv("MGLDG_VTAIL_ROWS", raising=False)
    else:
        monkeypatch.setenv("MGLDG_VTAIL_ROWS", str(rows))
    mg = mgldg.Multigrid(ctx, prob.ops, prob.T, **kw)
    ctx.prof_reset()
    ctx.prof_enable(True)
    try:
        x, hist = mgldg.pcg(ctx, prob.ops.A, b, precon=mg, tol=1e-10, maxit=200)
    finally:
        ctx.prof_enable(False)
    launches = sum(n for n, _ in ctx.prof().values())
    # the same solve again through the graph-replayed V-cycles
    x2, hist2 = mgldg.pcg(ctx, prob.ops.A, b, precon=mg, tol=1e-10, maxit=200)
    assert np.array_equal(x, x2) and np.array_equal(hist, hist2)
    return x, hist, launches


@pytest.mark.parametrize("P,n,npre,npost", [(4, 128, 2, 2), (4, 128, 1, 2), (4, 64, 3, 3)])
def test_tail_is_bit_identical_to_per_step_launches(ctx, monkeypatch, P, n, npre, npost):
    prob = mgldg.CartesianProblem(ctx, P, n)
    b = prob.rhs_gaussian(2001)
    kw = dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=npre, npost=npost, solver=mgldg.COARSE_DENSE,
              mean_project=0, precision=mgldg.PREC_MIXED)
    x0, h0, n0 = _solve(ctx, prob, b, monkeypatch, None, **kw)
    x1, h1, n1 = _solve(ctx, prob, b, monkeypatch, 4096, **kw)
    assert n1 < n0, (n1, n0)   # the tail is in use
    assert len(h1) == len(h0) and 5 < len(h0) < 200
    assert np.array_equal(h1, h0)
    assert np.array_equal(x1, x0)


def test_tail_starts_at_any_level(ctx, monkeypatch):
    # from the first level of <= 1024 rows instead of <= 4096
    prob = mgldg.CartesianProblem(ctx, 4, 128)
    b = prob.rhs_gaussian(7)
    kw = dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, npre=2, npost=2, solver=mgldg.COARSE_DENSE,
              mean_project=0, precision=mgldg.PREC_MIXED)
    x0, h0, _ = _solve(ctx, prob, b, monkeypatch, 0, **kw)
    x1, h1, _ = _solve(ctx, prob, b, monkeypatch, 1024, **kw)
    assert np.array_equal(h1, h0) and np.array_equal(x1, x0)


def test_tail_off_where_unsupported(ctx, monkeypatch):
    # mean projection, FP64 and Gauss-Seidel keep the per-step launches:
    # same launch counts with and without the tail requested
    prob = mgldg.CartesianProblem(ctx, 4, 64)
    b = prob.rhs_gaussian(3)
    for kw in (dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, mean_project=1, precision=mgldg.PREC_MIXED),
               dict(relaxation=mgldg.RELAX_JACOBI, omega=0.7, mean_project=0, precision=mgldg.PREC_FP64),
               dict(relaxation=mgldg.RELAX_GAUSS_SEIDEL, omega=0.8, mean_project=0, precision=mgldg.PREC_MIXED)):
        kw.update(npre=2, npost=2, solver=mgldg.COARSE_DENSE)
        x0, h0, n0 = _solve(ctx, prob, b, monkeypatch, None, **kw)
        x1, h1, n1 = _solve(ctx, prob, b, monkeypatch, 4096, **kw)
        assert n0 == n1 and np.array_equal(h0, h1) and np.array_equal(x0, x1)

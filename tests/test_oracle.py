"""CPU tests of the oracle (the checker) against the reference's own pins.

Pins: the reference's constant tables (src/cartesian/dg/master.h, read as
text into tests/golden/master_tables.json), the 2x2-block known answer of
tests/cartesian/matrix_tests.cpp, the manufactured-solution convergence rate
of tests/cartesian/dg_tests.cpp:232-254, and structural invariants of the
reference's operators.
"""
import json
import os

import numpy as np
import pytest

import oracle_py as O

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "master_tables.json")))


@pytest.mark.parametrize("P", range(1, 7))
def test_master_tables_match_reference_constants(P):
    t = O.master_tables(P)
    g = GOLDEN["tables"][str(P)]
    for key in ["nodes", "denom", "mass", "invmass", "diff"]:
        ref = np.array([float(s) for s in g[key]])
        assert np.array_equal(np.asarray(t[key]).ravel(), ref), key


def test_face_quadrature_matches_reference_constants():
    # Q = 10 is the face rule (common.h:15); all rules to within one ulp
    for Q in range(1, 13):
        x, w = O.quadrature(Q)
        g = GOLDEN["quadrature"][str(Q)]
        rx = np.array([float(s) for s in g["nodes"]])
        rw = np.array([float(s) for s in g["weights"]])
        if Q == 10:
            assert np.array_equal(x, rx) and np.array_equal(w, rw)
        assert np.all(np.abs(x - rx) <= np.spacing(np.abs(rx)))
        assert np.all(np.abs(w - rw) <= np.spacing(np.abs(rw)))


def test_matrix_tests_2x2_known_answer():
    kt = GOLDEN["matrix_tests_2x2"]
    A = O.BlockMatrix(2, 2, 2)
    for blk in kt["blocks"]:
        A.set_block(blk["i"], blk["j"], np.array(blk["vals"]).reshape(2, 2))
    y = A.mv(np.array(kt["x"]))
    assert np.array_equal(y, np.array(kt["y"]))
    assert np.array_equal(y, [22.0, 30.0, 37.0, 38.0])


def test_add_block_accumulates_and_mv_t():
    A = O.BlockMatrix(2, 3, 2, 3)
    rng = np.random.default_rng(0)
    B1, B2 = rng.standard_normal((2, 3)), rng.standard_normal((2, 3))
    A.add_block(1, 2, B1)
    A.add_block(1, 2, B2)
    D = np.zeros((4, 9))
    D[2:4, 6:9] = B1 + B2
    x = rng.standard_normal(9)
    assert np.allclose(A.mv(x), D @ x, rtol=0, atol=1e-14)
    z = rng.standard_normal(4)
    assert np.allclose(A.mv_t(z), D.T @ z, rtol=0, atol=1e-14)


@pytest.mark.parametrize("P", [2, 3, 4])
def test_operators_symmetric_and_structured(P):
    pr = O.Problem(P, 1 / 8, test=O.TEST_GAUSSIAN, seed=1001)
    A = pr.op(O.OP_A).todense()
    assert np.abs(A - A.T).max() <= 1e-12 * np.abs(A).max()
    ev = np.linalg.eigvalsh(0.5 * (A + A.T))
    assert ev.min() > 0
    M = pr.op(O.OP_M)
    assert np.array_equal(M.col_idx, np.arange(pr.ne))   # block diagonal
    # uniform 8x8: 64 elements, 2*8*7 interior faces, 32 boundary faces
    assert pr.ne == 64 and pr.nfaces == 112 + 32 and pr.nbfaces == 32
    assert pr.op(O.OP_A).nnzb == 64 + 2 * 112


def test_interpolation_reproduces_constants():
    pr = O.Problem(3, 1 / 8)
    for T in pr.hierarchy():
        ones_c = np.ones(T.nbc * T.bc)
        assert np.allclose(T.matvec(ones_c), 1.0, atol=1e-14)
        assert np.all(np.diff(T.row_ptr) == 1)   # one block per fine row


def test_element_order_is_reference_dfs():
    # quadtree.tpp:18-31: children (x-lo,y-lo),(x-lo,y-hi),(x-hi,y-lo),(x-hi,y-hi)
    pr = O.Problem(2, 1 / 4)
    lo, _ = pr.elements()
    first = lo[:4] * 4
    assert np.array_equal(first, [[0, 0], [0, 1], [1, 0], [1, 1]])
    assert np.array_equal(lo[4] * 4, [0, 2])


@pytest.mark.parametrize("P", [2, 3])
def test_manufactured_solution_rate(P):
    # u = cos(2 pi x) cos(2 pi y) + x + y with Dirichlet data; error ~ h^P
    errs = []
    for n in [4, 8, 16]:
        pr = O.Problem(P, 1 / n, test=O.TEST_SOLUTION, tau0=n, tauD=n)
        A = pr.op(O.OP_A).todense()
        u = np.linalg.solve(A, pr.rhs())
        errs.append(np.abs(u - pr.utrue()).max())
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert rates[-1] > P - 0.35, (errs, rates)


def test_pcg_mg_matches_direct_solve():
    pr = O.Problem(3, 1 / 16, seed=1001)
    b = pr.rhs()
    u = np.linalg.solve(pr.op(O.OP_A).todense(), b)
    mg = O.Multigrid(pr, npre=2, npost=2)
    x, hist, _ = pr.pcg(b, mg=mg, tol=1e-10)
    assert len(hist) < 20
    assert np.abs(x - u).max() <= 1e-8 * np.abs(u).max()


def test_ratrat_coarse_mass_block_diagonal_and_symmetric():
    pr = O.Problem(3, 1 / 8)
    mg = O.Multigrid(pr, npre=2, npost=2)
    for l in range(1, mg.nlevels):
        M = mg.level_op(l, O.OP_M)
        assert np.array_equal(M.col_idx, np.arange(M.nbr))
        A = mg.level_op(l, O.OP_A).todense()
        assert np.abs(A - A.T).max() <= 1e-10 * np.abs(A).max()


def test_adaptive_mesh_with_hanging_faces():
    # dg_tests.cpp:212-215 refines x < 0.5 further: non-canonical faces
    pr = O.Problem(3, 1 / 4, refine=O.REFINE_REF_ADAPTIVE, test=O.TEST_GAUSSIAN)
    A = pr.op(O.OP_A).todense()
    assert pr.ne > 16
    assert np.abs(A - A.T).max() <= 1e-10 * np.abs(A).max()
    assert np.linalg.eigvalsh(0.5 * (A + A.T)).min() > 0
    mg = O.Multigrid(pr, npre=2, npost=2)
    x, hist, _ = pr.pcg(pr.rhs(), mg=mg, tol=1e-10)
    assert hist[-1] < 1e-8 * max(1.0, hist[0])


@pytest.mark.parametrize("degrees,nh", [([4, 2], 3), ([4, 3, 2], 3)])
def test_hp_multigrid_converges_and_transfers_interpolate(degrees, nh):
    # Multigrid<N,P1,P2,...> (multigrid.h:436-560): p-levels, then h-levels
    pr = O.Problem(degrees[0], 1 / 16, seed=1001)
    mg = O.Multigrid.hp(pr, degrees, nh, npre=2, npost=2, solver=O.COARSE_DENSE, mean_project=False)
    assert mg.nlevels == len(degrees) + nh
    for l in range(mg.nlevels - 1):
        T = mg.transfer(l)
        assert np.allclose(T.matvec(np.ones(T.nbc * T.bc)), 1.0, atol=1e-13)
    x, hist, _ = pr.pcg(pr.rhs(), mg=mg, tol=1e-10)
    assert len(hist) < 30
    u = np.linalg.solve(pr.op(O.OP_A).todense(), pr.rhs())
    assert np.abs(x - u).max() <= 1e-8 * np.abs(u).max()


def test_gaussian_params_deterministic():
    a = O.gaussian_params(1001)
    b = O.gaussian_params(1001)
    c = O.gaussian_params(1002)
    assert all(np.array_equal(x, y) for x, y in zip(a, b))
    assert not np.array_equal(a[0], c[0])
    cx, cy, w, amp = a
    assert np.all((cx >= 0) & (cx < 1)) and np.all((w >= 0.05) & (w <= 0.2))

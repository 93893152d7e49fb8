"""On-disk formats (Matrix Market, .fun) written by the library against the
same files written by the oracle in the reference's format, and read back."""
import numpy as np
import pytest

import mgldg
import oracle_py as O

pytestmark = pytest.mark.gpu


def load_mtx(path):
    with open(path) as f:
        head = f.readline()
        assert head.startswith("%%MatrixMarket matrix coordinate real general")
        rows, cols, nnz = (int(v) for v in f.readline().split())
    data = np.loadtxt(path, skiprows=2).reshape(-1, 3)
    assert len(data) == nnz
    D = np.zeros((rows, cols))
    D[data[:, 0].astype(int) - 1, data[:, 1].astype(int) - 1] = data[:, 2]
    return D, nnz


def test_matrix_market_matches_oracle_and_round_trips(ctx, tmp_path):
    n, P = 8, 3
    prob = mgldg.CartesianProblem(ctx, P, n)
    pr = O.Problem(P, 1 / n, tau0=n, tauD=n)
    for which in (O.OP_M, O.OP_G0, O.OP_T, O.OP_A):
        ours, theirs = tmp_path / f"ours{which}.mtx", tmp_path / f"ref{which}.mtx"
        prob.ops.get(which).write_mtx(ours)
        pr.write_mtx(which, theirs)
        Do, nnz_o = load_mtx(ours)
        Dr, nnz_r = load_mtx(theirs)
        assert nnz_o == nnz_r
        assert np.abs(Do - Dr).max() <= 1e-13 * np.abs(Dr).max()
        back = mgldg.SparseBlockMatrix.read_mtx(ctx, theirs, P * P, P * P)
        rp, ci, v = back.download()
        csr = pr.op(which)
        assert np.array_equal(rp, csr.row_ptr) and np.array_equal(ci, csr.col_idx)
        assert np.array_equal(v, csr.vals)   # 17 digits round-trip exactly


def test_fun_file_matches_oracle(ctx, tmp_path):
    n, P = 8, 3
    prob = mgldg.CartesianProblem(ctx, P, n)
    pr = O.Problem(P, 1 / n, tau0=n, tauD=n, seed=5)
    u = np.random.default_rng(0).standard_normal(prob.ndof)
    prob.write_fun(u, tmp_path / "ours.fun")
    pr.write_fun(u, tmp_path / "ref.fun")
    a, b = open(tmp_path / "ours.fun").read().split("\n"), open(tmp_path / "ref.fun").read().split("\n")
    assert a[0] == b[0] == f"{P} 2 {n * n}"
    assert [len(l) == 0 for l in a] == [len(l) == 0 for l in b]
    A = np.array([[float(t) for t in l.split()] for l in a[1:] if l])
    B = np.array([[float(t) for t in l.split()] for l in b[1:] if l])
    assert np.array_equal(A, B)


def test_read_mtx_rejects_bad_files(ctx, tmp_path):
    p = tmp_path / "bad.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real general\n4 4 1\n5 1 2.0\n")
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.SparseBlockMatrix.read_mtx(ctx, p, 2, 2)
    assert e.value.code == mgldg.ERR_ARG
    p.write_text("%%MatrixMarket matrix coordinate real general\n3 3 1\n1 1 2.0\n")
    with pytest.raises(mgldg.MgldgError) as e:
        mgldg.SparseBlockMatrix.read_mtx(ctx, p, 2, 2)
    assert e.value.code == mgldg.ERR_SHAPE

"""CPU checks of the unstructured (triangle) path: the master element, the
disk mesher and .mesh reader (libmgldg host code, no GPU), and the oracle's
restatement of the reference's unstructured LDG discretisation
(src/unstructured/dg/ldgpoisson.tpp:27-100) pinned by the reference test's
exact solution u = (1 - |x|^2)/4 for f = 1 (tests/unstructured/dg_tests.cpp:
24-25) and by its second-order convergence on polygonal disks.
"""
import numpy as np
import pytest

import oracle_py as O

mgldg = pytest.importorskip("mgldg")
spla = pytest.importorskip("scipy.sparse.linalg")
sp = pytest.importorskip("scipy.sparse")
import adjoint_ref as R  # noqa: E402


def _lib_or_skip():
    try:
        mgldg.lib()
    except RuntimeError as e:
        pytest.skip(str(e))


@pytest.mark.parametrize("N,P", [(1, 1), (1, 3), (2, 1), (2, 2), (2, 3), (2, 4), (3, 1), (3, 2), (3, 3)])
def test_master_matches_oracle(N, P):
    _lib_or_skip()
    m, d, nodes = mgldg.simplex_master(N, P)
    mo, do, no = O.simplex_master(N, P)
    assert np.array_equal(nodes, no)
    assert np.abs(m - mo).max() <= 1e-15
    for a, c in zip(d, do):
        assert np.abs(a - c).max() <= 1e-14 * max(1, np.abs(c).max())
    # mass integrates 1 to the master volume; rows of diff kill constants
    vref = {1: 1.0, 2: 0.5, 3: 1 / 6}[N]
    assert abs(m.sum() - vref) <= 1e-15
    for a in d:
        assert np.abs(a.sum(axis=1)).max() <= 1e-13
    # diff of x_k at the nodes is the unit vector (linear functions need P >= 2)
    for k, a in enumerate(d if P >= 2 else []):
        for j in range(N):
            assert np.allclose(a @ nodes[:, j], 1.0 if j == k else 0.0, atol=1e-13)


def test_disk_mesh_is_a_conforming_triangulation():
    _lib_or_skip()
    p, t = mgldg.disk_mesh(0.05)
    assert np.all(t >= 0) and np.all(t < len(p))
    a = p[t[:, 1]] - p[t[:, 0]]
    b = p[t[:, 2]] - p[t[:, 0]]
    area = 0.5 * (a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])
    assert np.all(area > 0)
    assert abs(area.sum() - np.pi) < 0.01
    edges = {}
    for tri in t:
        for j in range(3):
            e = tuple(sorted((tri[j], tri[(j + 1) % 3])))
            edges[e] = edges.get(e, 0) + 1
    assert set(edges.values()) <= {1, 2}
    bverts = {v for e, c in edges.items() if c == 1 for v in e}
    r = np.linalg.norm(p[list(bverts)], axis=1)
    assert np.allclose(r, 1.0, atol=1e-14)
    assert len(p) - len(edges) + len(t) == 1          # Euler characteristic of a disk


def test_mesh_file_round_trip(tmp_path):
    _lib_or_skip()
    p, t = mgldg.disk_mesh(0.2)
    path = tmp_path / "disk.mesh"
    with open(path, "w") as f:
        f.write(f"{len(p)} {len(t)}\n")
        f.write("p\n")
        for x, y in p:
            f.write(f"{float(x)!r} {float(y)!r}\n")
        f.write("\n")
        for tri in t:
            f.write(f"{tri[0] + 1} {tri[1] + 1} {tri[2] + 1}\n")
        f.write("\n")
    q, s = mgldg.read_mesh(path)
    assert np.array_equal(q, p) and np.array_equal(s, t)
    bad = tmp_path / "bad.mesh"
    bad.write_text("3 1\np\n0 0\n1 0\n0 1\n\n1 2 4\n")
    with pytest.raises(mgldg.MgldgError):
        mgldg.read_mesh(bad)


def _nodes(p, t, P):
    _, _, nodes = O.simplex_master(2, P)
    P0 = p[t[:, 0]]
    J = np.stack([p[t[:, 1]] - P0, p[t[:, 2]] - P0], axis=2)     # ne x 2 x 2
    return (P0[:, None, :] + np.einsum("eij,qj->eqi", J, nodes)).reshape(-1, 2)


def test_oracle_reproduces_the_reference_disk_solution():
    _lib_or_skip()
    errs = []
    for h in (0.2, 0.1, 0.05):
        p, t = mgldg.disk_mesh(h)
        pr = O.Problem.simplex(p, t, 3, 1 / h, 1 / h, agg_levels=2, seed=0)
        A = R.to_scipy(pr.op(O.OP_A)).tocsc()
        assert abs(A - A.T).max() <= 1e-13 * abs(A).max()
        u = spla.spsolve(A, pr.rhs())
        X = _nodes(p, t, 3)
        errs.append(np.abs(u - (1 - (X ** 2).sum(1)) / 4).max())
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert errs[-1] < 2e-4 and np.all(rates > 1.8)


def test_agglomeration_covers_and_coarsens():
    _lib_or_skip()
    p, t = mgldg.disk_mesh(0.05)
    pr = O.Problem.simplex(p, t, 3, 20.0, 20.0, agg_levels=6)
    n = pr.ne
    for l in range(pr.nlevels - 1):
        a = pr.partition(l)
        assert len(a) == n
        counts = np.bincount(a)
        assert counts.min() >= 1 and len(counts) < n
        assert np.median(counts) >= 3
        n = len(counts)
    H = pr.hierarchy()
    assert (H[0].br, H[0].bc) == (6, 9) and all((T.br, T.bc) == (9, 9) for T in H[1:])
    # each aggregate's coarse basis is orthonormal in the fine mass inner
    # product (T0^T M T0 = I), and the coarse space still holds the constants
    M = R.to_scipy(pr.op(O.OP_M))
    T0 = R.to_scipy(H[0])
    G = (T0.T @ M @ T0).toarray()
    assert np.abs(G - np.eye(len(G))).max() <= 1e-6
    c, *_ = np.linalg.lstsq(T0.toarray(), np.ones(T0.shape[0]), rcond=None)
    assert np.abs(T0 @ c - 1).max() <= 1e-8


def test_external_agglomerator_graph_and_checks():
    # the oracle hands an external agglomerator each level's dual graph
    # (MGridGen's argument list) and rejects partitions that are out of
    # range, leave an aggregate empty or report a bad count
    _lib_or_skip()
    p, t = mgldg.disk_mesh(0.2)
    seen = []

    def pairs(n, xadj, adjncy, adjwgt, vvol, vsurf, N, part):
        seen.append((n, xadj.copy(), adjncy.copy(), adjwgt.copy(), vvol.copy(), vsurf.copy(), N))
        part[:] = np.arange(n) // 2
        return (n + 1) // 2

    cb = O.set_agglomerator(pairs)
    try:
        pr = O.Problem.simplex(p, t, 2, 5.0, 5.0, agg_levels=2)
    finally:
        O.set_agglomerator(None)
    del cb
    n, xadj, adj, w, vol, surf, N = seen[0]
    assert N == 2 and n == pr.ne and xadj[0] == 0 and len(adj) == xadj[-1] == 2 * (pr.nfaces - pr.nbfaces)
    # symmetric weights, every element's volume, the disk's boundary measure
    W = {(u, adj[k]): w[k] for u in range(n) for k in range(xadj[u], xadj[u + 1])}
    assert all(abs(W[(v, u)] - wt) <= 1e-15 for (u, v), wt in W.items())
    assert abs(vol.sum() - np.pi) < 0.2 and abs(surf.sum() - 2 * np.pi) < 0.1
    assert np.array_equal(pr.partition(0), np.arange(pr.ne) // 2)
    # the next level's graph sums the first level's pairs
    assert seen[1][0] == (pr.ne + 1) // 2 and abs(seen[1][4].sum() - vol.sum()) <= 1e-12

    for bad in (lambda n, part: (part.__setitem__(slice(None), n), n),         # out of range
                lambda n, part: (part.__setitem__(slice(None), 0), 2),         # empty aggregate
                lambda n, part: (part.__setitem__(slice(None), 0), 0)):        # bad count
        cb = O.set_agglomerator(lambda n, xa, aj, aw, vv, vs, N, part, f=bad: f(n, part)[1])
        try:
            with pytest.raises(RuntimeError):
                O.Problem.simplex(p, t, 2, 5.0, 5.0, agg_levels=2)
        finally:
            O.set_agglomerator(None)
        del cb


def test_ball_mesh_is_a_conforming_tetrahedralisation():
    _lib_or_skip()
    p, t = mgldg.ball_mesh(0.3)
    a, b, c = (p[t[:, k]] - p[t[:, 0]] for k in (1, 2, 3))
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)) / 6
    assert np.all(vol > 0)
    faces = {}
    edges = set()
    for tet in t:
        for j in range(4):
            f = tuple(sorted(tet[(j + k) % 4] for k in range(3)))
            faces[f] = faces.get(f, 0) + 1
        for i in range(4):
            for k in range(i + 1, 4):
                edges.add(tuple(sorted((tet[i], tet[k]))))
    assert set(faces.values()) <= {1, 2}
    bverts = {v for f, c in faces.items() if c == 1 for v in f}
    assert np.allclose(np.linalg.norm(p[list(bverts)], axis=1), 1.0, atol=1e-14)
    assert len(p) - len(edges) + len(faces) - len(t) == 1     # Euler characteristic of a ball


def test_oracle_reproduces_the_ball_solution():
    # u = (1 - |x|^2)/6 solves -Lap u = 1 (tests/unstructured/dg_tests.cpp:24-25
    # with N = 3); P2 holds it exactly, so the error is the polyhedral boundary's
    _lib_or_skip()
    errs = []
    for h in (0.5, 0.35):
        p, t = mgldg.ball_mesh(h)
        pr = O.Problem.simplex(p, t, 3, 1 / h, 1 / h, agg_levels=1, seed=0)
        A = R.to_scipy(pr.op(O.OP_A)).tocsc()
        assert abs(A - A.T).max() <= 1e-13 * abs(A).max()
        u = spla.spsolve(A, pr.rhs())
        _, _, nodes = O.simplex_master(3, 3)
        P0 = p[t[:, 0]]
        J = np.stack([p[t[:, k]] - P0 for k in (1, 2, 3)], axis=2)
        X = (P0[:, None, :] + np.einsum("eij,qj->eqi", J, nodes)).reshape(-1, 3)
        errs.append(np.abs(u - (1 - (X ** 2).sum(1)) / 6).max())
    assert errs[0] < 0.06 and errs[-1] < errs[0] / 2.2


def test_morton_order_is_a_stable_permutation_and_keeps_gauss_seidel_chains_short():
    _lib_or_skip()
    p, t = mgldg.disk_mesh(0.05)
    # the mesher's output is already in Morton order: reordering is the identity
    assert np.array_equal(mgldg.morton_order(p, t), t)
    rng = np.random.default_rng(7)
    s = mgldg.morton_order(p, t[rng.permutation(len(t))])
    assert np.array_equal(np.sort(s, axis=0), np.sort(t, axis=0))
    assert {tuple(x) for x in s} == {tuple(x) for x in t}
    c = p[s].mean(axis=1)
    lo, hi = c.min(0), c.max(0)
    q = np.minimum(np.floor((c - lo) / (hi - lo) * 2.0 ** 31), 2.0 ** 31 - 1).astype(np.uint64)
    key = np.zeros(len(s), np.uint64)
    for b in range(30, -1, -1):
        for d in range(2):
            key = (key << np.uint64(1)) | ((q[:, d] >> np.uint64(b)) & np.uint64(1))
    assert np.all(np.diff(key.astype(np.float64)) >= 0)
    # the LDG operator reaches two elements: its Gauss-Seidel dependency
    # chain on the Morton-ordered disk stays far below the element count
    pr = O.Problem.simplex(p, t, 1, 20.0, 20.0, agg_levels=1, seed=0)
    A = pr.op(O.OP_A)
    for rev in (False, True):
        _, _, depth = mgldg.gs_levels(A.row_ptr, A.col_idx, rev)
        assert depth < len(t) // 8, depth
    with pytest.raises(mgldg.MgldgError):
        mgldg.morton_order(p, np.full_like(t, len(p)))


def test_tetrahedral_coarse_bases_drop_dependent_directions():
    # the tensor Q2 space interpolated at the P2 nodes of a few tetrahedra is
    # rank deficient; dependent directions become exact zero columns, the
    # kept ones are mass-orthonormal, and the V-cycle over the result is a
    # working preconditioner
    _lib_or_skip()
    p, t = mgldg.ball_mesh(0.1)
    pr = O.Problem.simplex(p, t, 3, 1 / 0.1, 1 / 0.1, agg_levels=6, agg_seed=5000, seed=4001)
    H = pr.hierarchy()
    M = R.to_scipy(pr.op(O.OP_M))
    T0 = R.to_scipy(H[0])
    G = (T0.T @ M @ T0).tocsr()
    d = G.diagonal()
    off = G - sp.diags(d)
    assert (abs(off).max() if off.nnz else 0.0) <= 1e-6
    assert np.all((np.abs(d - 1) <= 1e-6) | (d == 0))
    zero_cols = np.flatnonzero(abs(T0).sum(axis=0).A1 == 0)
    assert len(zero_cols) > 0 and np.array_equal(zero_cols, np.flatnonzero(d == 0))
    for Tl in H:
        assert np.abs(Tl.vals).max() <= 1e4
    # constants stay in the coarse space: on each aggregate they are
    # M-orthogonal to nothing dropped, so the M-projection of 1 reproduces 1
    one = np.ones(T0.shape[0])
    assert np.abs(T0 @ (T0.T @ (M @ one)) - one).max() <= 1e-6
    p, t = mgldg.ball_mesh(0.2)
    pr = O.Problem.simplex(p, t, 3, 1 / 0.2, 1 / 0.2, agg_levels=6, agg_seed=5000, seed=4001)
    b = pr.rhs()
    for relax, omega, its in ((O.RELAX_GS, 1.0, 40), (O.RELAX_JACOBI, 0.4, 75)):
        mg = O.Multigrid(pr, relaxation=relax, omega=omega, npre=2, npost=2, solver=O.COARSE_DENSE,
                         restriction=O.RESTRICT_RAT, mean_project=False)
        x, hist, _ = pr.pcg(b, mg=mg, tol=1e-10, maxit=200)
        assert len(hist) < its, (relax, len(hist))
        A = R.to_scipy(pr.op(O.OP_A))
        assert np.linalg.norm(b - A @ x) <= 1e-9 * np.linalg.norm(b)


@pytest.mark.parametrize("h", [0.3, 0.1, 0.05, 0.03])
def test_ball_mesh_quality_does_not_degrade_with_h(h):
    # no tetrahedron has four vertices on the sphere, so no sliver flattens
    # as h shrinks: aspect ratio (longest edge^3 / (6 sqrt2 volume), 1 for a
    # regular tetrahedron) stays bounded
    _lib_or_skip()
    p, t = mgldg.ball_mesh(h)
    on_sphere = np.abs(np.linalg.norm(p, axis=1) - 1) < 1e-12
    assert not np.any(on_sphere[t].all(axis=1))
    a, b, c = (p[t[:, k]] - p[t[:, 0]] for k in (1, 2, 3))
    vol = np.einsum("ij,ij->i", a, np.cross(b, c)) / 6
    E = np.stack([np.linalg.norm(p[t[:, i]] - p[t[:, j]], axis=1) for i in range(4) for j in range(i + 1, 4)], 1)
    q = E.max(1) ** 3 / (6 * np.sqrt(2) * vol)
    assert q.max() < 15 and np.median(q) < 6, (q.max(), np.median(q))
    # Morton order already: reordering is the identity
    assert np.array_equal(mgldg.morton_order(p, t), t)

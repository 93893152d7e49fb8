"""The reference's own mesh files (data/*.mesh: the unit squares of its L2
projection test, the circles of its unstructured LDG test, a ball), copied
into oracle/_ref/data by oracle/Makefile when the reference tree is present
(the tests skip otherwise).

* The product's wireframe reader (mgldg_mesh_read / mgldg_mesh_read_nd,
  Wireframe<N>, wireframe.h:24-67) reads every file: counts as in the header,
  a conforming simplicial complex whose boundary facets lie on the domain's
  boundary.
* The oracle runs the reference's unstructured test case itself
  (tests/unstructured/dg_tests.cpp: data/circle.mesh, P2, zero Dirichlet,
  f = 1, tau0 = 100, tauD = 1000) and solves it: A symmetric, and the
  solution approaches u = (1 - |x|^2)/4 as the mesh is refined (circle ->
  circle2).  Measured: 6.8e-2 and 3.8e-3 of max|u| (the polygonal boundary
  dominates the error).
"""
import os
from collections import Counter

import numpy as np
import pytest

import oracle_py as O

mgldg = pytest.importorskip("mgldg")
spla = pytest.importorskip("scipy.sparse.linalg")
import adjoint_ref as R  # noqa: E402

DATA = os.path.join(os.path.dirname(O.__file__), "_ref", "data")
pytestmark = pytest.mark.skipif(not os.path.isdir(DATA), reason="reference mesh files not copied (reference absent)")

MESHES = [("square_4", 2), ("square_8", 2), ("square_16", 2), ("square_32", 2), ("square", 2),
          ("circle", 2), ("circle2", 2), ("ball", 3)]


def _read(name, N):
    try:
        mgldg.lib()
    except RuntimeError as e:
        pytest.skip(str(e))
    return mgldg.read_mesh(os.path.join(DATA, name + ".mesh"), N=N)


@pytest.mark.parametrize("name,N", MESHES)
def test_reader_reads_the_reference_meshes(name, N):
    p, t = _read(name, N)
    with open(os.path.join(DATA, name + ".mesh")) as f:
        np_, nt = (int(v) for v in f.readline().split())
    assert p.shape == (np_, N) and t.shape == (nt, N + 1)
    assert t.min() >= 0 and t.max() < np_
    # every facet of the complex belongs to one element (boundary) or two
    facets = Counter()
    for s in t:
        for k in range(N + 1):
            facets[tuple(sorted(np.delete(s, k)))] += 1
    assert set(facets.values()) <= {1, 2}
    bnd = np.array([f for f, c in facets.items() if c == 1])
    x = p[bnd.ravel()]
    if name.startswith("square"):
        assert np.all(np.min(np.minimum(np.abs(x), np.abs(x - 1)), axis=1) <= 1e-12)
    else:
        assert np.allclose(np.linalg.norm(x, axis=1), 1.0, atol=1e-5)
    # no degenerate simplices
    J = np.stack([p[t[:, k + 1]] - p[t[:, 0]] for k in range(N)], axis=2)
    assert np.abs(np.linalg.det(J)).min() > 0


def test_3d_reader_rejects_a_2d_file():
    with pytest.raises(mgldg.MgldgError):
        _read("circle", 3)
    with pytest.raises(mgldg.MgldgError):
        _read("ball", 2)


def _nodes(p, t, P):
    _, _, nd = O.simplex_master(2, P)
    P0 = p[t[:, 0]]
    J = np.stack([p[t[:, 1]] - P0, p[t[:, 2]] - P0], axis=2)
    return (P0[:, None, :] + np.einsum("eij,qj->eqi", J, nd)).reshape(-1, 2)


def test_oracle_solves_the_reference_circle_test_case():
    errs = []
    for name in ("circle", "circle2"):
        p, t = _read(name, 2)
        pr = O.Problem.simplex(p, t, 3, 100.0, 1000.0, agg_levels=1, seed=0)   # P2, f = 1
        A = R.to_scipy(pr.op(O.OP_A)).tocsc()
        assert abs(A - A.T).max() <= 1e-15 * abs(A).max()
        u = spla.spsolve(A, pr.rhs())
        ex = (1 - (_nodes(p, t, 3) ** 2).sum(1)) / 4
        errs.append(np.abs(u - ex).max() / np.abs(ex).max())
    assert errs[0] <= 0.08 and errs[1] <= 0.005 and errs[0] / errs[1] >= 10, errs

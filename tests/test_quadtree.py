"""Host-side adaptive quadtree (libmgldg, no GPU needed) against the oracle's
Quadtree<2>(h) (quadtree.tpp:10-40) and its 2:1 balance extension.

The leaf layer must list the same cells in the same depth-first order
(bit-exact integer work), for the reference's own adaptive mesh-size
function (dg_tests.cpp:212-215, passed as a Python callback) and for the
built-in seeded-points rule, balanced and unbalanced.
"""
import numpy as np
import pytest

import oracle_py as O

mgldg = pytest.importorskip("mgldg")


def _lib_or_skip():
    try:
        mgldg.lib()
    except RuntimeError as e:
        pytest.skip(str(e))


def boxes(qt):
    lev, ix, iy = qt.layer(0)
    w = np.ldexp(1.0, -lev)
    lo = np.stack([ix * w, iy * w], axis=1)
    return lo, lo + w[:, None]


@pytest.mark.parametrize("dx", [0.25, 0.125, 1 / 16])
def test_reference_adaptive_tree_matches_oracle(dx):
    _lib_or_skip()
    # h_adaptive (dg_tests.cpp:212-215)
    qt = mgldg.Quadtree(lambda x, y: dx if x > 0.5 else (0.25 * dx if x > 0.25 else 0.5 * dx))
    pr = O.Problem(2, dx, refine=O.REFINE_REF_ADAPTIVE)
    lo, hi = boxes(qt)
    rlo, rhi = pr.elements()
    assert np.array_equal(lo, rlo) and np.array_equal(hi, rhi)
    assert qt.nlevels == pr.nlevels


@pytest.mark.parametrize("base,extra,radius,balance", [(3, 3, 0.5, True), (4, 4, 0.5, True), (3, 4, 0.5, False),
                                                      (5, 3, 0.5, True), (3, 5, 0.1, True), (3, 5, 0.1, False)])
def test_points_tree_matches_oracle(base, extra, radius, balance):
    _lib_or_skip()
    pts = mgldg.seeded_points(3000, 4)
    assert np.array_equal(pts, O.seeded_points(3000, 4))
    qt = mgldg.Quadtree.points(pts, base, extra, radius=radius, balance=balance)
    pr = O.Problem.points(2, base, extra, radius=radius, balance=balance)
    lo, hi = boxes(qt)
    rlo, rhi = pr.elements()
    assert len(lo) == pr.ne
    assert np.array_equal(lo, rlo) and np.array_equal(hi, rhi)
    assert qt.nlevels == pr.nlevels


def _max_face_jump(qt):
    # largest level difference between face-adjacent leaves (brute force)
    lev, _, _ = qt.layer(0)
    lo, hi = boxes(qt)
    worst = 0
    for a in range(len(lev)):
        for d in (0, 1):
            t = 1 - d
            touch = (hi[a, d] == lo[:, d]) & (np.minimum(hi[a, t], hi[:, t]) > np.maximum(lo[a, t], lo[:, t]))
            if touch.any():
                worst = max(worst, int(np.abs(lev[touch] - lev[a]).max()))
    return worst


def test_balance_is_two_to_one():
    _lib_or_skip()
    pts = mgldg.seeded_points(3000, 4)
    # radius 0.1 refines sharply (jumps of 3 levels); radius 0.5 (the
    # multi-RHS workload's rule) grades geometrically and is already 2:1
    unbal = mgldg.Quadtree.points(pts, 3, 5, radius=0.1, balance=False)
    bal = mgldg.Quadtree.points(pts, 3, 5, radius=0.1, balance=True)
    assert _max_face_jump(unbal) >= 2
    assert _max_face_jump(bal) == 1
    assert bal.nleaves > unbal.nleaves
    assert bal.nlevels == unbal.nlevels
    graded = mgldg.Quadtree.points(pts, 3, 4, balance=False)
    assert _max_face_jump(graded) <= 1
    # a step in h: width 2^-6 left of x = 0.2, 2^-2 elsewhere
    h = lambda x, y: 2.0 ** -6 if x < 0.2 else 0.25
    assert _max_face_jump(mgldg.Quadtree(h, balance=False)) >= 2
    assert _max_face_jump(mgldg.Quadtree(h, balance=True)) == 1


def test_layers_shrink_to_the_root():
    _lib_or_skip()
    pts = mgldg.seeded_points(3000, 4)
    qt = mgldg.Quadtree.points(pts, 3, 3)
    sizes = [len(qt.layer(l)[0]) for l in range(qt.nlevels)]
    assert sizes[-1] == 1
    assert all(a >= b for a, b in zip(sizes, sizes[1:]))
    with pytest.raises(mgldg.MgldgError):
        qt.layer(qt.nlevels)

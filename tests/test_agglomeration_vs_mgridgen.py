"""Cross-check of the greedy seeded agglomeration (the product's simplex
hierarchy, bit-identical to the oracle's: tests/test_simplex_gpu.py) against
MGridGen, the agglomerator the reference calls
(src/unstructured/mesh/agglomeration.h:53-225 with minsize 1, maxsize 2^N,
options {4, 6, 1, N}; lib/ParMGridGen-1.0/MGridGen/Lib/mgridgen.c:18-51).

MGridGen is compiled from the reference's own vendored C sources into
oracle/_ref/libmgridgen.so by oracle/Makefile when the reference tree is
present; without it these tests skip.  The oracle builds the same disk
problem twice -- once with its greedy aggregates, once with MGridGen's
partitions of the same weighted dual graphs (face measures, element volumes,
boundary measures) -- and the tests compare the aggregates' shapes and the
MG-PCG iteration counts of the two hierarchies.

Measured on the 0.05 disk (2,514 triangles, Q2 on P_2 elements):
  level-1 aggregates   greedy 578 (mean isoperimetric ratio 1.70)
                       MGridGen 695 (1.44)
  level-2 aggregates   greedy 123 (2.01), MGridGen 203 (1.52)
  levels               greedy 5, MGridGen 7 (greedy coarsens 4.3x per level,
                       MGridGen 3.6x)
  PCG iterations       Jacobi: greedy 30, MGridGen 23
                       Gauss-Seidel: greedy 22, MGridGen 17
MGridGen's refinement buys rounder aggregates and about 25 % fewer
iterations; the greedy pass is a single sweep with no refinement and a
cheaper hierarchy.  On the reference's own distmesh circle (data/circle2.mesh,
661 triangles, its test's penalties tau0 = 100, tauD = 1000): greedy 33 / 26
iterations (Jacobi / Gauss-Seidel), MGridGen 28 / 22.  The bounds below hold those measured relations with a
margin, so a regression of the greedy aggregates shows up here.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle_py as O

mgldg = pytest.importorskip("mgldg")

LIB = os.path.join(os.path.dirname(O.__file__), "_ref", "libmgridgen.so")
pytestmark = pytest.mark.skipif(not os.path.exists(LIB), reason="MGridGen not built (reference tree absent)")

_IP, _DP = C.POINTER(C.c_int), C.POINTER(C.c_double)


def _mgridgen():
    lib = C.CDLL(LIB)
    lib.MGridGen.argtypes = [C.c_int, _IP, _DP, _DP, _IP, _DP, C.c_int, C.c_int, _IP, _IP, _IP, _IP]
    lib.MGridGen.restype = None
    calls = []

    def agglomerate(n, xadj, adjncy, adjwgt, vvol, vsurf, N, part):
        # private copies: MGridGen's arguments are not const
        xa, aj = np.array(xadj, np.int32), np.array(adjncy, np.int32)
        aw, vv, vs = np.array(adjwgt), np.array(vvol), np.array(vsurf)
        opts = (C.c_int * 4)(4, 6, 1, N)
        nmoves, nparts = C.c_int(), C.c_int()
        out = np.zeros(n, np.int32)
        lib.MGridGen(n, xa.ctypes.data_as(_IP), vv.ctypes.data_as(_DP), vs.ctypes.data_as(_DP),
                     aj.ctypes.data_as(_IP), aw.ctypes.data_as(_DP), 1, 1 << N, opts, C.byref(nmoves),
                     C.byref(nparts), out.ctypes.data_as(_IP))
        part[:] = out
        calls.append(n)
        return nparts.value

    return agglomerate, calls


def _hierarchies(h=0.05, P=3):
    try:
        mgldg.lib()
    except RuntimeError as e:
        pytest.skip(str(e))
    p, t = mgldg.disk_mesh(h)
    greedy = O.Problem.simplex(p, t, P, 1 / h, 1 / h, agg_levels=8)
    fn, calls = _mgridgen()
    cb = O.set_agglomerator(fn)
    try:
        mgg = O.Problem.simplex(p, t, P, 1 / h, 1 / h, agg_levels=8)
    finally:
        O.set_agglomerator(None)
    del cb
    assert calls and calls[0] == greedy.ne
    return greedy, mgg


@pytest.fixture(scope="module")
def hier():
    return _hierarchies()


def _levels(pr):
    return len(pr.hierarchy())


def test_both_partitions_cover_and_respect_maxsize(hier):
    greedy, mgg = hier
    for pr, cap in ((greedy, None), (mgg, 4)):
        n = pr.ne
        for l in range(_levels(pr)):
            a = pr.partition(l)
            assert len(a) == n
            counts = np.bincount(a)
            assert counts.min() >= 1 and len(counts) < n
            if cap:
                assert counts.max() <= cap   # MGridGen's maxsize 2^N
            n = len(counts)


def test_aggregate_shapes_against_mgridgen(hier):
    greedy, mgg = hier
    g1, m1 = greedy.agg_quality(0), mgg.agg_quality(0)
    # fewer, larger first-level aggregates (maxsize 4 plus merged remnants)
    assert g1[0] < m1[0]
    # rounder is better (1 = disk); greedy within 25 % of MGridGen's mean
    # ratio on the first level (measured 1.70 vs 1.44) and within 50 % on
    # the second (2.01 vs 1.52).  Deeper levels are not compared one to one:
    # greedy's hold far fewer aggregates (level 4: 6 against 18, ratios 3.73
    # against 1.81)
    assert g1[1] <= 1.25 * m1[1]
    assert greedy.agg_quality(1)[1] <= 1.5 * mgg.agg_quality(1)[1]
    # greedy coarsens faster: no more levels than MGridGen
    assert _levels(greedy) <= _levels(mgg)


@pytest.mark.parametrize("relax,omega", [(O.RELAX_JACOBI, 0.7), (O.RELAX_GS, 0.8)])
def test_pcg_iterations_against_mgridgen(hier, relax, omega):
    greedy, mgg = hier
    its = []
    for pr in (greedy, mgg):
        omg = O.Multigrid(pr, relaxation=relax, omega=omega, npre=2, npost=2, solver=O.COARSE_DENSE)
        _, hist, _ = pr.pcg(pr.rhs(), mg=omg, tol=1e-10)
        its.append(len(hist) - 1)
    # measured: Jacobi 30 vs 23, Gauss-Seidel 22 vs 17
    assert its[1] <= its[0] <= 1.4 * its[1], its


def test_iterations_on_the_reference_circle_mesh():
    # the reference's own input mesh, copied into oracle/_ref/data by
    # oracle/Makefile; measured 33 / 26 (greedy) against 28 / 22 (MGridGen)
    path = os.path.join(os.path.dirname(O.__file__), "_ref", "data", "circle2.mesh")
    if not os.path.exists(path):
        pytest.skip("reference mesh files not copied")
    p, t = mgldg.read_mesh(path)
    its = {}
    for name in ("greedy", "mgridgen"):
        cb = O.set_agglomerator(_mgridgen()[0]) if name == "mgridgen" else None
        try:
            pr = O.Problem.simplex(p, t, 3, 100.0, 1000.0, agg_levels=8, seed=0)
        finally:
            O.set_agglomerator(None)
        del cb
        its[name] = []
        for relax, omega in ((O.RELAX_JACOBI, 0.7), (O.RELAX_GS, 0.8)):
            omg = O.Multigrid(pr, relaxation=relax, omega=omega, npre=2, npost=2, solver=O.COARSE_DENSE)
            _, hist, _ = pr.pcg(pr.rhs(), mg=omg, tol=1e-10)
            its[name].append(len(hist) - 1)
    for g, m in zip(its["greedy"], its["mgridgen"]):
        assert m <= g <= 1.4 * m, its

"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg import
this module; the product never does.  The oracle restates the reference's
Cartesian solver path (danfortunato/multigrid-ldg, src/cartesian/...) in plain
C++ (oracle/oracle.cpp).
"""
import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

REFINE_UNIFORM, REFINE_REF_ADAPTIVE = 0, 1
BC_DIRICHLET, BC_NEUMANN, BC_PERIODIC = 0, 1, 2
TEST_CONVERGENCE, TEST_SOLUTION, TEST_GAUSSIAN = 0, 1, 2
RELAX_JACOBI, RELAX_GS = 0, 1
COARSE_CHOLESKY, COARSE_RELAX, COARSE_DENSE = 0, 1, 2
RESTRICT_RAT, RESTRICT_RATRAT = 0, 1
OP_M, OP_G0, OP_G1, OP_T, OP_A, OP_G2 = 0, 1, 2, 3, 4, 5

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_cip, _cdp = C.POINTER(C.c_int), C.POINTER(C.c_double)
# external agglomerator of the simplex hierarchies (oracle.h orc_agglomerator)
AGGLOMERATOR = C.CFUNCTYPE(C.c_int, C.c_int, _cip, _cip, _cdp, _cdp, _cdp, C.c_int, _cip)


def build():
    """Compile the oracle with its Makefile (gcc only, a few seconds)."""
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        vp = C.c_void_p
        pvp = C.POINTER(C.c_void_p)
        ip = C.POINTER(C.c_int)
        L.orc_master_tables.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp]
        L.orc_quadrature.argtypes = [C.c_int, _dp, _dp]
        L.orc_sbm_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, pvp]
        L.orc_sbm_set_block.argtypes = [vp, C.c_int, C.c_int, _dp]
        L.orc_sbm_add_block.argtypes = [vp, C.c_int, C.c_int, _dp]
        L.orc_sbm_mv.argtypes = [vp, C.c_double, _dp, C.c_double, _dp]
        L.orc_sbm_mv_t.argtypes = [vp, _dp, _dp]
        L.orc_sbm_destroy.argtypes = [vp]
        L.orc_problem_create.argtypes = [C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_double, C.c_double, C.c_uint64, pvp]
        L.orc_problem_destroy.argtypes = [vp]
        L.orc_problem_info.argtypes = [vp, ip, ip, ip, ip, ip, ip]
        L.orc_problem_elements.argtypes = [vp, _dp, _dp]
        L.orc_problem_nnzb.argtypes = [vp, C.c_int, ip]
        L.orc_problem_export.argtypes = [vp, C.c_int, _ip, _ip, _dp]
        L.orc_problem_rhs.argtypes = [vp, _dp]
        L.orc_problem_utrue.argtypes = [vp, _dp]
        L.orc_hier_size.argtypes = [vp, ip]
        L.orc_hier_shape.argtypes = [vp, C.c_int, ip, ip, ip]
        L.orc_hier_export.argtypes = [vp, C.c_int, _ip, _ip, _dp]
        L.orc_gaussian_params.argtypes = [C.c_uint64, _dp, _dp, _dp, _dp]
        L.orc_mg_create.argtypes = [vp, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.c_int, C.c_int, pvp]
        L.orc_mg_destroy.argtypes = [vp]
        L.orc_mg_create_hp.argtypes = [vp, _ip, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int,
                                       C.c_int, C.c_int, pvp]
        L.orc_mg_transfer_shape.argtypes = [vp, C.c_int, ip, ip, ip, ip, ip]
        L.orc_mg_transfer_export.argtypes = [vp, C.c_int, _ip, _ip, _dp]
        L.orc_mg_nlevels.argtypes = [vp, ip]
        L.orc_mg_level_nnzb.argtypes = [vp, C.c_int, C.c_int, ip, ip]
        L.orc_mg_level_export.argtypes = [vp, C.c_int, C.c_int, _ip, _ip, _dp]
        L.orc_mg_level_block.argtypes = [vp, C.c_int, ip]
        L.orc_mg_vcycle.argtypes = [vp, _dp, _dp]
        L.orc_mg_relax.argtypes = [vp, C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.orc_pcg.argtypes = [vp, vp, _dp, _dp, C.c_double, C.c_int, ip, _dp, _dp]
        L.orc_problem_mv.argtypes = [vp, C.c_int, C.c_double, _dp, C.c_double, _dp]
        L.orc_problem_write_mtx.argtypes = [vp, C.c_int, C.c_char_p]
        L.orc_problem_write_fun.argtypes = [vp, _dp, C.c_char_p]
        L.orc_problem_create_points.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_double,
                                                C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint64, pvp]
        L.orc_seeded_points.argtypes = [C.c_uint64, C.c_int, _dp]
        L.orc_simplex_problem_create.argtypes = [C.c_int, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double,
                                                 C.c_int, C.c_uint64, C.c_uint64, pvp]
        L.orc_hier_block.argtypes = [vp, C.c_int, ip, ip]
        L.orc_problem_partition.argtypes = [vp, C.c_int, _ip]
        L.orc_simplex_master.argtypes = [C.c_int, C.c_int, _dp, vp, vp, _dp]
        L.orc_simplex_problem_create_nd.argtypes = [C.c_int, C.c_int, _dp, C.c_int, _ip, C.c_int, C.c_double,
                                                    C.c_double, C.c_int, C.c_uint64, C.c_uint64, pvp]
        L.orc_simplex_master_nd.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.orc_set_agglomerator.argtypes = [AGGLOMERATOR]
        L.orc_problem_agg_quality.argtypes = [vp, C.c_int, _cip, _cdp, _cdp]
        _lib = L
    return _lib


def set_agglomerator(fn):
    """Python callable fn(n, xadj, adjncy, adjwgt, vvol, vsurf, N, part) -> count
    (numpy views of the level's dual graph; fills part) used by the simplex
    hierarchies created until the next call; None restores the greedy one.
    Returns the ctypes callback, which the caller keeps alive meanwhile."""
    if fn is None:
        lib().orc_set_agglomerator(AGGLOMERATOR())
        return None

    def tramp(n, xadj, adjncy, adjwgt, vvol, vsurf, N, part):
        try:
            xa = np.ctypeslib.as_array(xadj, (n + 1,))
            m = int(xa[n])
            views = (xa, np.ctypeslib.as_array(adjncy, (max(m, 1),))[:m],
                     np.ctypeslib.as_array(adjwgt, (max(m, 1),))[:m], np.ctypeslib.as_array(vvol, (n,)),
                     np.ctypeslib.as_array(vsurf, (n,)))
            return int(fn(n, *views, N, np.ctypeslib.as_array(part, (n,))))
        except Exception:
            return -1

    cb = AGGLOMERATOR(tramp)
    lib().orc_set_agglomerator(cb)
    return cb


def _ck(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle call {what} failed (rc={rc})")


def master_tables(P):
    out = [np.zeros(P), np.zeros(P), np.zeros(P * P), np.zeros(P * P), np.zeros(P * P)]
    _ck(lib().orc_master_tables(P, *out), "master_tables")
    nodes, denom, mass, invmass, diff = out
    return dict(nodes=nodes, denom=denom, mass=mass.reshape(P, P),
                invmass=invmass.reshape(P, P), diff=diff.reshape(P, P))


def quadrature(Q):
    x, w = np.zeros(Q), np.zeros(Q)
    _ck(lib().orc_quadrature(Q, x, w), "quadrature")
    return x, w


def simplex_master(N, P):
    """(mass, diff[N], nodes) of the master simplex (unstructured master.h)."""
    npl = {1: P, 2: P * (P + 1) // 2, 3: P * (P + 1) * (P + 2) // 6}[N]
    mass, diff, nodes = np.zeros(npl * npl), np.zeros(N * npl * npl), np.zeros(npl * N)
    _ck(lib().orc_simplex_master_nd(N, P, mass, diff, nodes), "simplex_master")
    return mass.reshape(npl, npl), list(diff.reshape(N, npl, npl)), nodes.reshape(npl, N)


def seeded_points(seed, n):
    xy = np.zeros(2 * n)
    _ck(lib().orc_seeded_points(seed, n, xy), "seeded_points")
    return xy.reshape(n, 2)


def gaussian_params(seed):
    out = [np.zeros(8) for _ in range(4)]
    _ck(lib().orc_gaussian_params(seed, *out), "gaussian_params")
    return out


class BlockMatrix:
    """SparseBlockMatrix<P,Q> (sparseblockmatrix.h:62-165)."""

    def __init__(self, m, n, P, Q=None):
        Q = P if Q is None else Q
        self.P, self.Q, self.m, self.n = P, Q, m, n
        h = C.c_void_p()
        _ck(lib().orc_sbm_create(m, n, P, Q, C.byref(h)), "sbm_create")
        self.h = h

    def set_block(self, i, j, blk):
        _ck(lib().orc_sbm_set_block(self.h, i, j, np.ascontiguousarray(blk, dtype=np.float64).ravel()), "set")

    def add_block(self, i, j, blk):
        _ck(lib().orc_sbm_add_block(self.h, i, j, np.ascontiguousarray(blk, dtype=np.float64).ravel()), "add")

    def mv(self, x, alpha=1.0, beta=0.0, y=None):
        y = np.zeros(self.m * self.P) if y is None else np.array(y, dtype=np.float64)
        _ck(lib().orc_sbm_mv(self.h, alpha, np.ascontiguousarray(x, dtype=np.float64), beta, y), "mv")
        return y

    def mv_t(self, x):
        y = np.zeros(self.n * self.Q)
        _ck(lib().orc_sbm_mv_t(self.h, np.ascontiguousarray(x, dtype=np.float64), y), "mv_t")
        return y

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_sbm_destroy(self.h)
            self.h = None


class CSR:
    """Block CSR export: row_ptr, col_idx (sorted), vals[nnzb, br, bc]."""

    def __init__(self, nbr, nbc, br, bc, row_ptr, col_idx, vals):
        self.nbr, self.nbc, self.br, self.bc = nbr, nbc, br, bc
        self.row_ptr, self.col_idx, self.vals = row_ptr, col_idx, vals

    @property
    def nnzb(self):
        return int(self.row_ptr[-1])

    def todense(self):
        D = np.zeros((self.nbr * self.br, self.nbc * self.bc))
        for i in range(self.nbr):
            for k in range(self.row_ptr[i], self.row_ptr[i + 1]):
                j = self.col_idx[k]
                D[i * self.br:(i + 1) * self.br, j * self.bc:(j + 1) * self.bc] = self.vals[k]
        return D

    def matvec(self, x):
        x = np.asarray(x).reshape(self.nbc, self.bc)
        y = np.zeros((self.nbr, self.br))
        rows = np.repeat(np.arange(self.nbr), np.diff(self.row_ptr))
        contrib = np.einsum("kij,kj->ki", self.vals, x[self.col_idx])
        np.add.at(y, rows, contrib)
        return y.ravel()


class Problem:
    """Quadtree -> Mesh -> LDGPoisson -> rhs (dg_tests.cpp:206-286)."""

    def __init__(self, P, dx, refine=REFINE_UNIFORM, coarsening=0, bc=BC_DIRICHLET,
                 test=TEST_GAUSSIAN, tau0=None, tauD=None, seed=1001):
        tau0 = 1.0 / dx if tau0 is None else tau0
        tauD = 1.0 / dx if tauD is None else tauD
        h = C.c_void_p()
        _ck(lib().orc_problem_create(P, dx, refine, coarsening, bc, test, tau0, tauD, seed,
                                     C.byref(h)), "problem_create")
        self._attach(h, P)

    @classmethod
    def points(cls, P, base_level, extra_levels, npoints=4, point_seed=3000, radius=0.5, balance=True,
               tau_per_face=True, tau0=1.0, tauD=1.0, seed=3001):
        """Adaptive quadtree of the seeded-points rule (see oracle.h)."""
        self = cls.__new__(cls)
        h = C.c_void_p()
        _ck(lib().orc_problem_create_points(P, base_level, extra_levels, npoints, point_seed, radius, int(balance),
                                            int(tau_per_face), tau0, tauD, seed, C.byref(h)), "create_points")
        self._attach(h, P)
        return self

    @classmethod
    def simplex(cls, points, tris, P, tau0, tauD, agg_levels=8, agg_seed=4000, seed=4001):
        """Unstructured P_{P-1} LDG on a triangle mesh (see oracle.h); seed 0: f = 1."""
        self = cls.__new__(cls)
        h = C.c_void_p()
        N = np.asarray(points).shape[1]
        p = np.ascontiguousarray(points, np.float64).ravel()
        t = np.ascontiguousarray(tris, np.int32).ravel()
        _ck(lib().orc_simplex_problem_create_nd(N, len(p) // N, p, len(t) // (N + 1), t, P, tau0, tauD, agg_levels,
                                                agg_seed, seed, C.byref(h)), "simplex_problem_create")
        self._attach(h, P)
        self.dim = N
        return self

    def partition(self, l):
        sizes = [self.ne]
        for k in range(l):
            sizes.append(int(self.partition(k).max()) + 1)
        agg = np.zeros(sizes[l], np.int32)
        _ck(lib().orc_problem_partition(self.h, l, agg), "partition")
        return agg

    def agg_quality(self, l):
        """(aggregates, mean and largest isoperimetric ratio) of agglomeration level l."""
        n, mean, mx = C.c_int(), C.c_double(), C.c_double()
        _ck(lib().orc_problem_agg_quality(self.h, l, C.byref(n), C.byref(mean), C.byref(mx)), "agg_quality")
        return n.value, mean.value, mx.value

    def _attach(self, h, P):
        self.h = h
        vals = [C.c_int() for _ in range(6)]
        _ck(lib().orc_problem_info(h, *[C.byref(v) for v in vals]), "info")
        self.ne, self.npl, self.ndof, self.nlevels, self.nfaces, self.nbfaces = [v.value for v in vals]
        self.P = P

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_problem_destroy(self.h)
            self.h = None

    def op(self, which):
        nnzb = C.c_int()
        _ck(lib().orc_problem_nnzb(self.h, which, C.byref(nnzb)), "nnzb")
        rp = np.zeros(self.ne + 1, np.int32)
        ci = np.zeros(nnzb.value, np.int32)
        v = np.zeros(nnzb.value * self.npl * self.npl)
        _ck(lib().orc_problem_export(self.h, which, rp, ci, v), "export")
        return CSR(self.ne, self.ne, self.npl, self.npl, rp, ci, v.reshape(-1, self.npl, self.npl))

    def rhs(self):
        b = np.zeros(self.ndof)
        _ck(lib().orc_problem_rhs(self.h, b), "rhs")
        return b

    def utrue(self):
        u = np.zeros(self.ndof)
        _ck(lib().orc_problem_utrue(self.h, u), "utrue")
        return u

    def elements(self):
        lo, hi = np.zeros(2 * self.ne), np.zeros(2 * self.ne)
        _ck(lib().orc_problem_elements(self.h, lo, hi), "elements")
        return lo.reshape(-1, 2), hi.reshape(-1, 2)

    def hierarchy(self):
        n = C.c_int()
        _ck(lib().orc_hier_size(self.h, C.byref(n)), "hier_size")
        out = []
        for l in range(n.value):
            nbr, nbc, nnzb = C.c_int(), C.c_int(), C.c_int()
            _ck(lib().orc_hier_shape(self.h, l, C.byref(nbr), C.byref(nbc), C.byref(nnzb)), "hshape")
            br, bc = C.c_int(), C.c_int()
            _ck(lib().orc_hier_block(self.h, l, C.byref(br), C.byref(bc)), "hblock")
            br, bc = br.value, bc.value
            rp = np.zeros(nbr.value + 1, np.int32)
            ci = np.zeros(nnzb.value, np.int32)
            v = np.zeros(nnzb.value * br * bc)
            _ck(lib().orc_hier_export(self.h, l, rp, ci, v), "hexport")
            out.append(CSR(nbr.value, nbc.value, br, bc, rp, ci, v.reshape(-1, br, bc)))
        return out

    def write_mtx(self, which, path):
        _ck(lib().orc_problem_write_mtx(self.h, which, str(path).encode()), "write_mtx")

    def write_fun(self, u, path):
        _ck(lib().orc_problem_write_fun(self.h, np.ascontiguousarray(u, np.float64), str(path).encode()), "write_fun")

    def mv(self, which, x, alpha=1.0, beta=0.0, y=None):
        y = np.zeros(self.ndof) if y is None else np.array(y, dtype=np.float64)
        _ck(lib().orc_problem_mv(self.h, which, alpha, np.ascontiguousarray(x, np.float64), beta, y), "mv")
        return y

    def pcg(self, b, x0=None, mg=None, tol=1e-10, maxit=200):
        x = np.zeros(self.ndof) if x0 is None else np.array(x0, dtype=np.float64)
        hist, dh = np.zeros(maxit), np.zeros(maxit)
        it = C.c_int()
        _ck(lib().orc_pcg(self.h, mg.h if mg is not None else None,
                          np.ascontiguousarray(b, np.float64), x, tol, maxit, C.byref(it), hist, dh), "pcg")
        return x, hist[:it.value].copy(), dh[:it.value].copy()


class Multigrid:
    """Multigrid<2,P>(ops, hierarchy, params) (multigrid.h:291-301)."""

    def __init__(self, problem, relaxation=RELAX_GS, omega=0.8, solver=COARSE_CHOLESKY, npre=3, npost=3,
                 restriction=RESTRICT_RATRAT, nlevels=0, mean_project=True):
        h = C.c_void_p()
        _ck(lib().orc_mg_create(problem.h, relaxation, omega, solver, npre, npost, restriction,
                                nlevels, int(mean_project), C.byref(h)), "mg_create")
        self.h = h
        self.pr = problem
        n = C.c_int()
        _ck(lib().orc_mg_nlevels(h, C.byref(n)), "nlevels")
        self.nlevels = n.value

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_mg_destroy(self.h)
            self.h = None

    @classmethod
    def hp(cls, problem, degrees, nh, relaxation=RELAX_GS, omega=0.8, solver=COARSE_CHOLESKY, npre=3, npost=3,
           restriction=RESTRICT_RATRAT, mean_project=True):
        """Multigrid<N,P1,P2,...>: p-levels over `degrees`, then nh h-levels."""
        self = cls.__new__(cls)
        h = C.c_void_p()
        deg = np.ascontiguousarray(degrees, dtype=np.int32)
        _ck(lib().orc_mg_create_hp(problem.h, deg, len(deg), nh, relaxation, omega, solver, npre, npost,
                                   restriction, int(mean_project), C.byref(h)), "mg_create_hp")
        self.h, self.pr = h, problem
        n = C.c_int()
        _ck(lib().orc_mg_nlevels(h, C.byref(n)), "nlevels")
        self.nlevels = n.value
        return self

    def transfer(self, l):
        """T[l]: interpolation from level l+1 to level l."""
        v = [C.c_int() for _ in range(5)]
        _ck(lib().orc_mg_transfer_shape(self.h, l, *[C.byref(x) for x in v]), "transfer_shape")
        nbr, nbc, br, bc, nnzb = [x.value for x in v]
        rp = np.zeros(nbr + 1, np.int32)
        ci = np.zeros(max(1, nnzb), np.int32)
        vals = np.zeros(max(1, nnzb * br * bc))
        _ck(lib().orc_mg_transfer_export(self.h, l, rp, ci, vals), "transfer_export")
        return CSR(nbr, nbc, br, bc, rp, ci[:nnzb], vals[:nnzb * br * bc].reshape(-1, br, bc))

    def level_op(self, l, which):
        nbr, nnzb = C.c_int(), C.c_int()
        _ck(lib().orc_mg_level_nnzb(self.h, l, which, C.byref(nbr), C.byref(nnzb)), "lnnzb")
        bb = C.c_int()
        _ck(lib().orc_mg_level_block(self.h, l, C.byref(bb)), "lblock")
        b = bb.value
        rp = np.zeros(nbr.value + 1, np.int32)
        ci = np.zeros(nnzb.value, np.int32)
        v = np.zeros(nnzb.value * b * b)
        _ck(lib().orc_mg_level_export(self.h, l, which, rp, ci, v), "lexport")
        return CSR(nbr.value, nbr.value, b, b, rp, ci, v.reshape(-1, b, b))

    def vcycle(self, b, x=None):
        x = np.zeros(len(b)) if x is None else np.array(x, dtype=np.float64)
        _ck(lib().orc_mg_vcycle(self.h, np.ascontiguousarray(b, np.float64), x), "vcycle")
        return x

    def relax(self, l, n, reverse, b, x):
        x = np.array(x, dtype=np.float64)
        _ck(lib().orc_mg_relax(self.h, l, n, int(reverse), np.ascontiguousarray(b, np.float64), x), "relax")
        return x

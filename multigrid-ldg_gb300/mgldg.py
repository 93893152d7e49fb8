"""Python host mirror of the reference's solver interface over the libmgldg C ABI.

The names follow danfortunato/multigrid-ldg: SparseBlockMatrix
(src/cartesian/util/sparseblockmatrix.h:62-165), LDGOperators
(src/cartesian/dg/ldgpoisson.h:15-53), MG parameters and Multigrid
(src/cartesian/multigrid/multigrid.h:48-62, 280-433) and pcg
(src/cartesian/multigrid/krylov.h:22-82).  Every call goes through the
C-ABI library libmgldg.so (CUDA, sm_103a); there is no CPU fallback: if the
library or a GPU is missing, the calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmgldg.so")

OK, ERR_ARG, ERR_SHAPE, ERR_CUDA, ERR_BREAKDOWN, ERR_TIMEOUT, ERR_NOT_SPD, ERR_NOMEM, ERR_UNSUPPORTED = range(9)
RELAX_JACOBI, RELAX_GAUSS_SEIDEL = 0, 1
COARSE_CHOLESKY, COARSE_RELAXATION, COARSE_DENSE = 0, 1, 2
RESTRICT_RAT, RESTRICT_RATRAT = 0, 1
PREC_FP64, PREC_MIXED, PREC_MIXED_F16, PREC_MIXED_TF32 = 0, 1, 2, 3
K_SPMV, K_GS, K_JACOBI, K_TRANSFER, K_COARSE, K_VECTOR, K_SETUP = range(7)
K_NAMES = ["spmv", "gauss_seidel", "jacobi", "transfer", "coarse", "vector", "setup"]

# every symbol declared in include/mgldg.h
EXPORTS = [
    "mgldg_ctx_create", "mgldg_ctx_destroy", "mgldg_last_error", "mgldg_ctx_sync", "mgldg_ctx_stream",
    "mgldg_master_tables", "mgldg_bsr_create", "mgldg_bsr_destroy", "mgldg_bsr_info", "mgldg_bsr_download",
    "mgldg_bsr_mv", "mgldg_bsr_mv_dev", "mgldg_bsr_mv_t", "mgldg_ops_create", "mgldg_ops_create_A",
    "mgldg_ops_construct_laplacian", "mgldg_ops_get", "mgldg_ops_destroy", "mgldg_mg_params_default",
    "mgldg_mg_create", "mgldg_mg_destroy", "mgldg_mg_nlevels", "mgldg_mg_level_op", "mgldg_mg_vcycle",
    "mgldg_mg_vcycle_dev", "mgldg_mg_relax", "mgldg_pcg", "mgldg_pcg_dev", "mgldg_cartesian_create",
    "mgldg_problem_destroy", "mgldg_problem_info", "mgldg_problem_ops", "mgldg_problem_interp",
    "mgldg_problem_rhs_gaussian", "mgldg_problem_rhs_gaussian_dev", "mgldg_prof_enable", "mgldg_prof_reset",
    "mgldg_prof_query", "mgldg_gs_levels", "mgldg_gs_pass_levels", "mgldg_selftest_wait_timeout", "mgldg_cg_noalloc_dev",
    "mgldg_prof_query_level", "mgldg_cartesian_h_interp", "mgldg_cartesian_p_interp",
    "mgldg_bsr_write_mtx", "mgldg_bsr_read_mtx", "mgldg_problem_write_fun",
    "mgldg_ops_construct_laplacian_kappa", "mgldg_kappa_gradient_dev", "mgldg_adjoint_l2_dev",
    "mgldg_bsr_mm_dev", "mgldg_mg_vcycle_batched_dev", "mgldg_pcg_batched_dev", "mgldg_pcg_batched",
    "mgldg_mg_batch_tiles", "mgldg_quadtree_create", "mgldg_quadtree_destroy", "mgldg_quadtree_info",
    "mgldg_quadtree_layer", "mgldg_h_points", "mgldg_seeded_points", "mgldg_quadtree_problem_create",
    "mgldg_problem_mesh_info", "mgldg_mesh_read", "mgldg_mesh_read_nd", "mgldg_disk_mesh", "mgldg_mesh_morton_order", "mgldg_simplex_problem_create",
    "mgldg_problem_partition", "mgldg_simplex_master", "mgldg_pcg_segmented_dev",
    "mgldg_simplex_problem_create_nd", "mgldg_ball_mesh", "mgldg_simplex_master_nd", "mgldg_bsr_clone",
    "mgldg_bsr_builder_create", "mgldg_bsr_builder_set", "mgldg_bsr_builder_add", "mgldg_bsr_builder_exists",
    "mgldg_bsr_builder_nnzb", "mgldg_bsr_builder_export", "mgldg_bsr_builder_finalize", "mgldg_bsr_builder_destroy",
]


def gs_levels(row_ptr, col_idx, reverse=False):
    """Host-side level schedule of a Gauss-Seidel sweep: (level per row, rows in level order, nlevels)."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col_idx, dtype=np.int32)
    if len(ci) == 0:
        ci = np.zeros(1, np.int32)
    n = len(rp) - 1
    lev = np.zeros(max(1, n), np.int32)
    order = np.zeros(max(1, n), np.int32)
    nl = C.c_int()
    rc = lib().mgldg_gs_levels(n, rp, ci, int(reverse), lev, order, C.byref(nl))
    if rc:
        raise MgldgError(rc, "gs_levels")
    return lev[:n], order[:n], nl.value


def gs_pass_levels(row_ptr, col_idx, nsw, reverse=False):
    """Host-side levels of an nsw-sweep Gauss-Seidel pass: (level[s, i] as an nsw x n array, nlevels)."""
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col_idx, dtype=np.int32)
    if len(ci) == 0:
        ci = np.zeros(1, np.int32)
    n = len(rp) - 1
    lev = np.zeros(max(1, nsw * n), np.int32)
    nl = C.c_int()
    rc = lib().mgldg_gs_pass_levels(n, rp, ci, int(reverse), nsw, lev, C.byref(nl))
    if rc:
        raise MgldgError(rc, "gs_pass_levels")
    return lev[:nsw * n].reshape(nsw, n), nl.value


class MgldgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libmgldg error {code}: {msg}")
        self.code = code


class MGParams(C.Structure):
    """MG::Parameters (multigrid.h:48-62) plus precision / level-count / mean-projection."""
    _fields_ = [("relaxation", C.c_int), ("omega", C.c_double), ("solver", C.c_int), ("npre", C.c_int),
                ("npost", C.c_int), ("restriction", C.c_int), ("precision", C.c_int), ("max_levels", C.c_int),
                ("mean_project", C.c_int)]


_lib = None
_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")


def lib():
    """Loads libmgldg.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run multigrid-ldg_gb300/build.py")
        L = C.CDLL(LIB_PATH)
        vp, pvp = C.c_void_p, C.POINTER(C.c_void_p)
        i64p = C.POINTER(C.c_int64)
        ip = C.POINTER(C.c_int)
        L.mgldg_ctx_create.argtypes = [C.c_int, pvp]
        L.mgldg_ctx_destroy.argtypes = [vp]
        L.mgldg_last_error.argtypes = [vp]
        L.mgldg_last_error.restype = C.c_char_p
        L.mgldg_ctx_sync.argtypes = [vp]
        L.mgldg_ctx_stream.argtypes = [vp]
        L.mgldg_ctx_stream.restype = C.c_void_p
        L.mgldg_master_tables.argtypes = [C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.mgldg_bsr_create.argtypes = [vp, C.c_int, C.c_int, C.c_int, C.c_int, _ip, _ip, _dp, pvp]
        L.mgldg_bsr_destroy.argtypes = [vp]
        L.mgldg_bsr_builder_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, pvp]
        L.mgldg_bsr_builder_set.argtypes = [vp, C.c_int, C.c_int, _dp]
        L.mgldg_bsr_builder_add.argtypes = [vp, C.c_int, C.c_int, _dp]
        L.mgldg_bsr_builder_exists.argtypes = [vp, C.c_int, C.c_int, ip]
        L.mgldg_bsr_builder_nnzb.argtypes = [vp, i64p]
        L.mgldg_bsr_builder_export.argtypes = [vp, vp, vp, vp]
        L.mgldg_bsr_builder_finalize.argtypes = [vp, vp, pvp]
        L.mgldg_bsr_builder_destroy.argtypes = [vp]
        L.mgldg_bsr_clone.argtypes = [vp, vp, pvp]
        L.mgldg_bsr_info.argtypes = [vp, ip, ip, ip, ip, i64p]
        L.mgldg_bsr_download.argtypes = [vp, vp, _ip, _ip, _dp]
        L.mgldg_bsr_mv.argtypes = [vp, C.c_double, vp, _dp, C.c_double, _dp]
        L.mgldg_bsr_mv_dev.argtypes = [vp, C.c_double, vp, vp, C.c_double, vp]
        L.mgldg_bsr_mv_t.argtypes = [vp, vp, _dp, _dp]
        L.mgldg_ops_create.argtypes = [vp, C.c_int, vp, C.POINTER(C.c_void_p), vp, pvp]
        L.mgldg_ops_create_A.argtypes = [vp, vp, pvp]
        L.mgldg_ops_construct_laplacian.argtypes = [vp, vp]
        L.mgldg_ops_get.argtypes = [vp, C.c_int, pvp]
        L.mgldg_ops_destroy.argtypes = [vp]
        L.mgldg_mg_params_default.argtypes = [C.POINTER(MGParams)]
        L.mgldg_mg_params_default.restype = None
        L.mgldg_mg_create.argtypes = [vp, vp, C.POINTER(C.c_void_p), C.c_int, C.POINTER(MGParams), pvp]
        L.mgldg_mg_destroy.argtypes = [vp]
        L.mgldg_mg_nlevels.argtypes = [vp, ip]
        L.mgldg_mg_level_op.argtypes = [vp, C.c_int, C.c_int, pvp]
        L.mgldg_mg_vcycle.argtypes = [vp, vp, _dp, _dp]
        L.mgldg_mg_vcycle_dev.argtypes = [vp, vp, vp, vp]
        L.mgldg_mg_relax.argtypes = [vp, vp, C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.mgldg_pcg.argtypes = [vp, vp, vp, _dp, _dp, C.c_double, C.c_int, ip, _dp]
        L.mgldg_pcg_dev.argtypes = [vp, vp, vp, vp, vp, C.c_double, C.c_int, ip, _dp]
        L.mgldg_cartesian_create.argtypes = [vp, C.c_int, C.c_int, C.c_double, C.c_double, pvp]
        L.mgldg_problem_destroy.argtypes = [vp]
        L.mgldg_problem_info.argtypes = [vp, ip, ip, i64p, ip]
        L.mgldg_problem_ops.argtypes = [vp, pvp]
        L.mgldg_problem_interp.argtypes = [vp, C.c_int, pvp]
        L.mgldg_problem_rhs_gaussian.argtypes = [vp, vp, C.c_uint64, _dp]
        L.mgldg_problem_rhs_gaussian_dev.argtypes = [vp, vp, C.c_uint64, vp]
        L.mgldg_prof_enable.argtypes = [vp, C.c_int]
        L.mgldg_prof_reset.argtypes = [vp]
        L.mgldg_prof_query.argtypes = [vp, C.c_int, i64p, C.POINTER(C.c_double)]
        L.mgldg_gs_levels.argtypes = [C.c_int, _ip, _ip, C.c_int, _ip, _ip, ip]
        L.mgldg_gs_pass_levels.argtypes = [C.c_int, _ip, _ip, C.c_int, C.c_int, _ip, ip]
        L.mgldg_selftest_wait_timeout.argtypes = [vp, C.c_int64, ip]
        L.mgldg_cg_noalloc_dev.argtypes = [vp, vp, vp, vp, C.c_double, C.c_int, ip, _dp]
        L.mgldg_prof_query_level.argtypes = [vp, C.c_int, C.c_int, i64p, C.POINTER(C.c_double)]
        L.mgldg_cartesian_h_interp.argtypes = [vp, C.c_int, C.c_int, pvp]
        L.mgldg_cartesian_p_interp.argtypes = [vp, C.c_int, C.c_int, C.c_int, pvp]
        L.mgldg_bsr_write_mtx.argtypes = [vp, vp, C.c_char_p]
        L.mgldg_bsr_read_mtx.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, pvp]
        L.mgldg_problem_write_fun.argtypes = [vp, vp, _dp, C.c_char_p]
        L.mgldg_ops_construct_laplacian_kappa.argtypes = [vp, vp, vp]
        L.mgldg_kappa_gradient_dev.argtypes = [vp, vp, vp, vp, vp]
        L.mgldg_adjoint_l2_dev.argtypes = [vp, vp, vp, vp, vp, C.c_double, C.c_int, vp, vp, vp,
                                           C.POINTER(C.c_double), ip]
        L.mgldg_bsr_mm_dev.argtypes = [vp, C.c_double, vp, C.c_int, vp, C.c_double, vp]
        L.mgldg_mg_vcycle_batched_dev.argtypes = [vp, vp, C.c_int, vp, vp]
        L.mgldg_pcg_batched_dev.argtypes = [vp, vp, vp, C.c_int, vp, vp, C.c_double, C.c_int, _ip, _dp]
        L.mgldg_pcg_batched.argtypes = [vp, vp, vp, C.c_int, _dp, _dp, C.c_double, C.c_int, _ip, _dp]
        L.mgldg_mg_batch_tiles.argtypes = [vp, C.c_int, ip, ip, ip, ip, ip]
        L.mgldg_quadtree_create.argtypes = [vp, vp, C.c_int, C.c_int, pvp]
        L.mgldg_quadtree_destroy.argtypes = [vp]
        L.mgldg_quadtree_info.argtypes = [vp, ip, ip, ip]
        L.mgldg_quadtree_layer.argtypes = [vp, C.c_int, ip, vp, vp, vp]
        L.mgldg_h_points.argtypes = [C.POINTER(C.c_double), vp]
        L.mgldg_h_points.restype = C.c_double
        L.mgldg_seeded_points.argtypes = [C.c_uint64, C.c_int, _dp]
        L.mgldg_quadtree_problem_create.argtypes = [vp, vp, C.c_int, C.c_double, C.c_double, C.c_int, pvp]
        L.mgldg_problem_mesh_info.argtypes = [vp, ip, ip, ip]
        L.mgldg_mesh_read.argtypes = [C.c_char_p, ip, ip, vp, vp]
        L.mgldg_mesh_read_nd.argtypes = [C.c_char_p, C.c_int, ip, ip, vp, vp]
        L.mgldg_disk_mesh.argtypes = [C.c_double, ip, ip, vp, vp]
        L.mgldg_simplex_problem_create.argtypes = [vp, C.c_int, _dp, C.c_int, _ip, C.c_int, C.c_double, C.c_double,
                                                   C.c_int, C.c_uint64, pvp]
        L.mgldg_problem_partition.argtypes = [vp, C.c_int, ip, vp]
        L.mgldg_simplex_master.argtypes = [C.c_int, C.c_int, _dp, vp, vp, _dp]
        L.mgldg_simplex_problem_create_nd.argtypes = [vp, C.c_int, C.c_int, _dp, C.c_int, _ip, C.c_int, C.c_double,
                                                      C.c_double, C.c_int, C.c_uint64, pvp]
        L.mgldg_ball_mesh.argtypes = [C.c_double, ip, ip, vp, vp]
        L.mgldg_mesh_morton_order.argtypes = [C.c_int, C.c_int, vp, C.c_int, vp]
        L.mgldg_simplex_master_nd.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp]
        L.mgldg_pcg_segmented_dev.argtypes = [vp, vp, vp, C.c_int, C.POINTER(C.c_int64), vp, vp, C.c_double,
                                              C.c_int, _ip, _dp]
        _lib = L
    return _lib


def master_tables(P):
    """Reference-element tables compiled into the library (master.h:147-214)."""
    out = [np.zeros(P), np.zeros(P), np.zeros(P * P), np.zeros(P * P), np.zeros(P * P), np.zeros(10), np.zeros(10)]
    rc = lib().mgldg_master_tables(P, *out)
    if rc:
        raise MgldgError(rc, "master_tables")
    nodes, denom, mass, invmass, diff, qx, qw = out
    return dict(nodes=nodes, denom=denom, mass=mass.reshape(P, P), invmass=invmass.reshape(P, P),
                diff=diff.reshape(P, P), quad_x=qx, quad_w=qw)


class Context:
    """One GPU and one CUDA stream (mgldg_ctx)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        rc = lib().mgldg_ctx_create(device, C.byref(h))
        if rc:
            raise MgldgError(rc, f"cannot create a context on device {device}")
        self.h = h

    def check(self, rc, what=""):
        if rc:
            raise MgldgError(rc, f"{what}: {lib().mgldg_last_error(self.h).decode()}")

    def sync(self):
        self.check(lib().mgldg_ctx_sync(self.h), "sync")

    @property
    def stream(self):
        return lib().mgldg_ctx_stream(self.h)

    def prof_enable(self, on=True):
        self.check(lib().mgldg_prof_enable(self.h, int(on)), "prof_enable")

    def prof_reset(self):
        self.check(lib().mgldg_prof_reset(self.h), "prof_reset")

    def prof(self):
        out = {}
        for k, name in enumerate(K_NAMES):
            n, ms = C.c_int64(), C.c_double()
            self.check(lib().mgldg_prof_query(self.h, k, C.byref(n), C.byref(ms)), "prof_query")
            out[name] = (n.value, ms.value)
        return out

    def prof_level(self, kclass, level):
        """(launches, ms) of one kernel class on one multigrid level (-1: outside the V-cycle)."""
        n, ms = C.c_int64(), C.c_double()
        self.check(lib().mgldg_prof_query_level(self.h, kclass, level, C.byref(n), C.byref(ms)), "prof_query_level")
        return n.value, ms.value

    def close(self):
        if getattr(self, "h", None):
            lib().mgldg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BlockBuilder:
    """Host-side block assembly with the reference's calls: reset (the
    constructor), setBlock, addToBlock, blockExists, nnzb; export() gives the
    sorted block-CSR, finalize(ctx) the GPU SparseBlockMatrix."""

    def __init__(self, nbr, nbc, br, bc):
        self.shape = (nbr, nbc, br, bc)
        self.h = C.c_void_p()
        rc = lib().mgldg_bsr_builder_create(nbr, nbc, br, bc, C.byref(self.h))
        if rc:
            raise MgldgError(rc, "bsr_builder_create")

    def _block(self, block):
        b = np.ascontiguousarray(block, dtype=np.float64).reshape(-1)
        if b.size != self.shape[2] * self.shape[3]:
            raise ValueError("block has the wrong size")
        return b

    def set_block(self, i, j, block):
        rc = lib().mgldg_bsr_builder_set(self.h, i, j, self._block(block))
        if rc:
            raise MgldgError(rc, "bsr_builder_set")

    def add_to_block(self, i, j, block):
        rc = lib().mgldg_bsr_builder_add(self.h, i, j, self._block(block))
        if rc:
            raise MgldgError(rc, "bsr_builder_add")

    def block_exists(self, i, j):
        e = C.c_int()
        rc = lib().mgldg_bsr_builder_exists(self.h, i, j, C.byref(e))
        if rc:
            raise MgldgError(rc, "bsr_builder_exists")
        return bool(e.value)

    def nnzb(self):
        n = C.c_int64()
        lib().mgldg_bsr_builder_nnzb(self.h, C.byref(n))
        return n.value

    def export(self):
        nbr, _, br, bc = self.shape
        n = self.nnzb()
        rp = np.zeros(nbr + 1, np.int32)
        ci = np.zeros(max(1, n), np.int32)
        v = np.zeros(max(1, n) * br * bc)
        rc = lib().mgldg_bsr_builder_export(self.h, rp.ctypes.data_as(C.c_void_p), ci.ctypes.data_as(C.c_void_p),
                                            v.ctypes.data_as(C.c_void_p))
        if rc:
            raise MgldgError(rc, "bsr_builder_export")
        return rp, ci[:n], v[:n * br * bc].reshape(n, br, bc)

    def finalize(self, ctx):
        h = C.c_void_p()
        ctx.check(lib().mgldg_bsr_builder_finalize(ctx.h, self.h, C.byref(h)), "bsr_builder_finalize")
        return SparseBlockMatrix(ctx, h)

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().mgldg_bsr_builder_destroy(self.h)
            except Exception:
                pass
            self.h = None


class SparseBlockMatrix:
    """Block-CSR matrix on the GPU (SparseBlockMatrix<P,Q>)."""

    def __init__(self, ctx, handle, owned=True):
        self.ctx, self.h, self.owned = ctx, handle, owned

    @classmethod
    def from_csr(cls, ctx, nbr, nbc, br, bc, row_ptr, col_idx, vals):
        h = C.c_void_p()
        rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
        ci = np.ascontiguousarray(col_idx, dtype=np.int32)
        v = np.ascontiguousarray(vals, dtype=np.float64).ravel()
        if len(ci) == 0:
            ci = np.zeros(1, np.int32)
            v = np.zeros(1)
        ctx.check(lib().mgldg_bsr_create(ctx.h, nbr, nbc, br, bc, rp, ci, v, C.byref(h)), "bsr_create")
        return cls(ctx, h)

    def clone(self):
        """A device-side copy owned by the caller."""
        h = C.c_void_p()
        self.ctx.check(lib().mgldg_bsr_clone(self.ctx.h, self.h, C.byref(h)), "bsr_clone")
        return SparseBlockMatrix(self.ctx, h)

    def info(self):
        a = [C.c_int() for _ in range(4)]
        nnzb = C.c_int64()
        self.ctx.check(lib().mgldg_bsr_info(self.h, *[C.byref(x) for x in a], C.byref(nnzb)), "bsr_info")
        return tuple(x.value for x in a) + (nnzb.value,)

    def download(self):
        nbr, nbc, br, bc, nnzb = self.info()
        rp = np.zeros(nbr + 1, np.int32)
        ci = np.zeros(max(1, nnzb), np.int32)
        v = np.zeros(max(1, nnzb * br * bc))
        self.ctx.check(lib().mgldg_bsr_download(self.ctx.h, self.h, rp, ci, v), "bsr_download")
        return rp, ci[:nnzb], v[:nnzb * br * bc].reshape(nnzb, br, bc)

    def mv(self, x, alpha=1.0, beta=0.0, y=None):
        nbr, nbc, br, bc, _ = self.info()
        y = np.zeros(nbr * br) if y is None else np.array(y, dtype=np.float64)
        self.ctx.check(lib().mgldg_bsr_mv(self.ctx.h, alpha, self.h, np.ascontiguousarray(x, np.float64), beta, y),
                       "bsr_mv")
        return y

    def mv_t(self, x):
        nbr, nbc, br, bc, _ = self.info()
        y = np.zeros(nbc * bc)
        self.ctx.check(lib().mgldg_bsr_mv_t(self.ctx.h, self.h, np.ascontiguousarray(x, np.float64), y), "bsr_mv_t")
        return y

    def write_mtx(self, path):
        """Matrix Market dump (the reference's SparseBlockMatrix::write format)."""
        self.ctx.check(lib().mgldg_bsr_write_mtx(self.ctx.h, self.h, str(path).encode()), "write_mtx")

    @classmethod
    def read_mtx(cls, ctx, path, br, bc):
        h = C.c_void_p()
        ctx.check(lib().mgldg_bsr_read_mtx(ctx.h, str(path).encode(), br, bc, C.byref(h)), "read_mtx")
        return cls(ctx, h)

    def release(self):
        """Gives up ownership (the C side took it)."""
        self.owned = False
        return self.h

    def __del__(self):
        if getattr(self, "owned", False) and self.h:
            try:
                lib().mgldg_bsr_destroy(self.h)
            except Exception:
                pass
            self.h = None


class LDGOperators:
    """LDGOperators<N,P>{M, G[N], T, A} (ldgpoisson.h:15-53)."""

    def __init__(self, ctx, handle, owned=True, keep=None):
        self.ctx, self.h, self.owned, self._keep = ctx, handle, owned, keep

    @classmethod
    def create(cls, ctx, M, G, T):
        h = C.c_void_p()
        arr = (C.c_void_p * len(G))(*[g.h for g in G])
        ctx.check(lib().mgldg_ops_create(ctx.h, len(G), M.h, arr, T.h, C.byref(h)), "ops_create")
        for m in [M, T] + list(G):
            m.release()
        return cls(ctx, h)

    @classmethod
    def create_A(cls, ctx, A):
        h = C.c_void_p()
        ctx.check(lib().mgldg_ops_create_A(ctx.h, A.h, C.byref(h)), "ops_create_A")
        A.release()
        return cls(ctx, h)

    def construct_laplacian(self):
        self.ctx.check(lib().mgldg_ops_construct_laplacian(self.ctx.h, self.h), "construct_laplacian")

    def construct_laplacian_kappa(self, kappa=None):
        """A = T + sum_d G_d^T diag(kappa_e M_e) G_d (kappa: one value per element, None = 1)."""
        k = None if kappa is None else np.ascontiguousarray(kappa, np.float64)
        ptr = None if k is None else k.ctypes.data_as(C.c_void_p)
        self.ctx.check(lib().mgldg_ops_construct_laplacian_kappa(self.ctx.h, self.h, ptr), "construct_laplacian_kappa")

    def get(self, which):
        out = C.c_void_p()
        self.ctx.check(lib().mgldg_ops_get(self.h, which, C.byref(out)), "ops_get")
        return SparseBlockMatrix(self.ctx, out, owned=False)

    @property
    def A(self):
        return self.get(4)

    def __del__(self):
        if getattr(self, "owned", False) and self.h:
            try:
                lib().mgldg_ops_destroy(self.h)
            except Exception:
                pass
            self.h = None


def mg_params(**kw):
    p = MGParams()
    lib().mgldg_mg_params_default(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


class Multigrid:
    """Multigrid<N,P>(ops, hierarchy, params) (multigrid.h:291-301)."""

    def __init__(self, ctx, ops, T, **params):
        self.ctx, self.ops = ctx, ops
        self.params = mg_params(**params)
        arr = (C.c_void_p * max(1, len(T)))(*[t.h for t in T])
        h = C.c_void_p()
        ctx.check(lib().mgldg_mg_create(ctx.h, ops.h, arr, len(T), C.byref(self.params), C.byref(h)), "mg_create")
        self.h = h
        n = C.c_int()
        ctx.check(lib().mgldg_mg_nlevels(h, C.byref(n)), "mg_nlevels")
        self.nlevels = n.value

    def level_op(self, level, which):
        out = C.c_void_p()
        self.ctx.check(lib().mgldg_mg_level_op(self.h, level, which, C.byref(out)), "level_op")
        return SparseBlockMatrix(self.ctx, out, owned=False)

    def vcycle(self, b, x=None):
        b = np.ascontiguousarray(b, np.float64)
        x = np.zeros_like(b) if x is None else np.array(x, dtype=np.float64)
        self.ctx.check(lib().mgldg_mg_vcycle(self.ctx.h, self.h, b, x), "vcycle")
        return x

    def relax(self, level, n, reverse, b, x):
        x = np.array(x, dtype=np.float64)
        self.ctx.check(lib().mgldg_mg_relax(self.ctx.h, self.h, level, n, int(reverse),
                                            np.ascontiguousarray(b, np.float64), x), "relax")
        return x

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().mgldg_mg_destroy(self.h)
            except Exception:
                pass
            self.h = None


def pcg(ctx, A, b, x=None, precon=None, tol=1e-8, maxit=200):
    """pcg(A, b, x, precon, tol, maxit) (krylov.h:22-68); returns (x, residual history)."""
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros_like(b) if x is None else np.array(x, dtype=np.float64)
    hist = np.zeros(max(1, maxit))
    it = C.c_int()
    rc = lib().mgldg_pcg(ctx.h, precon.h if precon is not None else None, A.h, b, x, tol, maxit, C.byref(it), hist)
    ctx.check(rc, "pcg")
    return x, hist[:it.value].copy()


def pcg_batched(ctx, A, B, X=None, precon=None, tol=1e-8, maxit=200):
    """pcg on the k columns of B (n x k) at once; returns (X, iterations[k], [history of column c])."""
    B = np.ascontiguousarray(B, np.float64)
    n, k = B.shape
    X = np.zeros_like(B) if X is None else np.array(X, dtype=np.float64, order="C")
    its = np.zeros(k, np.int32)
    hist = np.zeros(max(1, maxit) * k)
    rc = lib().mgldg_pcg_batched(ctx.h, precon.h if precon is not None else None, A.h, k, B, X, tol, maxit, its,
                                 hist)
    ctx.check(rc, "pcg_batched")
    hist = hist.reshape(k, max(1, maxit))
    return X, its, [hist[c, :its[c]].copy() for c in range(k)]


def batch_tiles(mg, level):
    """Autotuned column tiles of a level: (spmm, jacobi, restrict, prolong, outer)."""
    v = [C.c_int() for _ in range(5)]
    rc = lib().mgldg_mg_batch_tiles(mg.h, level, *[C.byref(x) for x in v])
    if rc:
        raise MgldgError(rc, "batch_tiles")
    return tuple(x.value for x in v)


def _device_vectors(*arrays):
    """float64 CUDA copies of host arrays (device memory comes from torch)."""
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a, np.float64)).to("cuda") for a in arrays]


def adjoint_l2(ctx, ops, b, u_obs, precon=None, tol=1e-10, maxit=200, u0=None):
    """L = 1/2 ||u - u_obs||^2 with A u = b (ops' Laplacian): forward and adjoint pcg
    with the same preconditioner, then dL/dkappa.  Returns
    (u, lambda = dL/db, dL/dkappa, L, (forward iterations, adjoint iterations))."""
    import torch
    b = np.ascontiguousarray(b, np.float64)
    n = len(b)
    ne = n // (ops.get(0).info()[2])
    db, dobs, du = _device_vectors(b, u_obs, np.zeros(n) if u0 is None else u0)
    dl = torch.zeros(n, dtype=torch.float64, device="cuda")
    dk = torch.zeros(max(1, ne), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    loss = C.c_double()
    its = (C.c_int * 2)()
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = lib().mgldg_adjoint_l2_dev(ctx.h, precon.h if precon is not None else None, ops.h, p(db), p(dobs), tol,
                                    maxit, p(du), p(dl), p(dk), C.byref(loss), its)
    ctx.check(rc, "adjoint_l2")
    ctx.sync()
    return (du.cpu().numpy(), dl.cpu().numpy(), dk.cpu().numpy()[:ne], loss.value, (its[0], its[1]))


def kappa_gradient(ctx, ops, u, lam):
    """dL/dkappa_e = -sum_d (G_d lam)_e^T M_e (G_d u)_e for host vectors u, lam."""
    import torch
    du, dl = _device_vectors(u, lam)
    ne = len(u) // (ops.get(0).info()[2])
    dk = torch.zeros(max(1, ne), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    p = lambda t: C.c_void_p(t.data_ptr())
    ctx.check(lib().mgldg_kappa_gradient_dev(ctx.h, ops.h, p(du), p(dl), p(dk)), "kappa_gradient")
    ctx.sync()
    return dk.cpu().numpy()[:ne]


def h_interp(ctx, n_fine, P):
    """One level of InterpolationHierarchy<2,P>: (n_fine/2)^2 -> n_fine^2 elements."""
    h = C.c_void_p()
    ctx.check(lib().mgldg_cartesian_h_interp(ctx.h, n_fine, P, C.byref(h)), "h_interp")
    return SparseBlockMatrix(ctx, h)


def p_interp(ctx, ne, P_fine, P_coarse):
    """InterpolationHierarchy<2,Pf,Pc>: degree Pc -> Pf on the same ne elements."""
    h = C.c_void_p()
    ctx.check(lib().mgldg_cartesian_p_interp(ctx.h, ne, P_fine, P_coarse, C.byref(h)), "p_interp")
    return SparseBlockMatrix(ctx, h)


def hp_chain(ctx, n, degrees, nh):
    """Transfers of Multigrid<2,P1,P2,...>: p-levels over `degrees`, then nh h-levels."""
    T = [p_interp(ctx, n * n, degrees[k - 1], degrees[k]) for k in range(1, len(degrees))]
    nf = n
    for _ in range(nh):
        T.append(h_interp(ctx, nf, degrees[-1]))
        nf //= 2
    return T


COARSEN_EQUAL, COARSEN_RAPID = 0, 1
H_FN = C.CFUNCTYPE(C.c_double, C.POINTER(C.c_double), C.c_void_p)


class PointsRule(C.Structure):
    _fields_ = [("npoints", C.c_int), ("points", C.POINTER(C.c_double)), ("base_level", C.c_int),
                ("extra_levels", C.c_int), ("radius", C.c_double)]


def seeded_points(seed, n):
    """n points in [0,1)^2 from mt19937_64 (53-bit uniforms, x/y pairs)."""
    xy = np.zeros(2 * n)
    rc = lib().mgldg_seeded_points(seed, n, xy)
    if rc:
        raise MgldgError(rc, "seeded_points")
    return xy.reshape(n, 2)


class Quadtree:
    """Quadtree<2>(h) on [0,1]^2 (host): h is a Python callable h(x, y) -> width,
    or use Quadtree.points(...) for the built-in seeded-points rule."""

    def __init__(self, h=None, balance=False, strategy=COARSEN_EQUAL, _native=None):
        out = C.c_void_p()
        if _native is not None:
            fn, user = _native
        else:
            self._cb = H_FN(lambda x, _u: float(h(x[0], x[1])))
            fn, user = C.cast(self._cb, C.c_void_p), None
        rc = lib().mgldg_quadtree_create(fn, user, int(balance), strategy, C.byref(out))
        if rc:
            raise MgldgError(rc, "quadtree_create")
        self.h = out
        a, b_, c = C.c_int(), C.c_int(), C.c_int()
        lib().mgldg_quadtree_info(out, C.byref(a), C.byref(b_), C.byref(c))
        self.nnodes, self.nlevels, self.nleaves = a.value, b_.value, c.value

    @classmethod
    def points(cls, points, base_level, extra_levels, radius=0.5, balance=True, strategy=COARSEN_EQUAL):
        pts = np.ascontiguousarray(points, np.float64).ravel()
        rule = PointsRule(len(pts) // 2, pts.ctypes.data_as(C.POINTER(C.c_double)), base_level, extra_levels, radius)
        fn = C.cast(lib().mgldg_h_points, C.c_void_p)
        self = cls(balance=balance, strategy=strategy, _native=(fn, C.cast(C.pointer(rule), C.c_void_p)))
        return self

    def layer(self, l):
        n = C.c_int()
        rc = lib().mgldg_quadtree_layer(self.h, l, C.byref(n), None, None, None)
        if rc:
            raise MgldgError(rc, "quadtree_layer")
        lev, ix, iy = (np.zeros(n.value, np.int32) for _ in range(3))
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        lib().mgldg_quadtree_layer(self.h, l, C.byref(n), p(lev), p(ix), p(iy))
        return lev, ix, iy

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().mgldg_quadtree_destroy(self.h)
            except Exception:
                pass
            self.h = None


def _two_call(fn, *head, N=2):
    np_, nt = C.c_int(), C.c_int()
    rc = fn(*head, C.byref(np_), C.byref(nt), None, None)
    if rc:
        raise MgldgError(rc, "mesh")
    p = np.zeros((np_.value, N))
    t = np.zeros((nt.value, N + 1), np.int32)
    rc = fn(*head, C.byref(np_), C.byref(nt), p.ctypes.data_as(C.c_void_p), t.ctypes.data_as(C.c_void_p))
    if rc:
        raise MgldgError(rc, "mesh")
    return p, t


def disk_mesh(h):
    """Triangles of the unit disk with spacing about h: (points[np,2], triangles[nt,3])."""
    return _two_call(lib().mgldg_disk_mesh, C.c_double(h))


def morton_order(p, t):
    """Elements of (p, t) reordered stably by the Morton key of their
    centroids (the block Gauss-Seidel order; see mgldg_mesh_morton_order)."""
    p = np.ascontiguousarray(p, np.float64)
    t = np.array(t, dtype=np.int32, order="C")
    N = p.shape[1]
    rc = lib().mgldg_mesh_morton_order(N, len(p), p.ctypes.data_as(C.c_void_p), len(t), t.ctypes.data_as(C.c_void_p))
    if rc:
        raise MgldgError(rc, "mesh_morton_order")
    return t


def ball_mesh(h):
    """Tetrahedra of the unit ball (Kuhn-split cube grid mapped onto the ball): (points[np,3], tets[nt,4])."""
    return _two_call(lib().mgldg_ball_mesh, C.c_double(h), N=3)


def read_mesh(path, N=2):
    """The reference's .mesh wireframe (Wireframe<N>): (points[np,N], simplices[nt,N+1], 0-based)."""
    if N == 2:
        return _two_call(lib().mgldg_mesh_read, str(path).encode())
    return _two_call(lib().mgldg_mesh_read_nd, str(path).encode(), N, N=N)


def mesh_union(meshes):
    """Disjoint union of simplex meshes: (points, simplices, element offsets[len+1])."""
    ps, ts, off, nv, ne = [], [], [0], 0, 0
    for p, t in meshes:
        ps.append(np.asarray(p, np.float64))
        ts.append(np.asarray(t, np.int32) + nv)
        nv += len(p)
        ne += len(t)
        off.append(ne)
    return np.concatenate(ps), np.concatenate(ts), np.array(off, np.int64)


def pcg_segmented(ctx, A, b, seg_offsets, precon, x=None, tol=1e-8, maxit=200):
    """pcg on independent segments of a block-diagonal system (host vectors):
    (x, iterations[nseg], [history of segment s])."""
    import torch
    b = np.ascontiguousarray(b, np.float64)
    off = np.ascontiguousarray(seg_offsets, np.int64)
    nseg = len(off) - 1
    db = torch.from_numpy(b).to("cuda")
    dx = torch.from_numpy(np.zeros_like(b) if x is None else np.array(x, np.float64)).to("cuda")
    torch.cuda.synchronize()
    its = np.zeros(nseg, np.int32)
    hist = np.zeros(max(1, maxit) * nseg)
    rc = lib().mgldg_pcg_segmented_dev(ctx.h, precon.h, A.h, nseg, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                       C.c_void_p(db.data_ptr()), C.c_void_p(dx.data_ptr()), tol, maxit, its, hist)
    ctx.check(rc, "pcg_segmented")
    ctx.sync()
    hist = hist.reshape(nseg, max(1, maxit))
    return dx.cpu().numpy(), its, [hist[s, :its[s]].copy() for s in range(nseg)]


def simplex_master(N, P):
    b = {1: P, 2: P * (P + 1) // 2, 3: P * (P + 1) * (P + 2) // 6}[N]
    mass, diff, nodes = np.zeros(b * b), np.zeros(N * b * b), np.zeros(b * N)
    rc = lib().mgldg_simplex_master_nd(N, P, mass, diff, nodes)
    if rc:
        raise MgldgError(rc, "simplex_master")
    return mass.reshape(b, b), list(diff.reshape(N, b, b)), nodes.reshape(b, N)


class CartesianProblem:
    """Uniform n x n quadtree mesh, Q_{P-1} LDG operators and hierarchy, built on the GPU
    (or, with quadtree=..., the leaves of an adaptive Quadtree)."""

    def __init__(self, ctx, P, n=None, tau0=None, tauD=None, quadtree=None, tau_per_face=False, mesh=None,
                 agg_levels=8, agg_seed=4000):
        h = C.c_void_p()
        if mesh is not None:
            pts, tris = mesh
            N = np.asarray(pts).shape[1]
            pts = np.ascontiguousarray(pts, np.float64).ravel()
            tris = np.ascontiguousarray(tris, np.int32).ravel()
            ctx.check(lib().mgldg_simplex_problem_create_nd(ctx.h, N, len(pts) // N, pts, len(tris) // (N + 1), tris,
                                                            P, float(tau0), float(tauD), agg_levels, agg_seed,
                                                            C.byref(h)), "simplex_problem_create")
        elif quadtree is None:
            tau0 = float(n) if tau0 is None else tau0
            tauD = float(n) if tauD is None else tauD
            ctx.check(lib().mgldg_cartesian_create(ctx.h, P, n, tau0, tauD, C.byref(h)), "cartesian_create")
        else:
            tau0 = 1.0 if tau0 is None else tau0
            tauD = 1.0 if tauD is None else tauD
            ctx.check(lib().mgldg_quadtree_problem_create(ctx.h, quadtree.h, P, tau0, tauD, int(tau_per_face),
                                                          C.byref(h)), "quadtree_problem_create")
        self.ctx, self.h = ctx, h
        nf, nb, nl = C.c_int(), C.c_int(), C.c_int()
        lib().mgldg_problem_mesh_info(h, C.byref(nf), C.byref(nb), C.byref(nl))
        self.nfaces, self.nbfaces, self.nlevels = nf.value, nb.value, nl.value
        ne, npl, nT = C.c_int(), C.c_int(), C.c_int()
        ndof = C.c_int64()
        ctx.check(lib().mgldg_problem_info(h, C.byref(ne), C.byref(npl), C.byref(ndof), C.byref(nT)), "info")
        self.ne, self.npl, self.ndof, self.nT = ne.value, npl.value, ndof.value, nT.value
        o = C.c_void_p()
        ctx.check(lib().mgldg_problem_ops(h, C.byref(o)), "problem_ops")
        self.ops = LDGOperators(ctx, o, owned=False, keep=self)
        self.T = []
        for l in range(self.nT):
            t = C.c_void_p()
            ctx.check(lib().mgldg_problem_interp(h, l, C.byref(t)), "problem_interp")
            self.T.append(SparseBlockMatrix(ctx, t, owned=False))

    def partition(self, l):
        n = C.c_int()
        self.ctx.check(lib().mgldg_problem_partition(self.h, l, C.byref(n), None), "partition")
        a = np.zeros(n.value, np.int32)
        self.ctx.check(lib().mgldg_problem_partition(self.h, l, C.byref(n), a.ctypes.data_as(C.c_void_p)),
                       "partition")
        return a

    def write_fun(self, u, path):
        """Nodal dump of u (the reference's Function::write format)."""
        self.ctx.check(lib().mgldg_problem_write_fun(self.ctx.h, self.h, np.ascontiguousarray(u, np.float64),
                                                     str(path).encode()), "write_fun")

    def rhs_gaussian(self, seed):
        b = np.zeros(self.ndof)
        self.ctx.check(lib().mgldg_problem_rhs_gaussian(self.ctx.h, self.h, seed, b), "rhs_gaussian")
        return b

    def __del__(self):
        if getattr(self, "h", None):
            try:
                lib().mgldg_problem_destroy(self.h)
            except Exception:
                pass
            self.h = None

/*
 * mgldg.h -- C ABI of the GB300 (sm_103a) multigrid-preconditioned CG solver
 * for LDG Poisson operators in block-sparse form.
 *
 * Drop-in for the solver path of danfortunato/multigrid-ldg.  The reference
 * exposes that path as C++ templates; each entry point below names the
 * reference interface it replaces (paths are relative to the reference tree).
 *
 *   SparseBlockMatrix<P,Q>      src/cartesian/util/sparseblockmatrix.h:62-165
 *   multiply_*_mv*              src/cartesian/util/sparseblockmatrix.tpp:288-422
 *   LDGOperators<N,P>           src/cartesian/dg/ldgpoisson.h:15-53
 *   MG::Parameters              src/cartesian/multigrid/multigrid.h:48-62
 *   Multigrid<N,P>              src/cartesian/multigrid/multigrid.h:280-433
 *   pcg                         src/cartesian/multigrid/krylov.h:22-82
 *
 * Conventions
 *  - Every call returns an int status (MGLDG_OK == 0).  The text of the last
 *    error of a context is returned by mgldg_last_error().  No C++ exception
 *    crosses this boundary.
 *  - Blocks are dense row-major br x bc doubles; vectors are element-major
 *    (dof = element * block_size + local node), the reference's layout.
 *  - Arguments without a _dev suffix are host pointers; they are copied.
 *    Functions with a _dev suffix take device pointers on the context's GPU
 *    and run asynchronously on the context's stream.
 *  - Handles own their device memory and free it in *_destroy.  A handle is
 *    used by one host thread at a time; each context owns one CUDA stream.
 */
#ifndef MGLDG_H
#define MGLDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the reference's bool shape returns,
 *      std::invalid_argument and asserts, mapped to codes) ---- */
#define MGLDG_OK              0
#define MGLDG_ERR_ARG         1  /* bad argument / unknown enum (multigrid.h:164,194,214) */
#define MGLDG_ERR_SHAPE       2  /* block shapes do not conform (sparseblockmatrix.tpp:181-184) */
#define MGLDG_ERR_CUDA        3  /* CUDA runtime failure */
#define MGLDG_ERR_BREAKDOWN   4  /* PCG breakdown: d.q <= 0, r.z < 0 or a non-finite scalar */
#define MGLDG_ERR_TIMEOUT     5  /* a bounded device-side wait ran out */
#define MGLDG_ERR_NOT_SPD     6  /* a block or the coarse matrix is singular / not SPD */
#define MGLDG_ERR_NOMEM       7  /* device allocation failed */
#define MGLDG_ERR_UNSUPPORTED 8  /* valid request this build does not implement */

typedef struct mgldg_ctx mgldg_ctx;
typedef struct mgldg_bsr mgldg_bsr;
typedef struct mgldg_ops mgldg_ops;
typedef struct mgldg_mg mgldg_mg;
typedef struct mgldg_problem mgldg_problem;

/* ------------------------------------------------------------ context -- */
/* Creates a context on CUDA device `device` with its own stream. */
int mgldg_ctx_create(int device, mgldg_ctx** ctx);
int mgldg_ctx_destroy(mgldg_ctx* ctx);
/* Text of the last error reported through this context ("" if none). */
const char* mgldg_last_error(const mgldg_ctx* ctx);
/* Waits for all work queued on the context's stream. */
int mgldg_ctx_sync(mgldg_ctx* ctx);
/* The context's stream (a cudaStream_t), for callers that pass _dev data. */
void* mgldg_ctx_stream(mgldg_ctx* ctx);
/* Reference-element tables (master.h:147-214): P = nodes per dimension,
 * 1..6.  nodes[P], denom[P], mass/invmass/diff[P*P]; quad_x/quad_w[10]. */
int mgldg_master_tables(int P, double* nodes, double* denom, double* mass,
                        double* invmass, double* diff, double* quad_x, double* quad_w);

/* ------------------------------------------- block-sparse matrix (BSR) -- */
/* Replaces SparseBlockMatrix<P,Q> assembly (setBlock/addToBlock,
 * sparseblockmatrix.h:113-125) by a block-CSR upload: nbr x nbc blocks of
 * br x bc; row_ptr[nbr+1], col_idx[nnzb] (any order within a row; stored
 * sorted), vals[nnzb*br*bc].  Duplicate (i,j) entries are summed, as
 * addToBlock does. */
int mgldg_bsr_create(mgldg_ctx* ctx, int nbr, int nbc, int br, int bc,
                     const int* row_ptr, const int* col_idx, const double* vals,
                     mgldg_bsr** A);
int mgldg_bsr_destroy(mgldg_bsr* A);
/* Incremental host-side assembly with the reference's block calls, for
 * callers that build a matrix block by block: create = reset(m, n)
 * (sparseblockmatrix.tpp:120-127), set = setBlock (:79-84, overwrites),
 * add = addToBlock (:93-100, sums in call order), exists = blockExists,
 * nnzb.  export writes the sorted block-CSR (pass NULL arrays to skip);
 * finalize uploads it as a device BSR. */
typedef struct mgldg_bsr_builder mgldg_bsr_builder;
int mgldg_bsr_builder_create(int nbr, int nbc, int br, int bc, mgldg_bsr_builder** out);
int mgldg_bsr_builder_set(mgldg_bsr_builder* b, int i, int j, const double* block);
int mgldg_bsr_builder_add(mgldg_bsr_builder* b, int i, int j, const double* block);
int mgldg_bsr_builder_exists(const mgldg_bsr_builder* b, int i, int j, int* exists);
int mgldg_bsr_builder_nnzb(const mgldg_bsr_builder* b, int64_t* nnzb);
int mgldg_bsr_builder_export(const mgldg_bsr_builder* b, int* row_ptr, int* col_idx, double* vals);
int mgldg_bsr_builder_finalize(mgldg_ctx* ctx, const mgldg_bsr_builder* b, mgldg_bsr** A);
int mgldg_bsr_builder_destroy(mgldg_bsr_builder* b);
/* A device-side copy of A (pattern and values), owned by the caller. */
int mgldg_bsr_clone(mgldg_ctx* ctx, const mgldg_bsr* A, mgldg_bsr** out);
/* blockRows/blockCols/rowsPerBlock/colsPerBlock/nnzb (sparseblockmatrix.h:82-110) */
int mgldg_bsr_info(const mgldg_bsr* A, int* nbr, int* nbc, int* br, int* bc,
                   int64_t* nnzb);
/* Sorted block-CSR download (the stored pattern and values). */
int mgldg_bsr_download(mgldg_ctx* ctx, const mgldg_bsr* A, int* row_ptr,
                       int* col_idx, double* vals);
/* y := alpha*A*x + beta*y  (multiply_add_mv / multiply_mv,
 * sparseblockmatrix.tpp:288-301,358-371).  Host vectors. */
int mgldg_bsr_mv(mgldg_ctx* ctx, double alpha, const mgldg_bsr* A,
                 const double* x, double beta, double* y);
int mgldg_bsr_mv_dev(mgldg_ctx* ctx, double alpha, const mgldg_bsr* A,
                     const double* x, double beta, double* y);
/* y := A^T x  (multiply_mv_t, sparseblockmatrix.tpp:322-335).  Host vectors. */
int mgldg_bsr_mv_t(mgldg_ctx* ctx, const mgldg_bsr* A, const double* x, double* y);

/* ------------------------------------------------------ LDG operators -- */
/* LDGOperators<N,P>{M, Minv, G[N], T, A} (ldgpoisson.h:15-31).  Takes
 * ownership of M, G[0..ndim-1] and T (they are destroyed with ops). */
int mgldg_ops_create(mgldg_ctx* ctx, int ndim, mgldg_bsr* M, mgldg_bsr* const* G,
                     mgldg_bsr* T, mgldg_ops** ops);
/* Operators holding only the Laplacian A (enough for RAT coarsening, for
 * pcg and for Jacobi / Gauss-Seidel).  Takes ownership of A. */
int mgldg_ops_create_A(mgldg_ctx* ctx, mgldg_bsr* A, mgldg_ops** ops);
/* A = T + sum_d G_d^T M G_d  (construct_laplacian, ldgpoisson.h:34-52),
 * symbolic product on the host, numeric product on the GPU. */
int mgldg_ops_construct_laplacian(mgldg_ctx* ctx, mgldg_ops* ops);
/* which: 0=M 1=G0 2=G1 3=T 4=A 5=G2 (three-dimensional meshes).  The handle
 * stays owned by ops. */
int mgldg_ops_get(const mgldg_ops* ops, int which, const mgldg_bsr** A);
int mgldg_ops_destroy(mgldg_ops* ops);

/* ---------------------------------------------------------- multigrid -- */
#define MGLDG_RELAX_JACOBI       0   /* MG::kJacobi */
#define MGLDG_RELAX_GAUSS_SEIDEL 1   /* MG::kGaussSeidel */
#define MGLDG_COARSE_CHOLESKY    0   /* MG::kCholesky: one-element coarsest level */
#define MGLDG_COARSE_RELAXATION  1   /* MG::kRelaxation */
#define MGLDG_COARSE_DENSE       2   /* extension: dense FP64 inverse (Gauss-Jordan) of a
                                        multi-element coarsest level, applied as a matvec */
#define MGLDG_RESTRICT_RAT       0   /* MG::kRAT */
#define MGLDG_RESTRICT_RATRAT    1   /* MG::kRATRAT */
#define MGLDG_PREC_FP64          0   /* plain form: FP64 throughout */
#define MGLDG_PREC_MIXED         1   /* FP32 V-cycle, FP64 coarsest solve and FP64 pcg
                                        vectors and scalars; pcg's q = A d (square blocks
                                        3..10 and 16) in double-float arithmetic on the
                                        FP32 pipes, about 2^-44 relative */
#define MGLDG_PREC_MIXED_F16     2   /* MIXED, with the level operators' Jacobi sweeps and
                                        residuals reading a block-scaled FP16 copy (one FP32
                                        scale per block) where the blocks are 16 x 16; other
                                        block sizes run as in MIXED */
#define MGLDG_PREC_MIXED_TF32    3   /* MIXED, with the multi-RHS V-cycle's level-operator
                                        products (square blocks 4..16) on the tensor cores:
                                        TF32 operands split in high and low parts (3xTF32),
                                        FP32 accumulation; single-RHS solves run as MIXED */

/* MG::Parameters (multigrid.h:48-62) plus the build's extensions. */
typedef struct mgldg_mg_params {
    int relaxation;     /* default MGLDG_RELAX_GAUSS_SEIDEL */
    double omega;       /* default 0.8 */
    int solver;         /* default MGLDG_COARSE_CHOLESKY */
    int npre;           /* default 3 */
    int npost;          /* default 3 */
    int restriction;    /* default MGLDG_RESTRICT_RATRAT */
    int precision;      /* default MGLDG_PREC_FP64 */
    int max_levels;     /* 0: the whole hierarchy (reference); k: keep k levels */
    int mean_project;   /* 1 (reference, multigrid.h:367): b -= mean(b) on the coarsest level */
} mgldg_mg_params;

void mgldg_mg_params_default(mgldg_mg_params* p);
/* Multigrid<N,P>(ops, hierarchy, params) (multigrid.h:291-301, setup
 * :404-411, Level constructors :83-171).  T[l] interpolates level l+1 to
 * level l (InterpolationHierarchy<N,P>::T, interpolationhierarchy.h:91);
 * its values are copied.  `fine` is borrowed and must outlive mg. */
int mgldg_mg_create(mgldg_ctx* ctx, const mgldg_ops* fine, const mgldg_bsr* const* T,
                    int nT, const mgldg_mg_params* params, mgldg_mg** mg);
int mgldg_mg_destroy(mgldg_mg* mg);
int mgldg_mg_nlevels(const mgldg_mg* mg, int* nlevels);
/* Operators of level l (level(i)->ops, multigrid.h:352-355); which as in
 * mgldg_ops_get.  Owned by mg. */
int mgldg_mg_level_op(const mgldg_mg* mg, int level, int which, const mgldg_bsr** A);
/* One V-cycle from level 0 (vcycle(), multigrid.h:361-383) on rhs b with
 * initial guess / result x (solution(), rhs()). */
int mgldg_mg_vcycle(mgldg_ctx* ctx, mgldg_mg* mg, const double* b, double* x);
int mgldg_mg_vcycle_dev(mgldg_ctx* ctx, mgldg_mg* mg, const double* b, double* x);
/* n relaxations on `level` (relax(n, reverse), multigrid.h:202-216). */
int mgldg_mg_relax(mgldg_ctx* ctx, mgldg_mg* mg, int level, int n, int reverse,
                   const double* b, double* x);

/* ---------------------------------------------------------------- pcg -- */
/* pcg(A, b, x, precon, tol, maxit) (krylov.h:22-68) with precon = one
 * V-cycle from x = 0 (dg_tests.cpp:300-305); mg == NULL gives the
 * unpreconditioned overload (krylov.h:78-82).  x is the initial guess and
 * the result.  iters (may be NULL) receives the iteration count; res_hist
 * (may be NULL, maxit doubles) receives ||r|| after each iteration, the
 * value the reference prints.  Returns MGLDG_OK also when maxit is reached. */
int mgldg_pcg(mgldg_ctx* ctx, mgldg_mg* mg, const mgldg_bsr* A, const double* b,
              double* x, double tol, int maxit, int* iters, double* res_hist);
int mgldg_pcg_dev(mgldg_ctx* ctx, mgldg_mg* mg, const mgldg_bsr* A, const double* b,
                  double* x, double tol, int maxit, int* iters, double* res_hist);

/* No counterpart in the reference.  The unpreconditioned CG of
 * mgldg_pcg_dev(ctx, NULL, ...) for callers that cannot allocate device
 * memory while they solve (a host framework whose caching allocator owns the
 * GPU's memory, or a caller held to a memory budget fixed at start-up).  It
 * calls no cudaMalloc/cudaFree or other allocating routine: its work vectors
 * live in one fixed device array of about 4.1 MiB that every GPU loading the
 * library holds until the process exits.  Limits: at most 131,072 unknowns
 * and maxit <= 1024 (larger requests return MGLDG_ERR_ARG).  b and x are
 * device pointers owned by the caller.  The first call on each device looks
 * up the array's device address, so make it before any stream capture; the
 * address belongs to the device's primary context, so do not call this entry
 * point again after resetting the device (cudaDeviceReset).  All
 * calls on a device share the array: calls that overlap on the GPU (other
 * streams, threads or contexts) race and must be serialised by the caller.
 * Non-finite b or x: MGLDG_ERR_BREAKDOWN with 0 iterations, as mgldg_pcg_dev. */
int mgldg_cg_noalloc_dev(mgldg_ctx* ctx, const mgldg_bsr* A, const double* b,
                         double* x, double tol, int maxit, int* iters, double* res_hist);

/* ------------------------------------- Cartesian problem builder ---------
 * The callers on either side of the path, for users without the reference's
 * assembly: a uniform quadtree mesh of n x n squares on [0,1]^2 (n a power
 * of two), elements in the reference's depth-first order, Q_{P-1} nodal LDG
 * with homogeneous Dirichlet data (LDGPoisson<2,P>, ldgpoisson.tpp:14-161,
 * assembled on the GPU) and its h-interpolation hierarchy
 * (interpolationhierarchy.h:30-82). */
int mgldg_cartesian_create(mgldg_ctx* ctx, int P, int n, double tau0, double tauD,
                           mgldg_problem** pr);
int mgldg_problem_destroy(mgldg_problem* pr);
int mgldg_problem_info(const mgldg_problem* pr, int* ne, int* npl, int64_t* ndof, int* nT);
/* Borrowed handles, owned by pr. */
int mgldg_problem_ops(mgldg_problem* pr, mgldg_ops** ops);
int mgldg_problem_interp(mgldg_problem* pr, int l, const mgldg_bsr** T);
/* b = M f with f the nodal interpolant of a sum of 8 Gaussians drawn from
 * `seed` (centres U[0,1]^2, widths U[0.05,0.2], amplitudes N(0,1)).
 * _dev writes a device vector. */
int mgldg_problem_rhs_gaussian(mgldg_ctx* ctx, mgldg_problem* pr, uint64_t seed, double* b);
/* Transfers for h-, p- and hp-multigrid on uniform meshes; the caller owns
 * the handle (mgldg_mg_create copies it).  h: one level of
 * InterpolationHierarchy<2,P> from the (n_fine/2)^2 to the n_fine^2 mesh
 * (interpolationhierarchy.h:30-82).  p: InterpolationHierarchy<2,Pf,Pc> on
 * ne elements, the block-diagonal evaluation of the degree-Pc basis at the
 * Pf nodes (interpolationhierarchy.h:99-129).  Passing a chain
 * [p transfers..., h levels at the last degree...] to mgldg_mg_create gives
 * the reference's Multigrid<N,P1,P2,...> (multigrid.h:436-560). */
int mgldg_cartesian_h_interp(mgldg_ctx* ctx, int n_fine, int P, mgldg_bsr** T);
int mgldg_cartesian_p_interp(mgldg_ctx* ctx, int ne, int P_fine, int P_coarse, mgldg_bsr** T);
int mgldg_problem_rhs_gaussian_dev(mgldg_ctx* ctx, mgldg_problem* pr, uint64_t seed, double* b);

/* ------------------------------------------------- adaptive quadtrees -- */
/* Quadtree<2>(h) on [0,1]^2 (quadtree.tpp:10-40): a cell is split while its
 * width exceeds h(centre).  balance != 0 adds 2:1 face balancing (no
 * reference counterpart: a leaf is split while a face neighbour is two or
 * more levels finer).  strategy: the coarsening of QuadTree::isLeaf
 * (quadtree.h:164-173).  Host only, no GPU needed. */
#define MGLDG_COARSEN_EQUAL 0
#define MGLDG_COARSEN_RAPID 1
typedef struct mgldg_quadtree mgldg_quadtree;
typedef double (*mgldg_h_fn)(const double* x, void* user);
int mgldg_quadtree_create(mgldg_h_fn h, void* user, int balance, int strategy, mgldg_quadtree** qt);
int mgldg_quadtree_destroy(mgldg_quadtree* qt);
int mgldg_quadtree_info(const mgldg_quadtree* qt, int* nnodes, int* nlevels, int* nleaves);
/* Cells of layer l (QuadTree::layer, quadtree.h:176-186) in depth-first
 * order as (level, ix, iy), cell = [ix, ix+1] x [iy, iy+1] * 2^-level.  With
 * level, ix and iy all NULL only *n is returned. */
int mgldg_quadtree_layer(const mgldg_quadtree* qt, int l, int* n, int* level, int* ix, int* iy);
/* Built-in mesh-size rule (no reference counterpart; the adaptive mesh of
 * the multi-RHS workload): a cell of width 2^-(base_level + l) is split while
 * l < extra_levels and its centre lies within radius * 2^-l of one of the
 * points, i.e. h(x) = min(2^-base, max(2^-(base+extra), d(x) / (radius 2^base)))
 * with d the distance to the nearest point.  Pass mgldg_h_points with a
 * mgldg_points_rule* as user. */
typedef struct {
    int npoints;
    const double* points;   /* x0 y0 x1 y1 ... */
    int base_level;
    int extra_levels;
    double radius;
} mgldg_points_rule;
double mgldg_h_points(const double* x, void* user);
/* n seeded points in [0,1)^2: mt19937_64, 53-bit uniforms, (x, y) pairs. */
int mgldg_seeded_points(uint64_t seed, int n, double* xy);
/* LDG problem on the leaves of qt (Mesh(qt), mesh.h:186-264;
 * LDGPoisson::discretize, ldgpoisson.tpp:27-100), homogeneous Dirichlet,
 * with its h-interpolation hierarchy over the tree's layers
 * (interpolationhierarchy.h:30-82).  tau_per_face != 0 (extension): interior
 * penalty tau0 / min(h_L, h_R) and boundary penalty tauD / h_L instead of
 * the constants tau0 and tauD. */
int mgldg_quadtree_problem_create(mgldg_ctx* ctx, const mgldg_quadtree* qt, int P, double tau0,
                                  double tauD, int tau_per_face, mgldg_problem** out);
/* Faces, boundary faces and quadtree levels of a problem's mesh. */
int mgldg_problem_mesh_info(const mgldg_problem* pr, int* nfaces, int* nbfaces, int* nlevels);

/* ---------------------------------------------- unstructured triangles -- */
/* Mesh input.  mgldg_mesh_read reads the reference's .mesh wireframe
 * (Wireframe(file), wireframe.h:24-67): "np nt", a header line, np lines of
 * x y, an empty line, nt lines of 1-based vertex triples; p[2*np], t[3*nt]
 * 0-based (pass p = t = NULL to get the counts first).  mgldg_disk_mesh (no
 * reference counterpart; the reference reads distmesh output) meshes the
 * unit disk with concentric rings of spacing 1/ceil(1/h), triangles in the
 * Morton order below, same calling pattern. */
int mgldg_mesh_read(const char* path, int* np, int* nt, double* p, int* t);
/* The same for Wireframe<N>, N = 2 (triangles) or 3 (tetrahedra: lines of
 * x y z, then 1-based vertex quadruples); p[N*np], t[(N+1)*nt]. */
int mgldg_mesh_read_nd(const char* path, int N, int* np, int* nt, double* p, int* t);
int mgldg_disk_mesh(double h, int* np, int* nt, double* p, int* t);
/* Reorders the N-simplices t[(N+1)*nt] in place, stably, by the Morton key
 * of their centroids (no reference counterpart).  Element order is block
 * Gauss-Seidel's order: an order whose dependency chain is as long as the
 * mesh (a ring around a disk, with the LDG operator's two-element reach)
 * serialises the sweep; a space-filling order keeps the chain short. */
int mgldg_mesh_morton_order(int N, int np, const double* p, int nt, int* t);
/* P_{P-1} LDG on a triangle mesh (Mesh(wireframe), mesh.h:187-300;
 * LDGPoisson::discretize, ldgpoisson.tpp:27-100), homogeneous Dirichlet on
 * every boundary edge, P in 1..4 (b = P(P+1)/2 unknowns per element), with
 * an agglomeration hierarchy of up to agg_levels levels
 * (InterpolationHierarchy(agglomeration), interpolationhierarchy.h:89-210:
 * tensor-product Q_{P-1} spaces on the aggregates' bounding boxes, so the
 * first transfer has b x P^2 blocks).  The aggregates come from a greedy
 * seeded agglomeration of at most four elements (plus merged singletons)
 * in place of MGridGen.  mgldg_problem_rhs_gaussian(_dev) on such a problem
 * draws the Gaussian centres uniformly on the unit disk; seed 0 gives f = 1. */
int mgldg_simplex_problem_create(mgldg_ctx* ctx, int np, const double* p, int nt, const int* t, int P,
                                 double tau0, double tauD, int agg_levels, uint64_t agg_seed,
                                 mgldg_problem** out);
/* The same for N = 2 (triangles, p[2*np], t[3*nt]) or N = 3 (tetrahedra,
 * p[3*np], t[4*nt], P in 1..3, b = P(P+1)(P+2)/6; coarse spaces Q_{P-1}
 * on aggregate boxes, P^3 per aggregate, aggregates grown breadth-first to
 * eight tetrahedra, at least six).  The right-hand side's Gaussian centres
 * are uniform in the unit ball.  Boundary faces use a 10 x 10 collapsed
 * Gauss rule on the master triangle with weights summing to 1, scaled by the
 * face area. */
int mgldg_simplex_problem_create_nd(mgldg_ctx* ctx, int N, int np, const double* p, int nt,
                                    const int* t, int P, double tau0, double tauD, int agg_levels,
                                    uint64_t agg_seed, mgldg_problem** out);
/* Tetrahedra of the unit ball (no reference counterpart), a cubed sphere:
 * a core cube [-0.45,0.45]^3 of hexahedra about 2h across and radial layers
 * of hexahedra over its faces out to the sphere, each hexahedron cut into 24
 * tetrahedra through its face and cell centres (no tetrahedron with four
 * vertices on the sphere), tetrahedra in Morton order; p[3*np], t[4*nt];
 * NULL arrays return the counts. */
int mgldg_ball_mesh(double h, int* np, int* nt, double* p, int* t);
/* Aggregate of every element of agglomeration level l's finer mesh (agg may
 * be NULL to get the count). */
int mgldg_problem_partition(const mgldg_problem* pr, int l, int* n, int* agg);
/* Master simplex (N = 1 or 2): mass, differentiation matrices (row-major
 * b x b) and nodes (b x N) in the reference's node order. */
int mgldg_simplex_master(int N, int P, double* mass, double* diff0, double* diff1, double* nodes);
/* N = 1..3: diff receives the N differentiation matrices one after the other. */
int mgldg_simplex_master_nd(int N, int P, double* mass, double* diff, double* nodes);

/* ---------------------------------------------------------- file formats -- */
/* Matrix Market dump of a BSR matrix, the format of the reference's
 * SparseBlockMatrix::write (sparseblockmatrix.tpp:145-164): coordinate real
 * general, 1-based, every entry of every stored block, 17 significant
 * digits (blocks in sorted order). */
int mgldg_bsr_write_mtx(mgldg_ctx* ctx, const mgldg_bsr* A, const char* path);
/* Reads such a file (e.g. the reference's data/A.mtx) into a BSR matrix with
 * br x bc blocks; entries of one block position are summed. */
int mgldg_bsr_read_mtx(mgldg_ctx* ctx, const char* path, int br, int bc, mgldg_bsr** A);
/* Nodal dump of a host vector u on a Cartesian problem, the reference's
 * Function::write format (function.h:173-190): "P N ne", then per element
 * one "x y value" line per node and an empty line. */
int mgldg_problem_write_fun(mgldg_ctx* ctx, const mgldg_problem* pr, const double* u, const char* path);

/* ------------------------------------------- many right-hand sides -- */
/* No counterpart in the reference (it solves one right-hand side at a time
 * with pcg, krylov.h:22-68).  A multi-vector of k columns (1 <= k <= 1024)
 * over n unknowns is row-major: X[u*k + c].
 *
 * Y := alpha*A*X + beta*Y on device multi-vectors (multiply_add_mv,
 * sparseblockmatrix.tpp:358-371, applied to k vectors at once). */
int mgldg_bsr_mm_dev(mgldg_ctx* ctx, double alpha, const mgldg_bsr* A, int k,
                     const double* X, double beta, double* Y);
/* One V-cycle per column (vcycle, multigrid.h:361-383) with X as the initial
 * guess (in/out).  Needs params.relaxation == MGLDG_RELAX_JACOBI. */
int mgldg_mg_vcycle_batched_dev(mgldg_ctx* ctx, mgldg_mg* mg, int k, const double* B, double* X);
/* pcg (krylov.h:22-68) on every column of B at once, sharing each SpMM and
 * V-cycle; column c stops on its own criterion and equals the single-RHS
 * solve of B[:,c].  iters[k] (host, may be NULL); res_hist (host, may be
 * NULL) receives maxit*k doubles, res_hist[c*maxit + i] = ||r_c|| after
 * iteration i.  MGLDG_ERR_BREAKDOWN names the first broken column.  The
 * column tile of every SpMM is autotuned on the first call for a given k. */
int mgldg_pcg_batched_dev(mgldg_ctx* ctx, mgldg_mg* mg, const mgldg_bsr* A, int k,
                          const double* B, double* X, double tol, int maxit, int* iters,
                          double* res_hist);
int mgldg_pcg_batched(mgldg_ctx* ctx, mgldg_mg* mg, const mgldg_bsr* A, int k,
                      const double* B, double* X, double tol, int maxit, int* iters,
                      double* res_hist);
/* No counterpart in the reference: many independent systems of uneven
 * sizes solved together.  A holds them as one block-diagonal operator (for
 * example the LDG operator of a union of meshes, whose multigrid hierarchy
 * is then block diagonal as well); segment s is unknowns
 * [seg_offsets[s], seg_offsets[s+1]) (host array of nseg+1 int64).  Every
 * SpMV and V-cycle covers all segments at once, every segment keeps its own
 * CG scalars and stopping test (krylov.h:22-68), so segment s reproduces the
 * pcg of its own system; iters[nseg] and res_hist[s*maxit + i] as in
 * mgldg_pcg_batched_dev.  Device vectors b, x. */
int mgldg_pcg_segmented_dev(mgldg_ctx* ctx, mgldg_mg* mg, const mgldg_bsr* A, int nseg,
                            const int64_t* seg_offsets, const double* b, double* x, double tol, int maxit,
                            int* iters, double* res_hist);
/* Column tile widths (32, 64 or 128) the autotuner chose for level `level`'s
 * SpMM, Jacobi sweep, restriction, prolongation and for the outer FP64 SpMM. */
int mgldg_mg_batch_tiles(const mgldg_mg* mg, int level, int* spmm, int* jacobi, int* restrict_,
                         int* prolong, int* outer);

/* ------------------------------------------- diffusivity and adjoints -- */
/* No counterpart in the reference (its operators have unit diffusivity);
 * these entries extend construct_laplacian (ldgpoisson.h:34-52) and the pcg
 * of krylov.h:22-68 to a per-element diffusivity kappa and its adjoint.
 *
 * A = T + sum_d G_d^T diag(kappa_e M_e) G_d, replacing ops' Laplacian.
 * kappa: host array, one positive value per element (row of M), or NULL
 * for kappa = 1 (then A equals mgldg_ops_construct_laplacian's). */
int mgldg_ops_construct_laplacian_kappa(mgldg_ctx* ctx, mgldg_ops* ops, const double* kappa);
/* dkappa[e] = -sum_d (G_d lambda)_e^T M_e (G_d u)_e  (device vectors):
 * the gradient of a loss L with respect to kappa_e when A(kappa) u = b and
 * lambda solves the adjoint system A lambda = dL/du. */
int mgldg_kappa_gradient_dev(mgldg_ctx* ctx, const mgldg_ops* ops, const double* u,
                             const double* lambda, double* dkappa);
/* Loss L = 1/2 ||u - u_obs||^2 of the solution of ops' A u = b: forward pcg
 * (u in/out, the initial guess on entry), adjoint pcg with the same
 * preconditioner mg (lambda in/out) and, if dkappa != NULL, dL/dkappa.
 * dL/db = lambda.  loss (host, may be NULL); iters[2] (host, may be NULL) =
 * forward and adjoint iteration counts.  All vectors are device pointers. */
int mgldg_adjoint_l2_dev(mgldg_ctx* ctx, mgldg_mg* mg, const mgldg_ops* ops, const double* b,
                         const double* u_obs, double tol, int maxit, double* u, double* lambda,
                         double* dkappa, double* loss, int* iters);

/* ------------------------------------------------------------ host logic -- */
/* Level sets of the block Gauss-Seidel sweep (host only, no GPU needed): for
 * the forward sweep of multigrid.h:240-249 (reverse=0) or the reverse sweep
 * of :251-261 (reverse=1), level[i] = 1 + max level of the rows that precede
 * row i in sweep order and share a block with it.  order[] lists the rows by
 * level; nlevels is the number of dependent steps of one sweep. */
int mgldg_gs_levels(int nbr, const int* row_ptr, const int* col_idx, int reverse,
                    int* level, int* order, int* nlevels);
/* Level sets of one smoothing pass of nsw (1..7) consecutive sweeps in one
 * direction, as the GPU runs them in one launch (multigrid.h:202-216 applies
 * the npre forward or npost reverse sweeps back to back): sweep s of row i,
 * level[s * nbr + i], follows sweep s of the earlier neighbours and sweep
 * s - 1 of the later neighbours and of row i itself.  nlevels receives the
 * number of dependent steps of the whole pass (host only, no GPU needed). */
int mgldg_gs_pass_levels(int nbr, const int* row_ptr, const int* col_idx, int reverse, int nsw,
                         int* level, int* nlevels);
/* Failure-detection self test (no reference counterpart): runs the
 * Gauss-Seidel kernel on a two-row system whose dependency is never
 * released, so its bounded wait expires after timeout_ns.  *status receives
 * MGLDG_ERR_TIMEOUT when the kernel reported the expiry; the call itself
 * returns MGLDG_OK when the context stayed usable. */
int mgldg_selftest_wait_timeout(mgldg_ctx* ctx, int64_t timeout_ns, int* status);

/* ------------------------------------------------------------ profiling -- */
#define MGLDG_K_SPMV      0   /* BSR SpMV / residual (FP64 or FP32) */
#define MGLDG_K_GS        1   /* level-scheduled block Gauss-Seidel sweep */
#define MGLDG_K_JACOBI    2   /* fused block-Jacobi sweep */
#define MGLDG_K_TRANSFER  3   /* restriction / prolongation */
#define MGLDG_K_COARSE    4   /* coarsest-level solve */
#define MGLDG_K_VECTOR    5   /* pcg dots / axpys / conversions */
#define MGLDG_K_SETUP     6   /* assembly, Galerkin products, block inverses */
#define MGLDG_K_NCLASS    7
/* on=1: time every kernel launch with CUDA events on the context's stream. */
int mgldg_prof_enable(mgldg_ctx* ctx, int on);
int mgldg_prof_reset(mgldg_ctx* ctx);
/* Launch count and summed event time (ms) of one kernel class since reset
 * (time only while enabled).  Synchronises the stream. */
int mgldg_prof_query(mgldg_ctx* ctx, int kclass, int64_t* launches, double* ms);
/* The same for the launches that worked on one multigrid level (0 = finest;
 * -1 = work outside the V-cycle, such as pcg's own products). */
int mgldg_prof_query_level(mgldg_ctx* ctx, int kclass, int level, int64_t* launches, double* ms);

#ifdef __cplusplus
}
#endif

#endif /* MGLDG_H */

/*
 * oracle.h -- C interface of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a plain C++17 restatement of the reference's Cartesian LDG
 * Poisson solver path (danfortunato/multigrid-ldg, src/cartesian/...).  It is
 * the checker for the CUDA product: only tests/, __graft_entry__.smoke() and
 * the cpu_baseline leg of bench.py load it.  Nothing in the product links it.
 *
 * Parity status: the reference itself cannot be compiled here (it needs
 * Eigen 3 and Intel MKL, neither is installed), so the oracle is pinned
 * against the reference's own constant tables (master.h), its only literal
 * known answer (tests/cartesian/matrix_tests.cpp) and the O(h^{p+1})
 * manufactured-solution rate; bit-level parity with the reference binary is
 * unpinned.
 *
 * All functions return 0 on success, non-zero on error.
 */
#ifndef MGLDG_ORACLE_H
#define MGLDG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_problem orc_problem;
typedef struct orc_mg orc_mg;
typedef struct orc_sbm orc_sbm;

/* ---- reference-element tables (src/cartesian/dg/master.h:147-250) ---- */
/* P = nodes per dimension (1..6).  Outputs: nodes[P], denom[P],
 * mass[P*P], invmass[P*P], diff[P*P] (row-major). */
int orc_master_tables(int P, double* nodes, double* denom, double* mass,
                      double* invmass, double* diff);
/* Gauss-Legendre rule on [0,1] with Q points (1..12). */
int orc_quadrature(int Q, double* nodes, double* weights);

/* ---- stand-alone sparse block matrix (sparseblockmatrix.h:62-165) ---- */
int orc_sbm_create(int m, int n, int P, int Q, orc_sbm** out);
int orc_sbm_set_block(orc_sbm* A, int i, int j, const double* blk);
int orc_sbm_add_block(orc_sbm* A, int i, int j, const double* blk);
/* y := alpha*A*x + beta*y   (multiply_add_mv, sparseblockmatrix.tpp:358-371) */
int orc_sbm_mv(const orc_sbm* A, double alpha, const double* x, double beta, double* y);
/* y := A^T x   (multiply_mv_t, sparseblockmatrix.tpp:322-335) */
int orc_sbm_mv_t(const orc_sbm* A, const double* x, double* y);
int orc_sbm_destroy(orc_sbm* A);

/* ---- problem: quadtree + mesh + LDG operators + rhs ---- */
enum { ORC_REFINE_UNIFORM = 0, ORC_REFINE_REF_ADAPTIVE = 1 };
enum { ORC_BC_DIRICHLET = 0, ORC_BC_NEUMANN = 1, ORC_BC_PERIODIC = 2 };
enum { ORC_TEST_CONVERGENCE = 0, ORC_TEST_SOLUTION = 1, ORC_TEST_GAUSSIAN = 2 };
enum { ORC_COARSEN_EQUAL = 0, ORC_COARSEN_RAPID = 1 };

/* Builds Quadtree<2>(h) -> Mesh<2,P> -> LDGPoisson<2,P> -> rhs, following
 * tests/cartesian/dg_tests.cpp:206-286.  `dx` is the mesh spacing passed to
 * the h() callback; `seed` selects the Gaussian-sum forcing (test=GAUSSIAN). */
int orc_problem_create(int P, double dx, int refine, int coarsening, int bctype,
                       int test, double tau0, double tauD, uint64_t seed,
                       orc_problem** out);
/* Adaptive quadtree of the seeded-points rule (extension; the multi-RHS
 * workload's mesh): a cell of width 2^-(base+l) is split while l < extra and
 * its centre lies within radius*2^-l of one of npoints seeded points
 * (mt19937_64, 53-bit uniforms, x/y pairs), optionally 2:1 face balanced;
 * tau_per_face: penalties tau0/min(h_L,h_R) and tauD/h_L instead of the
 * reference's constants.  Homogeneous Dirichlet, Gaussian-sum rhs. */
int orc_problem_create_points(int P, int base_level, int extra_levels, int npoints, uint64_t point_seed,
                              double radius, int balance, int tau_per_face, double tau0, double tauD,
                              uint64_t rhs_seed, orc_problem** out);
int orc_seeded_points(uint64_t seed, int n, double* xy);
/* Unstructured P_{P-1} LDG on a triangle mesh (points p[2*np], triangles
 * t[3*nt], 0-based), homogeneous Dirichlet on every boundary face, rhs = M f
 * with the disk Gaussian-sum forcing of rhs_seed, and an agglomeration
 * hierarchy of up to agg_levels levels (greedy seeded aggregates of <= 4,
 * tensor-product coarse spaces on the aggregates' bounding boxes). */
int orc_simplex_problem_create(int np, const double* p, int nt, const int* t, int P, double tau0, double tauD,
                               int agg_levels, uint64_t agg_seed, uint64_t rhs_seed, orc_problem** out);
/* N = 2 (triangles, p[2*np], t[3*nt]) or 3 (tetrahedra, p[3*np], t[4*nt]) */
int orc_simplex_problem_create_nd(int N, int np, const double* p, int nt, const int* t, int P, double tau0,
                                  double tauD, int agg_levels, uint64_t agg_seed, uint64_t rhs_seed,
                                  orc_problem** out);
int orc_simplex_master_nd(int N, int P, double* mass, double* diff, double* nodes);
/* block shape of hierarchy level l; aggregate of every finer element at agglomeration level l */
int orc_hier_block(const orc_problem* pr, int l, int* br, int* bc);
int orc_problem_partition(const orc_problem* pr, int l, int* agg);
/* External agglomerator for the simplex hierarchies created after this call
 * (null restores the greedy seeded one).  It receives one level's weighted
 * dual graph in CSR form -- n nodes, xadj[n+1], adjncy / adjwgt (shared face
 * measure), vvol (node volume), vsurf (boundary face measure) -- and the
 * dimension N, writes part[n] and returns the number of aggregates (the
 * argument list of MGridGen, lib/ParMGridGen-1.0/mgridgen.h, as the
 * reference's src/unstructured/mesh/agglomeration.h:53-225 fills it). */
typedef int (*orc_agglomerator)(int n, const int* xadj, const int* adjncy, const double* adjwgt,
                                const double* vvol, const double* vsurf, int N, int* part);
int orc_set_agglomerator(orc_agglomerator fn);
/* Shape of agglomeration level l's aggregates: count, mean and largest
 * isoperimetric ratio (2-D: S^2 / (4 pi V), 3-D: S^3 / (36 pi V^2), S the
 * aggregate's surface, V its volume; 1 for a disk / ball). */
int orc_problem_agg_quality(const orc_problem* pr, int l, int* naggs, double* mean_ratio, double* max_ratio);
/* simplex master element (N = 1 or 2): mass, diff matrices (row-major npl x npl), nodes[npl*N] */
int orc_simplex_master(int N, int P, double* mass, double* diff0, double* diff1, double* nodes);
int orc_problem_destroy(orc_problem* pr);
/* ne, npl (=P^2), number of DOFs, number of quadtree levels, faces, boundary faces */
int orc_problem_info(const orc_problem* pr, int* ne, int* npl, int* ndof,
                     int* nlevels, int* nfaces, int* nbfaces);
/* element bounding boxes in mesh (DFS) order: lower[2*ne], upper[2*ne] */
int orc_problem_elements(const orc_problem* pr, double* lower, double* upper);
/* which: 0=M 1=G0 2=G1 3=T 4=A.  Sorted-column CSR export. */
int orc_problem_nnzb(const orc_problem* pr, int which, int* nnzb);
int orc_problem_export(const orc_problem* pr, int which, int* row_ptr,
                       int* col_idx, double* vals);
/* right-hand side b (ndof) and exact nodal solution u_true (zeros if none) */
int orc_problem_rhs(const orc_problem* pr, double* b);
int orc_problem_utrue(const orc_problem* pr, double* u);
/* interpolation hierarchy T[l] (interpolationhierarchy.h:30-82) */
int orc_hier_size(const orc_problem* pr, int* nT);
int orc_hier_shape(const orc_problem* pr, int l, int* nbr, int* nbc, int* nnzb);
int orc_hier_export(const orc_problem* pr, int l, int* row_ptr, int* col_idx,
                    double* vals);
/* Gaussian-sum parameters actually drawn for `seed`: cx[8],cy[8],w[8],a[8] */
int orc_gaussian_params(uint64_t seed, double* cx, double* cy, double* w, double* a);

/* ---- multigrid (multigrid.h) ---- */
enum { ORC_RELAX_JACOBI = 0, ORC_RELAX_GS = 1 };
enum { ORC_COARSE_CHOLESKY = 0, ORC_COARSE_RELAX = 1, ORC_COARSE_DENSE = 2 };
enum { ORC_RESTRICT_RAT = 0, ORC_RESTRICT_RATRAT = 1 };

/* nlevels <= 0 : use the whole hierarchy (as the reference does);
 * otherwise keep only the first nlevels levels (extension).  mean_project=1
 * reproduces multigrid.h:367 (b -= mean(b) on the coarsest level). */
int orc_mg_create(const orc_problem* pr, int relaxation, double omega, int solver,
                  int npre, int npost, int restriction, int nlevels,
                  int mean_project, orc_mg** out);
/* hp-multigrid (multigrid.h:436-560): p-levels degrees[0] (= the problem's
 * P) -> ... -> degrees[ndeg-1] on the fine mesh, then nh h-levels at the
 * last degree.  Transfers are kept by the mg handle. */
int orc_mg_create_hp(const orc_problem* pr, const int* degrees, int ndeg, int nh, int relaxation,
                     double omega, int solver, int npre, int npost, int restriction,
                     int mean_project, orc_mg** out);
int orc_mg_transfer_shape(const orc_mg* mg, int l, int* nbr, int* nbc, int* br, int* bc, int* nnzb);
int orc_mg_transfer_export(const orc_mg* mg, int l, int* row_ptr, int* col_idx, double* vals);
int orc_mg_destroy(orc_mg* mg);
int orc_mg_nlevels(const orc_mg* mg, int* n);
/* level operator export: which 0=M 1=G0 2=G1 3=T 4=A */
int orc_mg_level_nnzb(const orc_mg* mg, int l, int which, int* nbr, int* nnzb);
int orc_mg_level_block(const orc_mg* mg, int l, int* b);   /* block size of level l */
int orc_mg_level_export(const orc_mg* mg, int l, int which, int* row_ptr,
                        int* col_idx, double* vals);
/* one V-cycle from level 0: x (in/out) with right-hand side b */
int orc_mg_vcycle(orc_mg* mg, const double* b, double* x);
/* n relaxations on level l (reverse=1: reverse GS order) */
int orc_mg_relax(orc_mg* mg, int l, int n, int reverse, const double* b, double* x);
/* pcg (krylov.h:22-68).  mg == NULL: identity preconditioner.
 * hist[k] = ||r|| printed after iteration k (needs maxit doubles). */
int orc_pcg(const orc_problem* pr, orc_mg* mg, const double* b, double* x,
            double tol, int maxit, int* iters, double* hist, double* delta_hist);
/* Matrix Market dump of a fine-level operator (SparseBlockMatrix::write,
 * sparseblockmatrix.tpp:145-164) and nodal dump of a vector
 * (Function::write, function.h:173-190). */
int orc_problem_write_mtx(const orc_problem* pr, int which, const char* path);
int orc_problem_write_fun(const orc_problem* pr, const double* u, const char* path);
/* y := alpha*A*x + beta*y with the fine-level operator `which` */
int orc_problem_mv(const orc_problem* pr, int which, double alpha, const double* x,
                   double beta, double* y);

#ifdef __cplusplus
}
#endif

#endif

// setup.cu -- Galerkin coarsening setup: block SpGEMM (symbolic pass in
// plan.cu, numeric pass here, both on the GPU), batched block inverses, the
// Laplacian triple product and the dense inverse of the coarsest level.
//
// Follows the reference's Level coarse constructor
// (src/cartesian/multigrid/multigrid.h:105-171), construct_laplacian
// (src/cartesian/dg/ldgpoisson.h:34-52) and multiply_mm / multiply_mm_t
// (src/cartesian/util/sparseblockmatrix.tpp:234-280).
//
// A product plan lists, for every output block, the ordered terms that sum
// into it.  The numeric kernel gives each output block to one CTA (one thread
// per block entry); each term's operands are staged in shared memory, so the
// sum over terms runs in a fixed order (the reference's order over d and k),
// and every output block is computed by exactly one CTA.
#include <algorithm>
#include <chrono>
#include <numeric>

#include "api.cuh"
#include "plan.cuh"

using namespace mg;

namespace mg {

// setup phase clocks (symbolic plans, numeric products), read by
// the MGLDG_SETUP_TRACE report of mgldg_mg_create
static double g_plan_ms = 0, g_prod_ms = 0;
void setup_clock_take(double* plan_ms, double* prod_ms) {
    *plan_ms = g_plan_ms;
    *prod_ms = g_prod_ms;
    g_plan_ms = g_prod_ms = 0;
}
struct Clock {
    double* acc;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    explicit Clock(double* a) : acc(a) {}
    ~Clock() { *acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
};

// ------------------------------------------------------------ numeric ------
struct Opnd {
    const double* val;
    const int* blk;
    int r, c;
    __device__ __forceinline__ const double* at(int k) const {
        return val + (size_t)(blk ? blk[k] : k) * r * c;
    }
};

// out[o] = init[o] (or 0) + sum_t opX(X[t.x]) * (M[t.m]) * Y[t.y]
__global__ void __launch_bounds__(1024)
    k_prod(int nout, int oR, int oC, Opnd X, int tX, Opnd Mm, Opnd Y, const int* __restrict__ tptr,
           const int3* __restrict__ terms, const double* init, double* out) {
    extern __shared__ double sm[];
    double* sX = sm;
    double* sM = sX + 1024;
    double* sY = sM + 1024;
    double* sW = sY + 1024;
    const int inner = tX ? X.r : X.c;   // columns of op(X)
    const int nth = blockDim.x;
    const int nent = oR * oC;
    for (int o = blockIdx.x; o < nout; o += gridDim.x) {
        double acc[1];
        const int e = threadIdx.x;
        const int r = e / oC, s = e - r * oC;
        acc[0] = (init && e < nent) ? init[(size_t)o * nent + e] : 0.0;
        for (int t = tptr[o]; t < tptr[o + 1]; ++t) {
            const int3 tm = terms[t];
            const double* px = X.at(tm.x);
            const double* py = Y.at(tm.z);
            for (int q = threadIdx.x; q < X.r * X.c; q += nth) sX[q] = px[q];
            for (int q = threadIdx.x; q < Y.r * Y.c; q += nth) sY[q] = py[q];
            if (tm.y >= 0) {
                const double* pm = Mm.at(tm.y);
                for (int q = threadIdx.x; q < Mm.r * Mm.c; q += nth) sM[q] = pm[q];
            }
            __syncthreads();
            const double* Wp;
            int wc;
            if (tm.y >= 0) {
                // W = op(X) * M   (oR x Mm.c)
                for (int q = threadIdx.x; q < oR * Mm.c; q += nth) {
                    int rr = q / Mm.c, cc = q - rr * Mm.c;
                    double v = 0;
                    for (int z = 0; z < inner; ++z) v += (tX ? sX[z * X.c + rr] : sX[rr * X.c + z]) * sM[z * Mm.c + cc];
                    sW[q] = v;
                }
                __syncthreads();
                Wp = sW;
                wc = Mm.c;
                if (e < nent) {
                    double v = 0;
                    for (int z = 0; z < wc; ++z) v += Wp[r * wc + z] * sY[z * Y.c + s];
                    acc[0] += v;
                }
            } else if (e < nent) {
                double v = 0;
                for (int z = 0; z < inner; ++z) v += (tX ? sX[z * X.c + r] : sX[r * X.c + z]) * sY[z * Y.c + s];
                acc[0] += v;
            }
            __syncthreads();
        }
        if (e < nent) out[(size_t)o * nent + e] = acc[0];
        __syncthreads();
    }
}

static Opnd opnd(const mgldg_bsr* A) { return Opnd{A->val, A->blk, A->br, A->bc}; }

static void run_plan(mgldg_ctx* ctx, const DPlan& P, int oR, int oC, Opnd X, bool tX, Opnd Mm, Opnd Y,
                     const double* init, double* out) {
    const int nout = P.nkeys;
    if (nout == 0) return;
    Clock clk(&g_prod_ms);
    MG_REQUIRE(oR * oC <= 1024 && X.r * X.c <= 1024 && Y.r * Y.c <= 1024 && Mm.r * Mm.c <= 1024,
               MGLDG_ERR_UNSUPPORTED, "block products limited to 32x32 blocks");
    const int nth = ((oR * oC + 31) / 32) * 32;
    const int grid = std::min(nout, 1 << 20);
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_prod<<<grid, nth, 4 * 1024 * sizeof(double), ctx->stream>>>(nout, oR, oC, X, tX ? 1 : 0, Mm, Y, P.tptr,
                                                                      P.terms, init, out);
    }
    check_launch();
    sync(ctx);
}

// C = op(X) * Y as a new BSR
static mgldg_bsr* mm(mgldg_ctx* ctx, const mgldg_bsr* X, bool tX, const mgldg_bsr* Y) {
    DPlan P;
    {
        Clock clk(&g_plan_ms);
        dplan_mm(ctx, X, tX, Y, &P);
    }
    const int oR = tX ? X->bc : X->br, oC = Y->bc;
    mgldg_bsr* C = bsr_from_dplan(ctx, P, oR, oC);
    try {
        run_plan(ctx, P, oR, oC, opnd(X), tX, Opnd{nullptr, nullptr, 0, 0}, opnd(Y), nullptr, C->val);
    } catch (...) {
        delete C;
        throw;
    }
    return C;
}

// ------------------------------------------------------- block inverses ----
// The inverse of each diagonal block, formed the way the reference solves
// with it: an LDL^T factorisation with symmetric diagonal pivoting (the
// Eigen::LDLT of multigrid.h:93-95,133-135,168-170; at step k the largest
// remaining diagonal entry in magnitude, the first one on ties, is swapped
// into position k), then one forward/diagonal/backward substitution per unit
// vector.  Every operation is rounded separately (no fused multiply-add), in
// the order of the textbook algorithm (Golub & Van Loan, 4.2), so a column of
// the inverse equals that LDL^T solve of the unit vector bit for bit.  An
// explicit inverse from Gauss-Jordan elimination instead moved the PCG
// residual history of a 128 x 128 Q3 problem 5x further from the oracle's.
// One warp per block (b <= 32): the factorisation's Schur updates run over
// the lanes, then lane j substitutes for column j.  An unknown whose row and
// column are exactly zero (a dropped coarse basis function) is absent: it is
// factored as a unit diagonal and its row and column of the inverse are zero
// (the pseudo-inverse of the block).
__global__ void k_block_inverse(int n, int b, const double* __restrict__ val, const int* __restrict__ blk,
                                const int* __restrict__ pos, double* __restrict__ out, int* status) {
    extern __shared__ double sm[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    // per warp: W (b x b), D (b), the lanes' substitution vectors X (b x 32),
    // the transpositions (b ints, stored as doubles)
    double* W = sm + (size_t)warp * (b * b + 2 * b + 32 * b);
    double* D = W + b * b;
    double* trd = D + b;
    double* X = trd + b;
    for (int i = blockIdx.x * wpb + warp; i < n; i += gridDim.x * wpb) {
        const int p = pos ? pos[i] : i;
        if (p < 0) {
            if (lane == 0) atomicOr(status, 2);
            continue;
        }
        const double* a = val + (size_t)(blk ? blk[p] : p) * b * b;
        for (int q = lane; q < b * b; q += 32) W[q] = a[q];
        __syncwarp();
        bool zero = lane < b;
        for (int c = 0; c < b && zero; ++c) zero = W[lane * b + c] == 0.0 && W[c * b + lane] == 0.0;
        const unsigned absent = __ballot_sync(0xffffffffu, zero);
        __syncwarp();
        if (zero) W[lane * b + lane] = 1.0;
        __syncwarp();
        bool bad = false;
        for (int k = 0; k < b; ++k) {
            // pivot: largest |W(r,r)|, r >= k, the first on ties
            double v = (lane >= k && lane < b) ? fabs(W[lane * b + lane]) : -1.0;
            int idx = lane;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
                const int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
                if (v2 > v || (v2 == v && i2 < idx)) { v = v2; idx = i2; }
            }
            if (lane == 0) trd[k] = (double)idx;
            if (idx != k) {
                for (int c = lane; c < b; c += 32) {
                    const double t = W[k * b + c];
                    W[k * b + c] = W[idx * b + c];
                    W[idx * b + c] = t;
                }
                __syncwarp();
                for (int r = lane; r < b; r += 32) {
                    const double t = W[r * b + k];
                    W[r * b + k] = W[r * b + idx];
                    W[r * b + idx] = t;
                }
                __syncwarp();
            }
            const double dk = W[k * b + k];
            if (!(fabs(dk) > 0.0) || !isfinite(dk)) bad = true;
            if (lane == 0) D[k] = dk;
            // column k of L
            for (int r = k + 1 + lane; r < b; r += 32) W[r * b + k] = __ddiv_rn(W[r * b + k], dk);
            __syncwarp();
            // Schur complement of the trailing block: W(r,c) -= (l_rk d_k) l_ck
            // for k < c <= r, mirrored into W(c,r)
            const int m = b - k - 1;
            for (int t = lane; t < m * (m + 1) / 2; t += 32) {
                int r = (int)((sqrtf(8.0f * t + 1.0f) - 1.0f) * 0.5f);
                while ((r + 1) * (r + 2) / 2 <= t) ++r;
                while (r * (r + 1) / 2 > t) --r;
                const int c = t - r * (r + 1) / 2;
                const int rr = k + 1 + r, cc = k + 1 + c;
                const double lik = W[rr * b + k];
                const double vv = __dsub_rn(W[rr * b + cc], __dmul_rn(__dmul_rn(lik, dk), W[cc * b + k]));
                W[rr * b + cc] = vv;
                W[cc * b + rr] = vv;
            }
            __syncwarp();
        }
        // lane j: x = LDL^T \ e_j (with the pivoting), column j of the inverse
        if (lane < b) {
            for (int r = 0; r < b; ++r) X[r * 32 + lane] = (r == lane) ? 1.0 : 0.0;
            for (int k = 0; k < b; ++k) {
                const int t = (int)trd[k];
                if (t != k) {
                    const double s = X[k * 32 + lane];
                    X[k * 32 + lane] = X[t * 32 + lane];
                    X[t * 32 + lane] = s;
                }
            }
            for (int r = 0; r < b; ++r) {
                double s = X[r * 32 + lane];
                for (int c = 0; c < r; ++c) s = __dsub_rn(s, __dmul_rn(W[r * b + c], X[c * 32 + lane]));
                X[r * 32 + lane] = s;
            }
            for (int r = 0; r < b; ++r) X[r * 32 + lane] = __ddiv_rn(X[r * 32 + lane], D[r]);
            for (int r = b - 1; r >= 0; --r) {
                double s = X[r * 32 + lane];
                for (int c = r + 1; c < b; ++c) s = __dsub_rn(s, __dmul_rn(W[c * b + r], X[c * 32 + lane]));
                X[r * 32 + lane] = s;
            }
            for (int k = b - 1; k >= 0; --k) {
                const int t = (int)trd[k];
                if (t != k) {
                    const double s = X[k * 32 + lane];
                    X[k * 32 + lane] = X[t * 32 + lane];
                    X[t * 32 + lane] = s;
                }
            }
        }
        __syncwarp();
        if (bad && lane == 0) atomicOr(status, 1);
        double* o = out + (size_t)i * b * b;
        for (int q = lane; q < b * b; q += 32) {
            const int r = q / b, c = q - r * b;
            o[q] = ((absent >> r) & 1u) || ((absent >> c) & 1u) ? 0.0 : X[r * 32 + c];
        }
        __syncwarp();
    }
}

void block_inverse(mgldg_ctx* ctx, const mgldg_bsr* A, double* out, int* dstatus) {
    MG_REQUIRE(A->br == A->bc && A->br <= 32, MGLDG_ERR_UNSUPPORTED, "block inverse needs square blocks <= 32");
    MG_REQUIRE(A->diag != nullptr, MGLDG_ERR_ARG, "diagonal index not built");
    const int b = A->br;
    const size_t per_warp = (size_t)(b * b + 2 * b + 32 * b) * sizeof(double);
    const int wpb = per_warp * 4 <= 48 * 1024 ? 4 : (per_warp * 2 <= 48 * 1024 ? 2 : 1);
    const size_t smem = (size_t)wpb * per_warp;
    int grid = std::max(1, std::min((A->nbr + wpb - 1) / wpb, ctx->sm_count * 16));
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_block_inverse<<<grid, wpb * 32, smem, ctx->stream>>>(A->nbr, b, A->val, A->blk, A->diag, out, dstatus);
    }
    check_launch();
}

static void check_status(mgldg_ctx* ctx, int* dstatus, const char* what) {
    int h = 0;
    download(ctx, &h, dstatus, 1);
    sync(ctx);
    if (h & 2) throw Error(MGLDG_ERR_SHAPE, std::string(what) + ": missing diagonal block");
    if (h & 1) throw Error(MGLDG_ERR_NOT_SPD, std::string(what) + ": singular diagonal block");
}

// out[q] = A's block src[q] (zero block where src[q] < 0)
__global__ void k_gather_blocks(int64_t n, int bsz, const int* __restrict__ src, const double* __restrict__ val,
                                const int* __restrict__ blk, double* __restrict__ out) {
    for (int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x; t < n * bsz; t += (int64_t)gridDim.x * 256) {
        int64_t q = t / bsz;
        int e = (int)(t - q * bsz);
        int s = src[q];
        out[t] = (s < 0) ? 0.0 : val[(size_t)(blk ? blk[s] : s) * bsz + e];
    }
}

// out[q] = A's block src[q] for the n output positions (src on the device)
static void gather_blocks(mgldg_ctx* ctx, int64_t n, const int* dsrc, const mgldg_bsr* A, double* out) {
    if (n == 0) return;
    const int g = (int)std::min<int64_t>((n * (int64_t)A->bsz() + 255) / 256, ctx->sm_count * 32);
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_gather_blocks<<<g, 256, 0, ctx->stream>>>(n, (int)A->bsz(), dsrc, A->val, A->blk, out);
    }
    check_launch();
}

// ------------------------------------------------------- construct_laplacian
// A = T + sum_d sum_k G_d(k,:)^T M(k,k) G_d(k,:)   (ldgpoisson.h:34-52)
static mgldg_bsr* laplacian(mgldg_ctx* ctx, mgldg_bsr* M, mgldg_bsr* const* G, int ndim, mgldg_bsr* T) {
    bsr_build_diag(M);
    std::vector<const mgldg_bsr*> Xs(G, G + ndim);
    std::vector<DPlan> per;
    DPlan U;
    {
        Clock clk(&g_plan_ms);
        dplan_triple(ctx, Xs, M, T, &per, &U);
    }
    const int b = T->br;
    mgldg_bsr* A = bsr_from_dplan(ctx, U, b, b);
    double* initv = nullptr;
    int* dsrc = nullptr;
    try {
        // A starts as a copy of T scattered into the union pattern
        initv = dalloc<double>(std::max<size_t>(1, (size_t)U.nkeys * A->bsz()));
        dsrc = dalloc<int>(std::max(1, U.nkeys));
        dplan_scatter_index(ctx, U, T, dsrc);
        gather_blocks(ctx, U.nkeys, dsrc, T, initv);
        double* src = initv;
        for (int d = 0; d < ndim; ++d) {
            run_plan(ctx, per[d], b, b, opnd(G[d]), true, opnd(M), opnd(G[d]), src, A->val);
            src = A->val;
        }
    } catch (...) {
        dfree(initv);
        dfree(dsrc);
        delete A;
        throw;
    }
    dfree(dsrc);
    dfree(initv);
    return A;
}

mgldg_bsr* laplacian_of(mgldg_ctx* ctx, mgldg_bsr* M, mgldg_bsr* const* G, int ndim, mgldg_bsr* T) {
    return laplacian(ctx, M, G, ndim, T);
}

void construct_laplacian(mgldg_ctx* ctx, mgldg_ops* ops) {
    MG_REQUIRE(ops->has_MGT(), MGLDG_ERR_ARG, "construct_laplacian needs M, G and T");
    mgldg_bsr* A = laplacian(ctx, ops->M, ops->G, ops->ndim, ops->T);
    delete ops->A;
    ops->A = A;
}

// ------------------------------------------------------------ Galerkin -----
// RATRAT (multigrid.h:115-157):
//   M_c = T^T M_f T ; Minv = M_c(i,i)^-1 ; G_c,d = M_c^-1 T^T M_f G_f,d T ;
//   T_c = T^T T_f T ; A_c = construct_laplacian(M_c, G_c, T_c)
mgldg_ops* galerkin_ratrat(mgldg_ctx* ctx, const mgldg_ops* f, const mgldg_bsr* T) {
    MG_REQUIRE(f->has_MGT(), MGLDG_ERR_ARG, "RATRAT needs M, G and T on the finer level");
    MG_REQUIRE(T->nbr == f->M->nbr && T->br == f->M->br, MGLDG_ERR_SHAPE, "interpolation shape mismatch");
    bsr_build_diag(f->M);
    mgldg_ops* c = new mgldg_ops();
    c->ctx = ctx;
    c->ndim = f->ndim;
    int* dstatus = nullptr;
    double* minv = nullptr;
    std::vector<mgldg_bsr*> tmp;
    try {
        const int bc = T->bc;
        // coarse mass matrix (block diagonal): sum_k T(k,i)^T M(k,k) T(k,j)
        std::vector<DPlan> per;
        DPlan U;
        {
            Clock clk(&g_plan_ms);
            dplan_triple(ctx, {T}, f->M, nullptr, &per, &U);
        }
        c->M = bsr_from_dplan(ctx, U, bc, bc);
        run_plan(ctx, per[0], bc, bc, opnd(T), true, opnd(f->M), opnd(T), nullptr, c->M->val);
        bsr_build_diag(c->M);
        // Minv: inverses of the diagonal blocks of M_c
        dstatus = dalloc<int>(1);
        MG_CHECK_CUDA(cudaMemsetAsync(dstatus, 0, sizeof(int), ctx->stream));
        minv = dalloc<double>((size_t)c->M->nbr * bc * bc);
        block_inverse(ctx, c->M, minv, dstatus);
        check_status(ctx, dstatus, "coarse mass matrix");
        for (int d = 0; d < f->ndim; ++d) {
            mgldg_bsr* t1 = mm(ctx, f->G[d], false, T);   // G_f T
            tmp.push_back(t1);
            mgldg_bsr* t2 = mm(ctx, f->M, false, t1);     // M_f (G_f T)
            tmp.push_back(t2);
            mgldg_bsr* g = mm(ctx, T, true, t2);          // T^T M_f G_f T
            tmp.push_back(g);
            // G_c(i,j) = Minv_i G(i,j)
            DPlan P;
            dplan_rowscale(ctx, g, &P);
            c->G[d] = bsr_new(ctx, g->nbr, g->nbc, bc, bc, g->h_row_ptr, g->h_col_idx);
            run_plan(ctx, P, bc, bc, Opnd{minv, nullptr, bc, bc}, false, Opnd{nullptr, nullptr, 0, 0}, opnd(g), nullptr,
                     c->G[d]->val);
            for (auto* m : tmp) delete m;
            tmp.clear();
        }
        // T_c = T^T T_f T
        mgldg_bsr* t1 = mm(ctx, f->T, false, T);
        tmp.push_back(t1);
        c->T = mm(ctx, T, true, t1);
        for (auto* m : tmp) delete m;
        tmp.clear();
        c->A = laplacian(ctx, c->M, c->G, c->ndim, c->T);
    } catch (...) {
        for (auto* m : tmp) delete m;
        dfree(dstatus);
        dfree(minv);
        delete c;
        throw;
    }
    dfree(dstatus);
    dfree(minv);
    return c;
}

// RAT (multigrid.h:158-163): A_c = T^T A_f T
mgldg_ops* galerkin_rat(mgldg_ctx* ctx, const mgldg_ops* f, const mgldg_bsr* T) {
    MG_REQUIRE(f->A != nullptr, MGLDG_ERR_ARG, "RAT needs A on the finer level");
    mgldg_ops* c = new mgldg_ops();
    c->ctx = ctx;
    c->ndim = f->ndim;
    mgldg_bsr* t1 = nullptr;
    try {
        t1 = mm(ctx, f->A, false, T);
        c->A = mm(ctx, T, true, t1);
    } catch (...) {
        delete t1;
        delete c;
        throw;
    }
    delete t1;
    return c;
}

// -------------------------------------------------- dense coarsest inverse --
__global__ void k_scatter_dense(int nbr, int b, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                                const double* __restrict__ val, const int* __restrict__ blk, int n, double* aug) {
    // aug is n x 2n: [A | I]
    for (int i = blockIdx.x; i < nbr; i += gridDim.x)
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            const double* a = val + (size_t)(blk ? blk[k] : k) * b * b;
            int j = col_idx[k];
            for (int q = threadIdx.x; q < b * b; q += blockDim.x) {
                int r = q / b, c = q - r * b;
                aug[(size_t)(i * b + r) * 2 * n + j * b + c] = a[q];
            }
        }
}
__global__ void k_identity_right(int n, double* aug) {
    for (int r = blockIdx.x; r < n; r += gridDim.x)
        for (int c = threadIdx.x; c < n; c += blockDim.x) aug[(size_t)r * 2 * n + n + c] = (r == c) ? 1.0 : 0.0;
}

// Gauss-Jordan on [A | I] with partial pivoting; one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) k_gauss_jordan(int n, double* aug, int* status) {
    __shared__ double sv[32];
    __shared__ int si[32];
    __shared__ int piv;
    __shared__ double pinv;
    const int w2 = 2 * n;
    for (int k = 0; k < n; ++k) {
        double v = -1.0;
        int idx = n;
        for (int r = k + threadIdx.x; r < n; r += blockDim.x) {
            double a = fabs(aug[(size_t)r * w2 + k]);
            if (a > v) { v = a; idx = r; }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            double v2 = __shfl_xor_sync(0xffffffffu, v, o);
            int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
            if (v2 > v || (v2 == v && i2 < idx)) { v = v2; idx = i2; }
        }
        if ((threadIdx.x & 31) == 0) { sv[threadIdx.x >> 5] = v; si[threadIdx.x >> 5] = idx; }
        __syncthreads();
        if (threadIdx.x == 0) {
            double bv = -1.0;
            int bi = n;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
                if (sv[w] > bv || (sv[w] == bv && si[w] < bi)) { bv = sv[w]; bi = si[w]; }
            if (!(bv > 0.0) || !isfinite(bv) || bi >= n) { *status = 1; bi = k; }
            piv = bi;
        }
        __syncthreads();
        const int p = piv;
        if (p != k)
            for (int c = threadIdx.x; c < w2; c += blockDim.x) {
                double t = aug[(size_t)k * w2 + c];
                aug[(size_t)k * w2 + c] = aug[(size_t)p * w2 + c];
                aug[(size_t)p * w2 + c] = t;
            }
        __syncthreads();
        if (threadIdx.x == 0) pinv = 1.0 / aug[(size_t)k * w2 + k];
        __syncthreads();
        for (int c = threadIdx.x; c < w2; c += blockDim.x) aug[(size_t)k * w2 + c] *= pinv;
        __syncthreads();
        // eliminate column k from every other row; the factors are read from
        // column k before it is overwritten (column k is done last)
        for (int q = threadIdx.x; q < n * w2; q += blockDim.x) {
            int r = q / w2, c = q - r * w2;
            if (r == k || c == k) continue;
            aug[q] -= aug[(size_t)r * w2 + k] * aug[(size_t)k * w2 + c];
        }
        __syncthreads();
        for (int r = threadIdx.x; r < n; r += blockDim.x)
            if (r != k) aug[(size_t)r * w2 + k] = 0.0;
        __syncthreads();
    }
}
// The same elimination for larger n, one pivot column per pair of launches:
// k_gj_pivot (one CTA) picks the pivot row, swaps it into row k, saves the
// column-k factors f[r] and scales row k; k_gj_eliminate (all SMs) subtracts
// f[r] times row k from every other row and zeroes column k.
__global__ void __launch_bounds__(1024) k_gj_pivot(int n, int k, double* aug, double* f, int* status) {
    __shared__ double sv[32];
    __shared__ int si[32];
    __shared__ int piv;
    __shared__ double pinv;
    const int w2 = 2 * n;
    double v = -1.0;
    int idx = n;
    for (int r = k + threadIdx.x; r < n; r += blockDim.x) {
        const double a = fabs(aug[(size_t)r * w2 + k]);
        if (a > v) { v = a; idx = r; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double v2 = __shfl_xor_sync(0xffffffffu, v, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, idx, o);
        if (v2 > v || (v2 == v && i2 < idx)) { v = v2; idx = i2; }
    }
    if ((threadIdx.x & 31) == 0) { sv[threadIdx.x >> 5] = v; si[threadIdx.x >> 5] = idx; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double bv = -1.0;
        int bi = n;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
            if (sv[w] > bv || (sv[w] == bv && si[w] < bi)) { bv = sv[w]; bi = si[w]; }
        if (!(bv > 0.0) || !isfinite(bv) || bi >= n) { *status = 1; bi = k; }
        piv = bi;
    }
    __syncthreads();
    const int p = piv;
    if (p != k)
        for (int c = threadIdx.x; c < w2; c += blockDim.x) {
            const double t = aug[(size_t)k * w2 + c];
            aug[(size_t)k * w2 + c] = aug[(size_t)p * w2 + c];
            aug[(size_t)p * w2 + c] = t;
        }
    __syncthreads();
    for (int r = threadIdx.x; r < n; r += blockDim.x) f[r] = (r == k) ? 0.0 : aug[(size_t)r * w2 + k];
    if (threadIdx.x == 0) pinv = 1.0 / aug[(size_t)k * w2 + k];
    __syncthreads();
    for (int c = threadIdx.x; c < w2; c += blockDim.x) aug[(size_t)k * w2 + c] *= pinv;
}

__global__ void __launch_bounds__(256) k_gj_eliminate(int n, int k, double* __restrict__ aug,
                                                     const double* __restrict__ f) {
    const int w2 = 2 * n;
    const double* __restrict__ pk = aug + (size_t)k * w2;
    for (int r = blockIdx.y; r < n; r += gridDim.y) {
        if (r == k) continue;
        const double fr = f[r];
        if (fr == 0.0) continue;
        double* row = aug + (size_t)r * w2;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < w2; c += gridDim.x * blockDim.x)
            row[c] = (c == k) ? 0.0 : row[c] - fr * pk[c];
    }
}

// Absent unknowns of the dense matrix (row and column exactly zero): unit
// diagonal for the elimination, zero rows and columns in the inverse.  One
// warp per row; a warp writes only its own diagonal entry, after its reads.
__global__ void k_mark_absent(int n, double* aug, int* absent) {
    const int lane = threadIdx.x & 31;
    const int w2 = 2 * n;
    for (int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n; r += (gridDim.x * blockDim.x) >> 5) {
        bool z = true;
        for (int c = lane; c < n && z; c += 32) z = aug[(size_t)r * w2 + c] == 0.0 && aug[(size_t)c * w2 + r] == 0.0;
        z = __all_sync(0xffffffffu, z);
        if (lane == 0) {
            absent[r] = z ? 1 : 0;
            if (z) aug[(size_t)r * w2 + r] = 1.0;
        }
    }
}

__global__ void k_extract_right(int n, const double* aug, const int* absent, double* out) {
    for (int r = blockIdx.x; r < n; r += gridDim.x)
        for (int c = threadIdx.x; c < n; c += blockDim.x)
            out[(size_t)r * n + c] = (absent[r] || absent[c]) ? 0.0 : aug[(size_t)r * 2 * n + n + c];
}

void dense_spd_inverse(mgldg_ctx* ctx, const mgldg_bsr* A, double* out_inv) {
    MG_REQUIRE(A->br == A->bc && A->nbr == A->nbc, MGLDG_ERR_SHAPE, "coarse matrix must be square");
    const int n = A->nbr * A->br;
    MG_REQUIRE(n <= 4096, MGLDG_ERR_UNSUPPORTED, "dense coarsest solve limited to 4096 unknowns");
    double* aug = nullptr;
    int* dstatus = nullptr;
    int* absent = nullptr;
    try {
        aug = dalloc<double>((size_t)n * 2 * n);
        dstatus = dalloc<int>(1);
        absent = dalloc<int>(n);
        MG_CHECK_CUDA(cudaMemsetAsync(aug, 0, (size_t)n * 2 * n * sizeof(double), ctx->stream));
        MG_CHECK_CUDA(cudaMemsetAsync(dstatus, 0, sizeof(int), ctx->stream));
        {
            Launch L(ctx, MGLDG_K_SETUP);
            k_scatter_dense<<<std::min(A->nbr, 1024), 256, 0, ctx->stream>>>(A->nbr, A->br, A->row_ptr, A->col_idx,
                                                                             A->val, A->blk, n, aug);
        }
        {
            Launch L(ctx, MGLDG_K_SETUP);
            k_identity_right<<<std::min(n, 1024), 256, 0, ctx->stream>>>(n, aug);
        }
        {
            Launch L(ctx, MGLDG_K_SETUP);
            k_mark_absent<<<(n + 7) / 8, 256, 0, ctx->stream>>>(n, aug, absent);
        }
        if (n <= 128) {
            Launch L(ctx, MGLDG_K_SETUP);
            k_gauss_jordan<<<1, 1024, 0, ctx->stream>>>(n, aug, dstatus);
        } else {
            double* f = dalloc<double>(n);
            try {
                const dim3 grid((unsigned)std::min(8, (2 * n + 255) / 256), (unsigned)std::min(n, ctx->sm_count * 8));
                Launch L(ctx, MGLDG_K_SETUP);
                for (int k = 0; k < n; ++k) {
                    k_gj_pivot<<<1, 1024, 0, ctx->stream>>>(n, k, aug, f, dstatus);
                    k_gj_eliminate<<<grid, 256, 0, ctx->stream>>>(n, k, aug, f);
                }
                check_launch();
                ctx->launches[MGLDG_K_SETUP] += 2 * (int64_t)n - 1;
                ctx->lv_launches[MGLDG_K_SETUP][L.lv] += 2 * (int64_t)n - 1;
            } catch (...) {
                dfree(f);
                throw;
            }
            sync(ctx);
            dfree(f);
        }
        {
            Launch L(ctx, MGLDG_K_SETUP);
            k_extract_right<<<std::min(n, 1024), 256, 0, ctx->stream>>>(n, aug, absent, out_inv);
        }
        check_launch();
        int h = 0;
        download(ctx, &h, dstatus, 1);
        sync(ctx);
        MG_REQUIRE(h == 0, MGLDG_ERR_NOT_SPD, "coarsest-level matrix is singular");
    } catch (...) {
        dfree(aug);
        dfree(dstatus);
        dfree(absent);
        throw;
    }
    dfree(aug);
    dfree(dstatus);
    dfree(absent);
}

}  // namespace mg

mgldg_ops::~mgldg_ops() {
    delete M;
    for (auto* g : G) delete g;
    delete T;
    delete A;
}

// ================================================================== C ABI ==
extern "C" int mgldg_ops_create(mgldg_ctx* ctx, int ndim, mgldg_bsr* M, mgldg_bsr* const* G, mgldg_bsr* T,
                                mgldg_ops** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(out && M && G && T && ndim >= 1 && ndim <= 3, MGLDG_ERR_ARG, "bad operator arguments");
    *out = nullptr;
    const int b = M->br;
    MG_REQUIRE(M->bc == b && T->br == b && T->bc == b && M->nbr == M->nbc && T->nbr == M->nbr && T->nbc == M->nbr,
               MGLDG_ERR_SHAPE, "M and T must be square with equal blocks");
    for (int d = 0; d < ndim; ++d) {
        MG_REQUIRE(G[d] != nullptr, MGLDG_ERR_ARG, "null gradient");
        MG_REQUIRE(G[d]->br == b && G[d]->bc == b && G[d]->nbr == M->nbr && G[d]->nbc == M->nbr, MGLDG_ERR_SHAPE,
                   "gradient shape mismatch");
    }
    mgldg_ops* o = new mgldg_ops();
    o->ctx = ctx;
    o->ndim = ndim;
    o->M = M;
    for (int d = 0; d < ndim; ++d) o->G[d] = G[d];
    o->T = T;
    *out = o;
    MG_API_END
}

extern "C" int mgldg_ops_create_A(mgldg_ctx* ctx, mgldg_bsr* A, mgldg_ops** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(out && A, MGLDG_ERR_ARG, "bad operator arguments");
    MG_REQUIRE(A->br == A->bc && A->nbr == A->nbc, MGLDG_ERR_SHAPE, "A must be square");
    mgldg_ops* o = new mgldg_ops();
    o->ctx = ctx;
    o->ndim = 0;
    o->A = A;
    *out = o;
    MG_API_END
}

extern "C" int mgldg_ops_construct_laplacian(mgldg_ctx* ctx, mgldg_ops* ops) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(ops != nullptr, MGLDG_ERR_ARG, "null operators");
    construct_laplacian(ctx, ops);
    MG_API_END
}

extern "C" int mgldg_ops_get(const mgldg_ops* ops, int which, const mgldg_bsr** A) {
    if (!ops || !A) return MGLDG_ERR_ARG;
    switch (which) {
        case 0: *A = ops->M; break;
        case 1: *A = ops->G[0]; break;
        case 2: *A = ops->G[1]; break;
        case 3: *A = ops->T; break;
        case 4: *A = ops->A; break;
        case 5: *A = ops->G[2]; break;
        default: return MGLDG_ERR_ARG;
    }
    return *A ? MGLDG_OK : MGLDG_ERR_ARG;
}

extern "C" int mgldg_ops_destroy(mgldg_ops* ops) {
    if (!ops) return MGLDG_OK;
    if (ops->ctx) cudaSetDevice(ops->ctx->device);
    delete ops;
    return MGLDG_OK;
}

// bsr.cu -- context, profiling, block-sparse (BSR) storage and SpMV.
//
// Replaces the reference's SparseBlockMatrix<P,Q> (hash map of dense blocks,
// src/cartesian/util/sparseblockmatrix.h:62-165) and its matrix-vector
// routines (sparseblockmatrix.tpp:288-371) by block-CSR in HBM: row_ptr,
// sorted col_idx and row-major br x bc blocks stored contiguously per row.
//
// SpMV: one warp per block row; a block row's values are contiguous, so a
// warp streams them with 128-bit loads (when the block row is 16-byte
// aligned) and every lane owns a fixed chunk of columns of one block row.
// Partial sums are combined with warp shuffles.  Optional epilogues compute
// y = alpha*A*x + beta*yin and the partial dot product y.v per CTA (summed in
// a fixed order afterwards, so results are run-to-run reproducible).
#include <algorithm>
#include <type_traits>
#include <map>
#include <numeric>
#include <unordered_map>

#include "api.cuh"
#include "master_tables.inc"
#include "rowdot.cuh"

using namespace mg;

// ================================================================ context ==
namespace mg {

static int prof_slot(int level) { return level < 0 ? 0 : (level + 1 < kProfLevels ? level + 1 : kProfLevels - 1); }

Launch::Launch(mgldg_ctx* c, int kclass) : ctx(c), kc(kclass), lv(prof_slot(c->cur_level)) {
    ctx->launches[kc]++;
    ctx->lv_launches[kc][lv]++;
    if (ctx->prof) {
        if (ctx->event_pool.size() < 2) {
            for (int i = 0; i < 64; ++i) {
                cudaEvent_t e;
                MG_CHECK_CUDA(cudaEventCreate(&e));
                ctx->event_pool.push_back(e);
            }
        }
        a = ctx->event_pool.back(); ctx->event_pool.pop_back();
        b = ctx->event_pool.back(); ctx->event_pool.pop_back();
        cudaEventRecord(a, ctx->stream);
    }
}
Launch::~Launch() {
    if (a) {
        cudaEventRecord(b, ctx->stream);
        ctx->pending.push_back(ProfEvent{a, b, kc, lv});
        if (ctx->pending.size() > 4096) {
            try { prof_flush(ctx); } catch (...) {}
        }
    }
}
void prof_flush(mgldg_ctx* ctx) {
    if (ctx->pending.empty()) return;
    MG_CHECK_CUDA(cudaStreamSynchronize(ctx->stream));
    for (auto& p : ctx->pending) {
        float t = 0;
        if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) {
            ctx->ms[p.kclass] += t;
            ctx->lv_ms[p.kclass][p.level] += t;
        }
        ctx->event_pool.push_back(p.a);
        ctx->event_pool.push_back(p.b);
    }
    ctx->pending.clear();
}

}  // namespace mg

extern "C" int mgldg_ctx_create(int device, mgldg_ctx** out) {
    if (!out) return MGLDG_ERR_ARG;
    *out = nullptr;
    mgldg_ctx* ctx = new (std::nothrow) mgldg_ctx();
    if (!ctx) return MGLDG_ERR_NOMEM;
    ctx->device = device;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        delete ctx;
        return MGLDG_ERR_CUDA;
    }
    if (cudaSetDevice(device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) {
        delete ctx;
        return MGLDG_ERR_CUDA;
    }
    ctx->n_partials = 8192;
    if (cudaMalloc(&ctx->d_partials, ctx->n_partials * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&ctx->d_err, sizeof(unsigned)) != cudaSuccess ||
        cudaMemset(ctx->d_err, 0, sizeof(unsigned)) != cudaSuccess) {
        cudaFree(ctx->d_partials);
        cudaFree(ctx->d_err);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return MGLDG_ERR_NOMEM;
    }
    *out = ctx;
    return MGLDG_OK;
}

extern "C" int mgldg_ctx_destroy(mgldg_ctx* ctx) {
    if (!ctx) return MGLDG_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& p : ctx->pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
    for (auto e : ctx->event_pool) cudaEventDestroy(e);
    cudaFree(ctx->d_partials);
    cudaFree(ctx->d_err);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MGLDG_OK;
}

extern "C" const char* mgldg_last_error(const mgldg_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

extern "C" int mgldg_ctx_sync(mgldg_ctx* ctx) {
    MG_API_BEGIN(ctx)
    sync(ctx);
    MG_API_END
}

extern "C" void* mgldg_ctx_stream(mgldg_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

extern "C" int mgldg_master_tables(int P, double* nodes, double* denom, double* mass, double* invmass,
                                   double* diff, double* quad_x, double* quad_w) {
    if (P < 1 || P > MGLDG_PMAX) return MGLDG_ERR_ARG;
    for (int i = 0; i < P; ++i) {
        if (nodes) nodes[i] = kNodes[P - 1][i];
        if (denom) denom[i] = kDenom[P - 1][i];
    }
    for (int i = 0; i < P * P; ++i) {
        if (mass) mass[i] = kMass1[P - 1][i];
        if (invmass) invmass[i] = kInvMass1[P - 1][i];
        if (diff) diff[i] = kDiff1[P - 1][i];
    }
    for (int q = 0; q < MGLDG_QF; ++q) {
        if (quad_x) quad_x[q] = kQuadNodes[q];
        if (quad_w) quad_w[q] = kQuadWeights[q];
    }
    return MGLDG_OK;
}

extern "C" int mgldg_prof_enable(mgldg_ctx* ctx, int on) {
    MG_API_BEGIN(ctx)
    prof_flush(ctx);
    ctx->prof = on != 0;
    MG_API_END
}
extern "C" int mgldg_prof_reset(mgldg_ctx* ctx) {
    MG_API_BEGIN(ctx)
    prof_flush(ctx);
    for (int k = 0; k < MGLDG_K_NCLASS; ++k) {
        ctx->launches[k] = 0;
        ctx->ms[k] = 0;
        for (int l = 0; l < kProfLevels; ++l) {
            ctx->lv_launches[k][l] = 0;
            ctx->lv_ms[k][l] = 0;
        }
    }
    MG_API_END
}

extern "C" int mgldg_prof_query_level(mgldg_ctx* ctx, int kclass, int level, int64_t* launches, double* ms) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(kclass >= 0 && kclass < MGLDG_K_NCLASS && level >= -1 && level + 1 < kProfLevels, MGLDG_ERR_ARG,
               "bad kernel class or level");
    prof_flush(ctx);
    if (launches) *launches = ctx->lv_launches[kclass][level + 1];
    if (ms) *ms = ctx->lv_ms[kclass][level + 1];
    MG_API_END
}
extern "C" int mgldg_prof_query(mgldg_ctx* ctx, int kclass, int64_t* launches, double* ms) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(kclass >= 0 && kclass < MGLDG_K_NCLASS, MGLDG_ERR_ARG, "bad kernel class");
    prof_flush(ctx);
    if (launches) *launches = ctx->launches[kclass];
    if (ms) *ms = ctx->ms[kclass];
    MG_API_END
}

// =============================================================== reductions ==
namespace mg {

template <int NT>
__device__ double block_sum(double v, double* sm) {
    // fixed-order block reduction: shuffles inside warps, then warp 0
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sm[w] = v;
    __syncthreads();
    double t = 0;
    if (w == 0) {
        t = (l < NT / 32) ? sm[l] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    __syncthreads();
    return t;   // valid in thread 0
}

template <class T>
__global__ void __launch_bounds__(256) k_dot(int n, const T* __restrict__ a, const T* __restrict__ b,
                                             double* __restrict__ partials) {
    __shared__ double sm[8];
    double s = 0;
    for (int i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) s += (double)a[i] * (double)b[i];
    s = block_sum<256>(s, sm);
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_finish(const double* __restrict__ partials, int npart, double* out) {
    __shared__ double sm[8];
    double s = 0;
    for (int i = threadIdx.x; i < npart; i += 256) s += partials[i];
    s = block_sum<256>(s, sm);
    if (threadIdx.x == 0) *out = s;
}

int reduce_grid(int n) { return std::max(1, std::min(1024, (n + 255) / 256)); }

template <class T>
void dot_partials(mgldg_ctx* ctx, int n, const T* a, const T* b, double* partials, int* npart) {
    int g = reduce_grid(n);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_dot<T><<<g, 256, 0, ctx->stream>>>(n, a, b, partials);
    }
    check_launch();
    *npart = g;
}
template void dot_partials<double>(mgldg_ctx*, int, const double*, const double*, double*, int*);
template void dot_partials<float>(mgldg_ctx*, int, const float*, const float*, double*, int*);

void finish_sum(mgldg_ctx* ctx, const double* partials, int npart, double* out) {
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_finish<<<1, 256, 0, ctx->stream>>>(partials, npart, out);
    }
    check_launch();
}

// ==================================================================== SpMV ==
template <class T>
struct Vec16;
template <>
struct Vec16<double> { typedef double2 type; static constexpr int n = 2; };
template <>
struct Vec16<float> { typedef float4 type; static constexpr int n = 4; };

// Accumulates the lane's chunk of (block row r) . (x chunk).
template <class T, int BR, int BC>
__device__ __forceinline__ T chunk_dot(const T* __restrict__ a, const T* __restrict__ xj, int r, int c0) {
    using L = WL<BR, BC>;
    T acc = 0;
    constexpr bool vec = ((BC * sizeof(T)) % 16 == 0) && ((L::CH * sizeof(T)) % 16 == 0) &&
                         (L::CH * L::S == BC);
    if constexpr (vec) {
        typedef typename Vec16<T>::type V;
        constexpr int NV = L::CH * sizeof(T) / 16;
        const V* av = reinterpret_cast<const V*>(a + r * BC + c0);
        const V* xv = reinterpret_cast<const V*>(xj + c0);
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            V u = __ldg(av + q);
            V w = __ldg(xv + q);
            if constexpr (sizeof(T) == 8) {
                acc += u.x * w.x;
                acc += u.y * w.y;
            } else {
                acc += u.x * w.x;
                acc += u.y * w.y;
                acc += u.z * w.z;
                acc += u.w * w.w;
            }
        }
    } else {
#pragma unroll
        for (int c = 0; c < L::CH; ++c)
            if (c0 + c < BC) acc += __ldg(a + r * BC + c0 + c) * __ldg(xj + c0 + c);
    }
    return acc;
}

template <class T, int BR, int BC, int WPB>
__global__ void __launch_bounds__(WPB * 32, 2)
    k_spmv(int nbr, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
           const T* __restrict__ val, const int* __restrict__ blk, T alpha, const T* __restrict__ x, T beta,
           const T* yin, T* y, const T* dotv, int self_dot, double* __restrict__ partials) {
    using L = WL<BR, BC>;
    __shared__ double sm[WPB];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = lane / L::S, s = lane - r * L::S;
    const bool active = r < BR;
    const int c0 = s * L::CH;
    double dacc = 0;
    for (int row = blockIdx.x * WPB + warp; row < nbr; row += gridDim.x * WPB) {
        const int k0 = __ldg(row_ptr + row), k1 = __ldg(row_ptr + row + 1);
        T acc = row_product<T, BR, BC>(col_idx, val, blk, x, k0, k1, r, c0, active, lane);
        acc = seg_sum<L::S>(acc);
        if (active && s == 0) {
            const size_t o = (size_t)row * BR + r;
            T v = alpha * acc;
            if (beta != T(0)) v += beta * yin[o];
            y[o] = v;
            if (self_dot) dacc += (double)v * (double)v;
            else if (dotv) dacc += (double)v * (double)dotv[o];
        }
    }
    if (partials) {
        // fixed-order CTA sum of the dot epilogue
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dacc += __shfl_xor_sync(0xffffffffu, dacc, o);
        if (lane == 0) sm[warp] = dacc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int w = 0; w < WPB; ++w) t += sm[w];
            partials[blockIdx.x] = t;
        }
    }
}

// Small square blocks (3..10): 32 / B block rows per warp, one lane per
// block column (cols_accumulate, rows_reduce); the same epilogue and CTA
// partials as k_spmv.  (The transfers' rectangular blocks, 6x9 and 9x6 on
// triangles, ran slower this way than one thread per output entry: one
// block per prolongation row leaves the reduction unamortised.)
template <class T, class VT, int BR, int BC, int MAXB>
__global__ void __launch_bounds__(256)
    k_spmv_rows(int nbr, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                const VT* __restrict__ val, const float* __restrict__ scl, const int* __restrict__ blk, T alpha,
                const T* __restrict__ x, T beta, const T* yin, T* y, const T* dotv, int self_dot,
                double* __restrict__ partials) {
    using R = Rows<BR, BC>;
    __shared__ T sr[8 * R::SM];
    __shared__ double sm[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane / R::S, c = lane - g * R::S;
    T* s = sr + warp * R::SM;
    double dacc = 0;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int base = (blockIdx.x * (blockDim.x >> 5) + warp) * R::G; base < nbr; base += nw * R::G) {
        const int row = base + g;
        const bool valid = g < R::G && row < nbr;
        T acc[BR];
#pragma unroll
        for (int r = 0; r < BR; ++r) acc[r] = 0;
        if (valid && c < BC)
            cols_accumulate<T, VT, BR, BC, MAXB>(col_idx, val, scl, blk, x, __ldg(row_ptr + row),
                                                 __ldg(row_ptr + row + 1), c, acc);
        const T sum = rows_reduce<T, BR, BC>(acc, s, g, c, g < R::G);
        if (valid && c < BR) {
            const size_t o = (size_t)row * BR + c;
            T v = alpha * sum;
            if (beta != T(0)) v += beta * yin[o];
            y[o] = v;
            if (self_dot) dacc += (double)v * (double)v;
            else if (dotv) dacc += (double)v * (double)dotv[o];
        }
    }
    if (partials) {
        dacc = block_sum<256>(dacc, sm);
        if (threadIdx.x == 0) partials[blockIdx.x] = dacc;
    }
}

template <class T, int BR, int BC, class VT = T>
static void launch_spmv_rows(mgldg_ctx* ctx, const mgldg_bsr* A, T alpha, const T* x, T beta, const T* yin, T* y,
                             const T* dotv, double* partials, int* npart, int kclass, const VT* vals = nullptr,
                             const float* scl = nullptr) {
    constexpr int B = BR > BC ? BR : BC;
    constexpr int MAXB = sizeof(T) == 4 ? (BR <= 10 ? 4 : 2) : (B <= 4 ? 4 : (BR <= 10 ? 2 : 1));
    const int rows_per_cta = 8 * Rows<BR, BC>::G;
    int grid = std::max(1, std::min((A->nbr + rows_per_cta - 1) / rows_per_cta, ctx->sm_count * 8));
    if (partials) grid = std::min(grid, ctx->n_partials);
    {
        Launch L(ctx, kclass);
        const int self_dot = (dotv != nullptr && dotv == y) ? 1 : 0;
        k_spmv_rows<T, VT, BR, BC, MAXB><<<grid, 256, 0, ctx->stream>>>(
            A->nbr, A->row_ptr, A->col_idx, vals ? vals : (const VT*)bsr_vals<T>(A), scl, A->blk, alpha, x, beta, yin,
            y, self_dot ? nullptr : dotv, self_dot, partials);
    }
    check_launch();
    if (npart) *npart = grid;
}

// Any block shape: one thread per output row entry.
template <class T>
__global__ void __launch_bounds__(256)
    k_spmv_generic(int nbr, int br, int bc, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
                   const T* __restrict__ val, const int* __restrict__ blk, T alpha, const T* __restrict__ x,
                   T beta, const T* yin, T* y, const T* dotv, int self_dot, double* __restrict__ partials) {
    __shared__ double sm[8];
    double dacc = 0;
    const int64_t n = (int64_t)nbr * br;
    for (int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x; t < n; t += (int64_t)gridDim.x * 256) {
        const int row = (int)(t / br), r = (int)(t - (int64_t)row * br);
        T acc = 0;
        for (int k = row_ptr[row]; k < row_ptr[row + 1]; ++k) {
            const T* a = val + (size_t)(blk ? blk[k] : k) * br * bc + (size_t)r * bc;
            const T* xj = x + (size_t)col_idx[k] * bc;
            for (int c = 0; c < bc; ++c) acc += a[c] * xj[c];
        }
        T v = alpha * acc;
        if (beta != T(0)) v += beta * yin[t];
        y[t] = v;
        if (self_dot) dacc += (double)v * (double)v;
        else if (dotv) dacc += (double)v * (double)dotv[t];
    }
    if (partials) {
        dacc = block_sum<256>(dacc, sm);
        if (threadIdx.x == 0) partials[blockIdx.x] = dacc;
    }
}

// Interpolation-type operators (restriction T^T, prolongation T): a handful
// of distinct blocks and one to four blocks per row.  One thread per output
// entry; the block table is staged in shared memory with rows padded to
// BC+1 values (conflict-free across the BR rows of a block).
template <class T, int BR, int BC>
__global__ void __launch_bounds__(256)
    k_transfer(int nbr, const int* __restrict__ row_ptr, const int* __restrict__ col_idx,
               const T* __restrict__ table, int ntab, const int* __restrict__ blk, T alpha,
               const T* __restrict__ x, T beta, const T* yin, T* y) {
    extern __shared__ unsigned char smraw[];
    T* st = reinterpret_cast<T*>(smraw);
    constexpr int LD = BC + 1;
    for (int q = threadIdx.x; q < ntab * BR * BC; q += 256) {
        const int b = q / (BR * BC), e = q - b * (BR * BC);
        const int rr = e / BC, cc = e - rr * BC;
        st[(b * BR + rr) * LD + cc] = table[q];
    }
    __syncthreads();
    const int64_t n = (int64_t)nbr * BR;
    for (int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x; t < n; t += (int64_t)gridDim.x * 256) {
        const int row = (int)(t / BR), r = (int)(t - (int64_t)row * BR);
        T acc = 0;
        const int k0 = __ldg(row_ptr + row), k1 = __ldg(row_ptr + row + 1);
        for (int k = k0; k < k1; ++k) {
            const T* a = st + (__ldg(blk + k) * BR + r) * LD;
            const T* xj = x + (size_t)__ldg(col_idx + k) * BC;
#pragma unroll
            for (int c = 0; c < BC; ++c) acc = fma(a[c], __ldg(xj + c), acc);
        }
        T v = alpha * acc;
        if (beta != T(0)) v += beta * yin[t];
        y[t] = v;
    }
}

template <class T, int BR, int BC>
static bool launch_transfer(mgldg_ctx* ctx, const mgldg_bsr* A, T alpha, const T* x, T beta, const T* yin, T* y,
                            int kclass) {
    const size_t smem = (size_t)A->nuniq * BR * (BC + 1) * sizeof(T);
    if (smem > 48 * 1024) return false;
    const int64_t n = (int64_t)A->nbr * BR;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, ctx->sm_count * 16));
    {
        Launch L(ctx, kclass);
        k_transfer<T, BR, BC><<<grid, 256, smem, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, bsr_vals<T>(A),
                                                                (int)A->nuniq, A->blk, alpha, x, beta, yin, y);
    }
    check_launch();
    return true;
}

template <>
const double* bsr_vals<double>(const mgldg_bsr* A) { return A->val; }
template <>
const float* bsr_vals<float>(const mgldg_bsr* A) {
    MG_REQUIRE(A->val32 != nullptr, MGLDG_ERR_ARG, "FP32 values not built");
    return A->val32;
}

template <class T, int BR, int BC>
static void launch_spmv(mgldg_ctx* ctx, const mgldg_bsr* A, T alpha, const T* x, T beta, const T* yin, T* y,
                        const T* dotv, double* partials, int* npart, int kclass) {
    constexpr int WPB = 8;
    int grid = std::max(1, std::min((A->nbr + WPB - 1) / WPB, ctx->sm_count * 16));
    if (partials) grid = std::min(grid, ctx->n_partials);
    {
        Launch L(ctx, kclass);
        const int self_dot = (dotv != nullptr && dotv == y) ? 1 : 0;
        k_spmv<T, BR, BC, WPB><<<grid, WPB * 32, 0, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, bsr_vals<T>(A),
                                                                   A->blk, alpha, x, beta, yin, y,
                                                                   self_dot ? nullptr : dotv, self_dot, partials);
    }
    check_launch();
    if (npart) *npart = grid;
}

template <class T>
void spmv(mgldg_ctx* ctx, const mgldg_bsr* A, T alpha, const T* x, T beta, const T* yin, T* y, const T* dotv,
          double* partials, int* npart, int kclass) {
    if (A->nbr == 0) {
        if (npart) *npart = 0;
        return;
    }
    const int br = A->br, bc = A->bc;
    // FP32 16x16 products without a dot epilogue: bulk-copy pipeline
    if constexpr (std::is_same<T, float>::value) {
        if (!dotv && !partials && bulk_spmv_f32(ctx, A, alpha, x, beta, yin, y, kclass)) {
            if (npart) *npart = 0;
            return;
        }
    }
    // operators stored as a small block table (interpolation on quadtrees)
    if (A->blk && !dotv && !partials && A->nuniq <= 16) {
#define MG_TRANSFER_CASE(R)                                                                            \
        if (br == R && bc == R && launch_transfer<T, R, R>(ctx, A, alpha, x, beta, yin, y, kclass)) {  \
            if (npart) *npart = 0;                                                                     \
            return;                                                                                    \
        }
        MG_TRANSFER_CASE(4)
        MG_TRANSFER_CASE(9)
        MG_TRANSFER_CASE(16)
        MG_TRANSFER_CASE(25)
#undef MG_TRANSFER_CASE
    }
#define MG_SPMV_ROWS_CASE(R, Cc)                                                                       \
    if (br == R && bc == Cc) {                                                                         \
        launch_spmv_rows<T, R, Cc>(ctx, A, alpha, x, beta, yin, y, dotv, partials, npart, kclass);     \
        return;                                                                                        \
    }
    MG_SPMV_ROWS_CASE(3, 3)
    MG_SPMV_ROWS_CASE(4, 4)
    MG_SPMV_ROWS_CASE(6, 6)
    MG_SPMV_ROWS_CASE(8, 8)
    MG_SPMV_ROWS_CASE(9, 9)
    MG_SPMV_ROWS_CASE(10, 10)
#undef MG_SPMV_ROWS_CASE
#define MG_SPMV_CASE(R, Cc)                                                                            \
    if (br == R && bc == Cc) {                                                                         \
        launch_spmv<T, R, Cc>(ctx, A, alpha, x, beta, yin, y, dotv, partials, npart, kclass);          \
        return;                                                                                        \
    }
    MG_SPMV_CASE(1, 1)
    MG_SPMV_CASE(3, 3)
    MG_SPMV_CASE(4, 4)
    MG_SPMV_CASE(6, 6)
    MG_SPMV_CASE(8, 8)
    MG_SPMV_CASE(9, 9)
    MG_SPMV_CASE(10, 10)
    MG_SPMV_CASE(16, 16)
    MG_SPMV_CASE(25, 25)
    MG_SPMV_CASE(27, 27)
#undef MG_SPMV_CASE
    int grid = (int)std::max<int64_t>(1, std::min<int64_t>(((int64_t)A->nbr * br + 255) / 256, ctx->sm_count * 8));
    if (partials) grid = std::min(grid, ctx->n_partials);
    {
        Launch L(ctx, kclass);
        const int self_dot = (dotv != nullptr && dotv == y) ? 1 : 0;
        k_spmv_generic<T><<<grid, 256, 0, ctx->stream>>>(A->nbr, br, bc, A->row_ptr, A->col_idx, bsr_vals<T>(A),
                                                         A->blk, alpha, x, beta, yin, y, self_dot ? nullptr : dotv,
                                                         self_dot, partials);
    }
    check_launch();
    if (npart) *npart = grid;
}
template void spmv<double>(mgldg_ctx*, const mgldg_bsr*, double, const double*, double, const double*, double*,
                           const double*, double*, int*, int);
template void spmv<float>(mgldg_ctx*, const mgldg_bsr*, float, const float*, float, const float*, float*,
                          const float*, double*, int*, int);

// ============================================================ BSR storage ==
mgldg_bsr* bsr_new(mgldg_ctx* ctx, int nbr, int nbc, int br, int bc, const std::vector<int>& row_ptr,
                   const std::vector<int>& col_idx) {
    mgldg_bsr* A = new mgldg_bsr();
    A->ctx = ctx;
    A->nbr = nbr; A->nbc = nbc; A->br = br; A->bc = bc;
    A->h_row_ptr = row_ptr;
    A->h_col_idx = col_idx;
    A->nnzb = (int64_t)col_idx.size();
    try {
        A->row_ptr = dalloc<int>(nbr + 1);
        // four spare entries: bulk copies of index runs move whole 16-byte words
        A->col_idx = dalloc<int>(col_idx.size() + 4);
        A->val = dalloc<double>(std::max<size_t>(1, col_idx.size() * A->bsz()));
        upload(ctx, A->row_ptr, row_ptr.data(), row_ptr.size());
        upload(ctx, A->col_idx, col_idx.data(), col_idx.size());
    } catch (...) {
        delete A;
        throw;
    }
    return A;
}

void bsr_build_diag(mgldg_bsr* A) {
    if (A->diag) return;
    A->h_diag.assign(A->nbr, -1);
    for (int i = 0; i < A->nbr; ++i)
        for (int k = A->h_row_ptr[i]; k < A->h_row_ptr[i + 1]; ++k)
            if (A->h_col_idx[k] == i) A->h_diag[i] = k;
    A->diag = dalloc<int>(std::max(1, A->nbr));
    upload(A->ctx, A->diag, A->h_diag.data(), A->h_diag.size());
}

__global__ void k_to_fp32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) b[i] = (float)a[i];
}

void bsr_ensure_fp32(mgldg_bsr* A) {
    if (A->val32) return;
    int64_t n = A->nvals_blocks() * (int64_t)A->bsz();
    A->val32 = dalloc<float>(std::max<int64_t>(1, n));
    if (n) {
        int g = (int)std::min<int64_t>((n + 255) / 256, A->ctx->sm_count * 32);
        Launch L(A->ctx, MGLDG_K_SETUP);
        k_to_fp32<<<g, 256, 0, A->ctx->stream>>>(n, A->val, A->val32);
    }
    check_launch();
}

bool spmv_f16(mgldg_ctx* ctx, const mgldg_bsr* A, float alpha, const float* x, float beta, const float* yin, float* y,
              int kclass) {
    if (!A->val16 || A->nbr == 0 || !f16_shape(A->br, A->bc)) return false;
    return bulk_spmv_f16(ctx, A, alpha, x, beta, yin, y, kclass);
}

__global__ void k_to_lo32(int64_t n, const double* __restrict__ a, float* __restrict__ lo) {
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
        const double v = a[i];
        lo[i] = (float)(v - (double)(float)v);
    }
}

void bsr_ensure_lo32(mgldg_bsr* A) {
    if (A->lo32) return;
    const int64_t n = A->nvals_blocks() * (int64_t)A->bsz();
    A->lo32 = dalloc<float>(std::max<int64_t>(1, n));
    if (n) {
        const int g = (int)std::min<int64_t>((n + 255) / 256, A->ctx->sm_count * 32);
        Launch L(A->ctx, MGLDG_K_SETUP);
        k_to_lo32<<<g, 256, 0, A->ctx->stream>>>(n, A->val, A->lo32);
    }
    check_launch();
}

// one thread per block: scale = largest magnitude, entries / scale in FP16
__global__ void k_to_f16(int64_t nblk, int bsz, const double* __restrict__ a, __half* __restrict__ h,
                         float* __restrict__ scale) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < nblk; k += (int64_t)gridDim.x * blockDim.x) {
        const double* ak = a + k * bsz;
        double m = 0;
        for (int e = 0; e < bsz; ++e) m = fmax(m, fabs(ak[e]));
        const double s = m > 0 ? m : 1.0;
        scale[k] = (float)s;
        for (int e = 0; e < bsz; ++e) h[k * bsz + e] = __float2half_rn((float)(ak[e] / s));
    }
}

void bsr_ensure_f16(mgldg_bsr* A) {
    if (A->val16) return;
    const int64_t nb = A->nvals_blocks();
    A->val16 = dalloc<__half>(std::max<int64_t>(1, nb * (int64_t)A->bsz()));
    A->scale16 = dalloc<float>(nb + 4);
    MG_CHECK_CUDA(cudaMemsetAsync(A->scale16, 0, (nb + 4) * sizeof(float), A->ctx->stream));
    if (nb) {
        const int g = (int)std::min<int64_t>((nb + 255) / 256, A->ctx->sm_count * 32);
        Launch L(A->ctx, MGLDG_K_SETUP);
        k_to_f16<<<g, 256, 0, A->ctx->stream>>>(nb, (int)A->bsz(), A->val, A->val16, A->scale16);
    }
    check_launch();
}

}  // namespace mg

mgldg_bsr::~mgldg_bsr() {
    dfree(row_ptr);
    dfree(col_idx);
    dfree(val);
    dfree(val32);
    dfree(val16);
    dfree(scale16);
    dfree(lo32);
    dfree(blk);
    dfree(diag);
}

namespace mg {

__global__ void k_transpose_blocks(int64_t n, int br, int bc, const int* __restrict__ src, const double* __restrict__ in,
                                   double* __restrict__ out) {
    // out block p (bc x br) = transpose of in block src[p] (br x bc)
    const int64_t bs = (int64_t)br * bc;
    for (int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x; t < n * bs; t += (int64_t)gridDim.x * 256) {
        int64_t p = t / bs;
        int e = (int)(t - p * bs);
        int rr = e / br, cc = e - rr * br;   // out(rr, cc) = in(cc, rr)
        int64_t s = src ? src[p] : p;
        out[t] = in[s * bs + (int64_t)cc * bc + rr];
    }
}

mgldg_bsr* bsr_transpose(mgldg_ctx* ctx, const mgldg_bsr* A) {
    std::vector<int> cnt(A->nbc + 1, 0);
    for (int64_t k = 0; k < A->nnzb; ++k) cnt[A->h_col_idx[k] + 1]++;
    for (int j = 0; j < A->nbc; ++j) cnt[j + 1] += cnt[j];
    std::vector<int> rp(cnt), ci(A->nnzb), src(A->nnzb);
    std::vector<int> pos(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < A->nbr; ++i)
        for (int k = A->h_row_ptr[i]; k < A->h_row_ptr[i + 1]; ++k) {
            int j = A->h_col_idx[k];
            int p = pos[j]++;
            ci[p] = i;
            src[p] = k;
        }
    mgldg_bsr* B = nullptr;
    if (A->blk) {
        // transpose the distinct-block table; permute the indirection
        B = new mgldg_bsr();
        B->ctx = ctx;
        B->nbr = A->nbc; B->nbc = A->nbr; B->br = A->bc; B->bc = A->br;
        B->h_row_ptr = rp; B->h_col_idx = ci; B->nnzb = A->nnzb; B->nuniq = A->nuniq;
        B->h_blk.resize(A->nnzb);
        for (int64_t p = 0; p < A->nnzb; ++p) B->h_blk[p] = A->h_blk[src[p]];
        try {
            B->row_ptr = dalloc<int>(B->nbr + 1);
            B->col_idx = dalloc<int>(B->nnzb + 4);
            B->blk = dalloc<int>(std::max<int64_t>(1, B->nnzb));
            B->val = dalloc<double>(std::max<int64_t>(1, A->nuniq * (int64_t)A->bsz()));
            upload(ctx, B->row_ptr, rp.data(), rp.size());
            upload(ctx, B->col_idx, ci.data(), ci.size());
            upload(ctx, B->blk, B->h_blk.data(), B->h_blk.size());
            if (A->nuniq) {
                int g = (int)std::min<int64_t>((A->nuniq * (int64_t)A->bsz() + 255) / 256, ctx->sm_count * 32);
                Launch L(ctx, MGLDG_K_SETUP);
                k_transpose_blocks<<<g, 256, 0, ctx->stream>>>(A->nuniq, A->br, A->bc, nullptr, A->val, B->val);
            }
            check_launch();
        } catch (...) {
            delete B;
            throw;
        }
        return B;
    }
    B = bsr_new(ctx, A->nbc, A->nbr, A->bc, A->br, rp, ci);
    int* dsrc = nullptr;
    try {
        dsrc = dalloc<int>(std::max<int64_t>(1, A->nnzb));
        upload(ctx, dsrc, src.data(), src.size());
        if (A->nnzb) {
            int g = (int)std::min<int64_t>((A->nnzb * (int64_t)A->bsz() + 255) / 256, ctx->sm_count * 32);
            Launch L(ctx, MGLDG_K_SETUP);
            k_transpose_blocks<<<g, 256, 0, ctx->stream>>>(A->nnzb, A->br, A->bc, dsrc, A->val, B->val);
        }
        check_launch();
        sync(ctx);
    } catch (...) {
        dfree(dsrc);
        delete B;
        throw;
    }
    dfree(dsrc);
    return B;
}

void bsr_dedupe(mgldg_ctx* ctx, mgldg_bsr* A) {
    if (A->blk) return;
    const size_t bs = A->bsz();
    // operators whose blocks are mostly distinct (transfers of unstructured
    // hierarchies) are left as they are: look at a sample first
    {
        const int64_t ns = std::min<int64_t>(A->nnzb, 4096);
        std::vector<double> hs((size_t)ns * bs);
        download(ctx, hs.data(), A->val, hs.size());
        sync(ctx);
        std::unordered_map<std::string, int> sample;
        for (int64_t k = 0; k < ns; ++k)
            sample.emplace(std::string((const char*)(hs.data() + k * bs), bs * sizeof(double)), 0);
        if (A->nnzb > 64 && (int64_t)sample.size() * 4 > ns) return;
    }
    std::vector<double> h((size_t)A->nnzb * bs);
    download(ctx, h.data(), A->val, h.size());
    sync(ctx);
    std::unordered_map<std::string, int> seen;
    std::vector<double> table;
    A->h_blk.resize(A->nnzb);
    for (int64_t k = 0; k < A->nnzb; ++k) {
        std::string key((const char*)(h.data() + k * bs), bs * sizeof(double));
        auto it = seen.find(key);
        int id;
        if (it == seen.end()) {
            id = (int)seen.size();
            seen.emplace(std::move(key), id);
            table.insert(table.end(), h.begin() + k * bs, h.begin() + (k + 1) * bs);
        } else {
            id = it->second;
        }
        A->h_blk[k] = id;
    }
    A->nuniq = (int64_t)seen.size();
    int* dblk = dalloc<int>(std::max<int64_t>(1, A->nnzb));
    double* dval = nullptr;
    try {
        dval = dalloc<double>(std::max<size_t>(1, table.size()));
        upload(ctx, dblk, A->h_blk.data(), A->h_blk.size());
        upload(ctx, dval, table.data(), table.size());
        sync(ctx);
    } catch (...) {
        dfree(dblk);
        dfree(dval);
        throw;
    }
    dfree(A->val);
    dfree(A->val32);
    A->val = dval;
    A->blk = dblk;
}

mgldg_bsr* bsr_clone(mgldg_ctx* ctx, const mgldg_bsr* A) {
    mgldg_bsr* B = bsr_new(ctx, A->nbr, A->nbc, A->br, A->bc, A->h_row_ptr, A->h_col_idx);
    try {
        if (A->blk) {
            dfree(B->val);
            B->nuniq = A->nuniq;
            B->h_blk = A->h_blk;
            B->blk = dalloc<int>(std::max<int64_t>(1, A->nnzb));
            B->val = dalloc<double>(std::max<int64_t>(1, A->nuniq * (int64_t)A->bsz()));
            upload(ctx, B->blk, A->h_blk.data(), A->h_blk.size());
        }
        size_t n = (size_t)A->nvals_blocks() * A->bsz();
        if (n) MG_CHECK_CUDA(cudaMemcpyAsync(B->val, A->val, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    } catch (...) {
        delete B;
        throw;
    }
    return B;
}

}  // namespace mg

// ================================================================== C ABI ==
extern "C" int mgldg_bsr_clone(mgldg_ctx* ctx, const mgldg_bsr* A, mgldg_bsr** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && out, MGLDG_ERR_ARG, "null argument");
    *out = nullptr;
    *out = bsr_clone(ctx, A);
    sync(ctx);
    MG_API_END
}

extern "C" int mgldg_bsr_create(mgldg_ctx* ctx, int nbr, int nbc, int br, int bc, const int* row_ptr,
                                const int* col_idx, const double* vals, mgldg_bsr** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(out && row_ptr && nbr >= 0 && nbc >= 0 && br >= 1 && bc >= 1, MGLDG_ERR_ARG, "bad BSR arguments");
    *out = nullptr;
    MG_REQUIRE(row_ptr[0] == 0, MGLDG_ERR_ARG, "row_ptr[0] must be 0");
    for (int i = 0; i < nbr; ++i) MG_REQUIRE(row_ptr[i + 1] >= row_ptr[i], MGLDG_ERR_ARG, "row_ptr not monotone");
    const int64_t nnz_in = row_ptr[nbr];
    MG_REQUIRE(nnz_in == 0 || (col_idx && vals), MGLDG_ERR_ARG, "missing col_idx/vals");
    const size_t bs = (size_t)br * bc;
    // sort each row by column and sum duplicates (addToBlock semantics)
    std::vector<int> rp(nbr + 1, 0), ci;
    std::vector<double> v;
    ci.reserve(nnz_in);
    v.reserve(nnz_in * bs);
    std::vector<std::pair<int, int64_t>> row;
    for (int i = 0; i < nbr; ++i) {
        row.clear();
        for (int64_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            MG_REQUIRE(col_idx[k] >= 0 && col_idx[k] < nbc, MGLDG_ERR_ARG, "column index out of range");
            row.push_back({col_idx[k], k});
        }
        std::stable_sort(row.begin(), row.end(),
                         [](const std::pair<int, int64_t>& a, const std::pair<int, int64_t>& b) { return a.first < b.first; });
        for (size_t q = 0; q < row.size(); ++q) {
            const double* src = vals + row[q].second * bs;
            if (q > 0 && row[q].first == row[q - 1].first) {
                double* dst = v.data() + (ci.size() - 1) * bs;
                for (size_t e = 0; e < bs; ++e) dst[e] += src[e];
            } else {
                ci.push_back(row[q].first);
                v.insert(v.end(), src, src + bs);
            }
        }
        rp[i + 1] = (int)ci.size();
    }
    mgldg_bsr* A = bsr_new(ctx, nbr, nbc, br, bc, rp, ci);
    try {
        upload(ctx, A->val, v.data(), v.size());
        sync(ctx);
    } catch (...) {
        delete A;
        throw;
    }
    *out = A;
    MG_API_END
}

extern "C" int mgldg_bsr_destroy(mgldg_bsr* A) {
    if (!A) return MGLDG_OK;
    if (A->ctx) cudaSetDevice(A->ctx->device);
    delete A;
    return MGLDG_OK;
}

extern "C" int mgldg_bsr_info(const mgldg_bsr* A, int* nbr, int* nbc, int* br, int* bc, int64_t* nnzb) {
    if (!A) return MGLDG_ERR_ARG;
    if (nbr) *nbr = A->nbr;
    if (nbc) *nbc = A->nbc;
    if (br) *br = A->br;
    if (bc) *bc = A->bc;
    if (nnzb) *nnzb = A->nnzb;
    return MGLDG_OK;
}

extern "C" int mgldg_bsr_download(mgldg_ctx* ctx, const mgldg_bsr* A, int* row_ptr, int* col_idx, double* vals) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A != nullptr, MGLDG_ERR_ARG, "null matrix");
    if (row_ptr) std::memcpy(row_ptr, A->h_row_ptr.data(), A->h_row_ptr.size() * sizeof(int));
    if (col_idx) std::memcpy(col_idx, A->h_col_idx.data(), A->h_col_idx.size() * sizeof(int));
    if (vals) {
        const size_t bs = A->bsz();
        if (A->blk) {
            std::vector<double> table((size_t)A->nuniq * bs);
            download(ctx, table.data(), A->val, table.size());
            sync(ctx);
            for (int64_t k = 0; k < A->nnzb; ++k)
                std::memcpy(vals + k * bs, table.data() + (size_t)A->h_blk[k] * bs, bs * sizeof(double));
        } else {
            download(ctx, vals, A->val, (size_t)A->nnzb * bs);
            sync(ctx);
        }
    }
    MG_API_END
}

extern "C" int mgldg_bsr_mv_dev(mgldg_ctx* ctx, double alpha, const mgldg_bsr* A, const double* x, double beta,
                                double* y) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && x && y, MGLDG_ERR_ARG, "null argument");
    spmv<double>(ctx, A, alpha, x, beta, y, y);
    MG_API_END
}

extern "C" int mgldg_bsr_mv(mgldg_ctx* ctx, double alpha, const mgldg_bsr* A, const double* x, double beta,
                            double* y) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && x && y, MGLDG_ERR_ARG, "null argument");
    size_t nx = (size_t)A->nbc * A->bc, ny = (size_t)A->nbr * A->br;
    double *dx = nullptr, *dy = nullptr;
    try {
        dx = dalloc<double>(std::max<size_t>(1, nx));
        dy = dalloc<double>(std::max<size_t>(1, ny));
        upload(ctx, dx, x, nx);
        if (beta != 0.0) upload(ctx, dy, y, ny);
        spmv<double>(ctx, A, alpha, dx, beta, dy, dy);
        download(ctx, y, dy, ny);
        sync(ctx);
    } catch (...) {
        dfree(dx);
        dfree(dy);
        throw;
    }
    dfree(dx);
    dfree(dy);
    MG_API_END
}

extern "C" int mgldg_bsr_mv_t(mgldg_ctx* ctx, const mgldg_bsr* A, const double* x, double* y) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && x && y, MGLDG_ERR_ARG, "null argument");
    mgldg_bsr* At = bsr_transpose(ctx, A);
    size_t nx = (size_t)A->nbr * A->br, ny = (size_t)A->nbc * A->bc;
    double *dx = nullptr, *dy = nullptr;
    try {
        dx = dalloc<double>(std::max<size_t>(1, nx));
        dy = dalloc<double>(std::max<size_t>(1, ny));
        upload(ctx, dx, x, nx);
        spmv<double>(ctx, At, 1.0, dx, 0.0, nullptr, dy);
        download(ctx, y, dy, ny);
        sync(ctx);
    } catch (...) {
        dfree(dx);
        dfree(dy);
        delete At;
        throw;
    }
    dfree(dx);
    dfree(dy);
    delete At;
    MG_API_END
}

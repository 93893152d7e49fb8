// mg.cu -- multigrid hierarchy, V-cycle and preconditioned CG.
//
// Reference: Multigrid<N,P> (src/cartesian/multigrid/multigrid.h:280-433),
// its Level constructors (:83-171), relax/solve (:181-216), vcycle
// (:361-383), restrict/correct (:414-425); pcg (krylov.h:22-82) and the
// preconditioner closure of tests/cartesian/dg_tests.cpp:300-305.
//
// Precision forms: MGLDG_PREC_FP64 runs everything in FP64.  MGLDG_PREC_MIXED
// keeps FP32 copies of every level operator, inverse diagonal block and
// transfer, runs the whole V-cycle in FP32 with FP32 accumulation, and keeps
// the coarsest solve (mean projection and dense inverse), the outer CG
// residuals, dot products and updates in FP64 (the CG's q = A d in
// double-float arithmetic, k_spmv_df64 below).  MGLDG_PREC_MIXED_F16 is the
// mixed form with the level operators' Jacobi sweeps and residuals reading a
// block-scaled FP16 copy (one FP32 scale per block, entries / scale in FP16)
// where the blocks are 16 x 16 (f16_shape); everything else, including the
// inverse diagonal blocks and the transfers, stays FP32.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <string>

#include "api.cuh"
#include "mg.cuh"
#include "tail.cuh"
#include "rowdot.cuh"

using namespace mg;

namespace mg {

// ------------------------------------------------------------- small kernels
template <class A, class B>
__global__ void k_convert(int64_t n, const A* __restrict__ a, B* __restrict__ b) {
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) b[i] = (B)a[i];
}

template <class A, class B>
static void convert(mgldg_ctx* ctx, int64_t n, const A* a, B* b) {
    if (n == 0) return;
    int g = (int)std::min<int64_t>((n + 255) / 256, ctx->sm_count * 16);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_convert<A, B><<<g, 256, 0, ctx->stream>>>(n, a, b);
    }
    check_launch();
}

// coarsest level: x = Cinv b in FP64, one warp per row over all SMs (each
// CTA stages b in shared memory; Cinv, at most 128 MB, stays L2-resident
// across V-cycles when it fits).  The optional b -= mean(b) runs first in
// k_mean_project.
template <class T>
__global__ void __launch_bounds__(256) k_coarse_solve(int n, const T* __restrict__ b, T* __restrict__ x,
                                                      const double* __restrict__ Cinv) {
    extern __shared__ double sb[];
    for (int i = threadIdx.x; i < n; i += blockDim.x) sb[i] = (double)b[i];
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    for (int row = blockIdx.x * wpb + (threadIdx.x >> 5); row < n; row += gridDim.x * wpb) {
        const double* cr = Cinv + (size_t)row * n;
        double a = 0;
        for (int c = lane; c < n; c += 32) a += cr[c] * sb[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) x[row] = (T)a;
    }
}

template <class T>
__global__ void k_mean_project(int n, T* b) {
    __shared__ double red[32];
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += (double)b[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        red[0] = t / n;
    }
    __syncthreads();
    const double mean = red[0];
    for (int i = threadIdx.x; i < n; i += blockDim.x) b[i] = (T)((double)b[i] - mean);
}

// ----------------------------------------------------------------- V-cycle --
// the FP16-copy forms of the level products (FP32 vectors only)
template <class T>
static bool jacobi_f16_t(mgldg_ctx*, const mgldg_bsr*, const T*, const T*, const T*, T*, T, bool) { return false; }
template <>
bool jacobi_f16_t<float>(mgldg_ctx* ctx, const mgldg_bsr* A, const float* D, const float* b, const float* xin,
                         float* xout, float omega, bool xzero) {
    return jacobi_f16(ctx, A, D, b, xin, xout, omega, xzero);
}
template <class T>
static bool spmv_f16_t(mgldg_ctx*, const mgldg_bsr*, T, const T*, T, const T*, T*) { return false; }
template <>
bool spmv_f16_t<float>(mgldg_ctx* ctx, const mgldg_bsr* A, float alpha, const float* x, float beta, const float* yin,
                       float* y) {
    return spmv_f16(ctx, A, alpha, x, beta, yin, y, MGLDG_K_SPMV);
}

// n smoothing sweeps on level i; xzero: the level's x is the zero vector
// (not materialised: only the Jacobi smoother takes it, see zero_start)
template <class T>
static void relax(mgldg_mg* m, int i, int n, bool reverse, bool xzero = false) {
    LevelData& L = m->L[i];
    m->ctx->cur_level = i;
    const T* vals = bsr_vals<T>(L.A);
    const bool f16 = m->p.precision == MGLDG_PREC_MIXED_F16;
    if (m->p.relaxation == MGLDG_RELAX_GAUSS_SEIDEL) {
        // the n sweeps run as one dataflow pass (sweep k+1 trails sweep k)
        gs_sweeps<T>(m->ctx, L.A, vals, LV<T>::D(L), LV<T>::b(L), LV<T>::x(L), L.sched, (T)m->p.omega, reverse, n);
        return;
    }
    for (int k = 0; k < n; ++k) {
        const bool z = xzero && k == 0;
        if (!(f16 && jacobi_f16_t<T>(m->ctx, L.A, LV<T>::D(L), LV<T>::b(L), LV<T>::x(L), LV<T>::xt(L),
                                      (T)m->p.omega, z)))
            jacobi_sweep<T>(m->ctx, L.A, vals, LV<T>::D(L), LV<T>::b(L), LV<T>::x(L), LV<T>::xt(L), (T)m->p.omega,
                            z);
        std::swap(LV<T>::x(L), LV<T>::xt(L));
    }
}

// True when level i starts a V-cycle from x = 0 with a Jacobi sweep, which
// then reads neither x nor A (the V-cycle skips zeroing x as well): every
// level but a directly solved coarsest one, with npre >= 1.  Gauss-Seidel
// reads the old values of the rows after the current one, so its x stays
// materialised.
bool zero_start(const mgldg_mg* m, int i) {
    if (m->p.relaxation != MGLDG_RELAX_JACOBI || m->p.npre < 1) return false;
    return i < (int)m->L.size() - 1 || m->p.solver == MGLDG_COARSE_RELAXATION;
}

template <class T>
static void coarse_solve(mgldg_mg* m, int i, bool xzero) {
    LevelData& L = m->L[i];
    mgldg_ctx* ctx = m->ctx;
    ctx->cur_level = i;
    if (m->p.solver == MGLDG_COARSE_RELAXATION) {
        if (m->p.mean_project) {
            Launch K(ctx, MGLDG_K_COARSE);
            k_mean_project<T><<<1, 1024, 0, ctx->stream>>>((int)L.n, LV<T>::b(L));
        }
        check_launch();
        relax<T>(m, i, m->p.npre, false, xzero);
        relax<T>(m, i, m->p.npost, true);
        return;
    }
    if (m->p.mean_project) {
        Launch K(ctx, MGLDG_K_COARSE);
        k_mean_project<T><<<1, 1024, 0, ctx->stream>>>((int)L.n, LV<T>::b(L));
    }
    {
        const int n = (int)L.n;
        const int grid = std::max(1, std::min((n + 7) / 8, ctx->sm_count * 8));
        Launch K(ctx, MGLDG_K_COARSE);
        k_coarse_solve<T><<<grid, 256, L.n * sizeof(double), ctx->stream>>>(n, LV<T>::b(L), LV<T>::x(L), m->Cinv);
    }
    check_launch();
}

// xzero: level i's x is zero and not materialised (zero_start(m, i))
template <class T>
static void vcycle(mgldg_mg* m, int i, bool xzero) {
    mgldg_ctx* ctx = m->ctx;
    if (i == (int)m->L.size() - 1) {
        coarse_solve<T>(m, i, xzero);
        return;
    }
    if constexpr (std::is_same<T, float>::value) {
        if (i == m->tail_start && xzero) {
            // levels i .. last in one launch; the host's iterate buffers
            // follow the sweeps' swaps as relax() would leave them
            ctx->cur_level = i;
            tail_launch(m, i, m->tail_count);
            if ((m->p.npre + m->p.npost) & 1)
                for (int l = i; l < (int)m->L.size() - 1; ++l) std::swap(m->L[l].x32, m->L[l].xt32);
            return;
        }
    }
    LevelData& L = m->L[i];
    LevelData& C = m->L[i + 1];
    relax<T>(m, i, m->p.npre, false, xzero);
    // r = b - A x ; b_c = T^T r ; x_c = 0
    ctx->cur_level = i;
    if (!(m->p.precision == MGLDG_PREC_MIXED_F16 &&
          spmv_f16_t<T>(ctx, L.A, T(-1), LV<T>::x(L), T(1), LV<T>::b(L), LV<T>::r(L))))
        spmv<T>(ctx, L.A, T(-1), LV<T>::x(L), T(1), LV<T>::b(L), LV<T>::r(L));
    spmv<T>(ctx, L.Tt, T(1), LV<T>::r(L), T(0), (const T*)nullptr, LV<T>::b(C), nullptr, nullptr, nullptr,
            MGLDG_K_TRANSFER);
    const bool czero = zero_start(m, i + 1);
    if (!czero) MG_CHECK_CUDA(cudaMemsetAsync(LV<T>::x(C), 0, C.n * sizeof(T), ctx->stream));
    vcycle<T>(m, i + 1, czero);
    // x += T x_c
    ctx->cur_level = i;
    spmv<T>(ctx, L.T, T(1), LV<T>::x(C), T(1), LV<T>::x(L), LV<T>::x(L), nullptr, nullptr, nullptr, MGLDG_K_TRANSFER);
    relax<T>(m, i, m->p.npost, true);
}

static void take_errors(mgldg_mg* m) {
    int e = 0;
    for (auto& L : m->L)
        if (L.has_sched) e |= gs_take_error(m->ctx, L.sched);
    if (e) throw Error(MGLDG_ERR_TIMEOUT, "a Gauss-Seidel dependency wait ran out");
    take_device_error(m->ctx);
}

// The V-cycle's output s = x_level0 (converted to FP64 in the mixed forms)
// and the partial sums of b.s, the PCG's r.z, in one pass over the vectors
// instead of a copy followed by a separate dot product.
template <class T>
__global__ void __launch_bounds__(256) k_out_dot(int64_t n, const T* __restrict__ xl, const double* __restrict__ b,
                                                 double* __restrict__ s, double* __restrict__ partials) {
    __shared__ double sm[8];
    double acc = 0;
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
        const double v = (double)xl[i];
        s[i] = v;
        acc += b[i] * v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < 8; ++w) t += sm[w];
        partials[blockIdx.x] = t;
    }
}

template <class T>
static void out_dot(mgldg_ctx* ctx, int64_t n, const T* xl, const double* b, double* s, double* partials) {
    const int g = reduce_grid((int)std::min<int64_t>(n, 1 << 30));
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_out_dot<T><<<g, 256, 0, ctx->stream>>>(n, xl, b, s, partials);
    }
    check_launch();
}

// one V-cycle on device vectors b (FP64) and x (FP64, in/out); with
// `dot_part`, also the reduce_grid(n) partial sums of b.x of the result
static void vcycle_dev(mgldg_mg* m, const double* b, double* x, bool x_is_zero, double* dot_part = nullptr) {
    mgldg_ctx* ctx = m->ctx;
    LevelData& L = m->L[0];
    struct LevelReset {
        mgldg_ctx* c;
        ~LevelReset() { c->cur_level = -1; }
    } reset{ctx};
    if (m->p.precision != MGLDG_PREC_FP64) {
        convert<double, float>(ctx, L.n, b, L.b32);
        const bool z = x_is_zero && zero_start(m, 0);
        if (x_is_zero && !z) MG_CHECK_CUDA(cudaMemsetAsync(L.x32, 0, L.n * sizeof(float), ctx->stream));
        else if (!x_is_zero) convert<double, float>(ctx, L.n, x, L.x32);
        vcycle<float>(m, 0, z);
        if (dot_part) out_dot<float>(ctx, L.n, L.x32, b, x, dot_part);
        else convert<float, double>(ctx, L.n, L.x32, x);
    } else {
        MG_CHECK_CUDA(cudaMemcpyAsync(L.bb, b, L.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        const bool z = x_is_zero && zero_start(m, 0);
        if (x_is_zero && !z) MG_CHECK_CUDA(cudaMemsetAsync(L.x, 0, L.n * sizeof(double), ctx->stream));
        else if (!x_is_zero)
            MG_CHECK_CUDA(cudaMemcpyAsync(L.x, x, L.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        vcycle<double>(m, 0, z);
        if (dot_part) out_dot<double>(ctx, L.n, L.x, b, x, dot_part);
        else MG_CHECK_CUDA(cudaMemcpyAsync(x, L.x, L.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    }
}

// -------------------------------------------------------------------- PCG --
__global__ void k_pcg_init(PcgScalars* sc, const double* partials, int np) {
    // delta_new = delta_0 = r.d
    __shared__ double sm[32];
    double s = 0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
        sc->delta_new = t;
        sc->delta0 = t;
        sc->it = 0;
        // r.z < 0: preconditioner not positive definite; NaN/inf: it failed
        sc->breakdown = (t < 0.0 || !isfinite(t)) ? 1 : 0;
    }
}

__device__ double block_total(const double* partials, int np, double* sm) {
    double s = 0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) s += partials[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
    __syncthreads();
    double t = 0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += sm[w];
    __syncthreads();
    return t;
}

__global__ void k_pcg_alpha(PcgScalars* sc, const double* partials, int np) {
    __shared__ double sm[32];
    double dq = block_total(partials, np, sm);
    if (threadIdx.x == 0) {
        sc->dq = dq;
        double a = sc->delta_new / dq;
        if (!(dq > 0.0) || !isfinite(a)) sc->breakdown = 1;
        sc->alpha = a;
    }
}

// it < 0: the iteration index is the device-side counter
__global__ void k_pcg_rr(PcgScalars* sc, const double* partials, int np, double* hist, int it) {
    __shared__ double sm[32];
    double rr = block_total(partials, np, sm);
    if (threadIdx.x == 0) {
        sc->rr = rr;
        hist[it >= 0 ? it : sc->it] = sqrt(rr);
    }
}

__global__ void k_pcg_beta(PcgScalars* sc, const double* partials, int np) {
    __shared__ double sm[32];
    double rs = block_total(partials, np, sm);
    if (threadIdx.x == 0) {
        sc->delta_old = sc->delta_new;
        sc->delta_new = rs;
        double b = rs / sc->delta_old;
        // r.z < 0: the preconditioner is not positive definite (for example
        // a damped Jacobi smoother that diverges on some level); stop with an
        // error instead of meeting the r.z test spuriously
        if (!isfinite(b) || rs < 0.0) sc->breakdown = 1;
        sc->beta = b;
        sc->it += 1;
    }
}

// while-loop condition of a block of PCG iterations: go on while the
// reference's test (krylov.h:40) holds, no breakdown was seen, maxit is not
// reached and the next iteration is not a residual-replacement one (those
// start the next block, after the host has looked at the scalars)
__global__ void k_pcg_cond(const PcgScalars* sc, double tol2, int maxit, cudaGraphConditionalHandle h) {
    const int it = sc->it;
    const bool go = it < maxit && (it % 50) != 0 && sc->delta_new > tol2 * sc->delta0 && !sc->breakdown;
    cudaGraphSetConditional(h, go ? 1u : 0u);
}

// x += alpha d ; (r -= alpha q) ; partial r.r
__global__ void __launch_bounds__(256) k_pcg_update(int64_t n, const PcgScalars* sc, const double* __restrict__ d,
                                                    const double* __restrict__ q, double* __restrict__ x,
                                                    double* __restrict__ r, int update_r, double* partials) {
    __shared__ double sm[8];
    const double alpha = sc->alpha;
    double s = 0;
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
        x[i] += alpha * d[i];
        if (update_r) {
            double v = r[i] - alpha * q[i];
            r[i] = v;
            s += v * v;
        }
    }
    if (update_r) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int w = 0; w < 8; ++w) t += sm[w];
            partials[blockIdx.x] = t;
        }
    }
}

// d = s + beta d
__global__ void __launch_bounds__(256) k_pcg_dir(int64_t n, const PcgScalars* sc, const double* __restrict__ s,
                                                 double* __restrict__ d) {
    const double beta = sc->beta;
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256)
        d[i] = s[i] + beta * d[i];
}

// ------------------------------------------------- double-float outer product --
// In the mixed forms the outer CG's q = A d runs on the FP32 pipes in
// double-float arithmetic (GB300's FP64 rate bounds the FP64 product at about
// 1 TFLOP/s, below HBM): A = A_hi + A_lo (val32 + lo32) and d = d_hi + d_lo
// as float pairs, each product a*d formed as the exact FP32 product of the
// high parts (its error recovered with an FMA) plus the two cross terms,
// accumulated as an unnormalised (sum, error) float pair with a two-sum per
// product (Dekker's and Knuth's error-free transformations).  Relative error
// of a row sum about 2^-44 of sum |a d|; the lane pair's sums, the output
// and the fused q.d are FP64.  16 x 16 blocks, one warp per block row.
// (explicitly rounded operations: a product contracted into the two-sum's
// addition would break the error-free identities)
__device__ __forceinline__ void df_fma(float& sh, float& sl, float ah, float al, float dh, float dl) {
    const float p = __fmul_rn(ah, dh);
    const float pe = fmaf(ah, dh, -p);
    const float t = fmaf(ah, dl, fmaf(al, dh, pe));
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(e, t));
}

__global__ void __launch_bounds__(256) k_spmv_df64(int nbr, const int* __restrict__ row_ptr,
                                                   const int* __restrict__ col_idx, const float* __restrict__ ahi,
                                                   const float* __restrict__ alo, const float* __restrict__ dhi,
                                                   const float* __restrict__ dlo, const double* __restrict__ d,
                                                   double* __restrict__ q, double* __restrict__ partials) {
    __shared__ double sm[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = lane >> 1, c0 = (lane & 1) * 8;
    double dacc = 0;
    for (int row = blockIdx.x * 8 + warp; row < nbr; row += gridDim.x * 8) {
        const int k0 = __ldg(row_ptr + row), k1 = __ldg(row_ptr + row + 1);
        float sh = 0.f, sl = 0.f;
#pragma unroll 2
        for (int k = k0; k < k1; ++k) {
            const int j = __ldg(col_idx + k);
            const float4* ah = reinterpret_cast<const float4*>(ahi + (size_t)k * 256 + r * 16 + c0);
            const float4* al = reinterpret_cast<const float4*>(alo + (size_t)k * 256 + r * 16 + c0);
            const float4* xh = reinterpret_cast<const float4*>(dhi + (size_t)j * 16 + c0);
            const float4* xl = reinterpret_cast<const float4*>(dlo + (size_t)j * 16 + c0);
            const float4 a0 = __ldg(ah), a1 = __ldg(ah + 1), l0 = __ldg(al), l1 = __ldg(al + 1);
            const float4 h0 = __ldg(xh), h1 = __ldg(xh + 1), e0 = __ldg(xl), e1 = __ldg(xl + 1);
            df_fma(sh, sl, a0.x, l0.x, h0.x, e0.x);
            df_fma(sh, sl, a0.y, l0.y, h0.y, e0.y);
            df_fma(sh, sl, a0.z, l0.z, h0.z, e0.z);
            df_fma(sh, sl, a0.w, l0.w, h0.w, e0.w);
            df_fma(sh, sl, a1.x, l1.x, h1.x, e1.x);
            df_fma(sh, sl, a1.y, l1.y, h1.y, e1.y);
            df_fma(sh, sl, a1.z, l1.z, h1.z, e1.z);
            df_fma(sh, sl, a1.w, l1.w, h1.w, e1.w);
        }
        double v = (double)sh + (double)sl;
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        if ((lane & 1) == 0) {
            const size_t o = (size_t)row * 16 + r;
            q[o] = v;
            dacc += v * d[o];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dacc += __shfl_xor_sync(0xffffffffu, dacc, o);
    if (lane == 0) sm[warp] = dacc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < 8; ++w) t += sm[w];
        partials[blockIdx.x] = t;
    }
}

// The same product for square blocks of 3..10 (triangles, tetrahedra,
// agglomerated levels): 32 / B block rows per warp, lane (g, c) owning block
// column c as in the small-block kernels (coalesced rows of each block, one
// entry of each d pair), B double-float partial sums per lane, reduced in
// FP64 through shared memory in column order.
template <int B>
__global__ void __launch_bounds__(256) k_spmv_rows_df64(int nbr, const int* __restrict__ row_ptr,
                                                        const int* __restrict__ col_idx, const float* __restrict__ ahi,
                                                        const float* __restrict__ alo, const float* __restrict__ dhi,
                                                        const float* __restrict__ dlo, const double* __restrict__ d,
                                                        double* __restrict__ q, double* __restrict__ partials) {
    using R = Rows<B>;
    __shared__ double sr[8 * R::SM];
    __shared__ double sm[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane / R::S, c = lane - g * R::S;
    double* sw = sr + warp * R::SM;
    double dacc = 0;
    const int nw = gridDim.x * 8;
    for (int base = (blockIdx.x * 8 + warp) * R::G; base < nbr; base += nw * R::G) {
        const int row = base + g;
        const bool valid = g < R::G && row < nbr;
        float sh[B], sl[B];
#pragma unroll
        for (int r = 0; r < B; ++r) sh[r] = sl[r] = 0.f;
        if (valid) {
            const int k0 = __ldg(row_ptr + row), k1 = __ldg(row_ptr + row + 1);
#pragma unroll 2
            for (int k = k0; k < k1; ++k) {
                const int j = __ldg(col_idx + k);
                const float xh = __ldg(dhi + (size_t)j * B + c), xl = __ldg(dlo + (size_t)j * B + c);
                const float* ph = ahi + (size_t)k * (B * B) + c;
                const float* pl = alo + (size_t)k * (B * B) + c;
#pragma unroll
                for (int r = 0; r < B; ++r) df_fma(sh[r], sl[r], __ldg(ph + r * B), __ldg(pl + r * B), xh, xl);
            }
        }
        double acc[B];
#pragma unroll
        for (int r = 0; r < B; ++r) acc[r] = (double)sh[r] + (double)sl[r];
        const double v = rows_reduce<double, B, B>(acc, sw, g, c, g < R::G);
        if (valid) {
            const size_t o = (size_t)row * B + c;
            q[o] = v;
            dacc += v * d[o];
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dacc += __shfl_xor_sync(0xffffffffu, dacc, o);
    if (lane == 0) sm[warp] = dacc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < 8; ++w) t += sm[w];
        partials[blockIdx.x] = t;
    }
}

// d as a float pair: hi = fl32(d), lo = fl32(d - hi)
__global__ void __launch_bounds__(256) k_split(int64_t n, const double* __restrict__ d, float* __restrict__ hi,
                                               float* __restrict__ lo) {
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
        const double v = d[i];
        const float h = (float)v;
        hi[i] = h;
        lo[i] = (float)(v - (double)h);
    }
}

// d = s + beta d, and its float pair
__global__ void __launch_bounds__(256) k_pcg_dir_split(int64_t n, const PcgScalars* sc, const double* __restrict__ s,
                                                       double* __restrict__ d, float* __restrict__ hi,
                                                       float* __restrict__ lo) {
    const double beta = sc->beta;
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) {
        const double v = s[i] + beta * d[i];
        d[i] = v;
        const float h = (float)v;
        hi[i] = h;
        lo[i] = (float)(v - (double)h);
    }
}

static bool df64_shape(int b) { return b == 3 || b == 4 || b == 6 || b == 8 || b == 9 || b == 10 || b == 16; }

static bool df64_ok(const mgldg_mg* m, const mgldg_bsr* A) {
    return m->p.precision != MGLDG_PREC_FP64 && A->br == A->bc && df64_shape(A->br) && !A->blk && A->val32 &&
           A->lo32;
}

template <int B>
static int launch_rows_df64(mgldg_ctx* ctx, const mgldg_bsr* A, const mgldg_mg* m, double* partials) {
    const int rows_per_cta = 8 * Rows<B>::G;
    const int grid =
        std::max(1, std::min(std::min((A->nbr + rows_per_cta - 1) / rows_per_cta, ctx->sm_count * 8), ctx->n_partials));
    Launch L(ctx, MGLDG_K_SPMV);
    k_spmv_rows_df64<B><<<grid, 256, 0, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, A->val32, A->lo32, m->dhi,
                                                       m->dlo, m->d, m->q, partials);
    return grid;
}

static void spmv_df64(mgldg_ctx* ctx, const mgldg_bsr* A, const mgldg_mg* m, double* partials, int* np) {
    if (A->br == 16) {
        const int grid = std::max(1, std::min(std::min((A->nbr + 7) / 8, ctx->sm_count * 16), ctx->n_partials));
        {
            Launch L(ctx, MGLDG_K_SPMV);
            k_spmv_df64<<<grid, 256, 0, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, A->val32, A->lo32, m->dhi,
                                                       m->dlo, m->d, m->q, partials);
        }
        *np = grid;
    } else {
        switch (A->br) {
            case 3: *np = launch_rows_df64<3>(ctx, A, m, partials); break;
            case 4: *np = launch_rows_df64<4>(ctx, A, m, partials); break;
            case 6: *np = launch_rows_df64<6>(ctx, A, m, partials); break;
            case 8: *np = launch_rows_df64<8>(ctx, A, m, partials); break;
            case 9: *np = launch_rows_df64<9>(ctx, A, m, partials); break;
            case 10: *np = launch_rows_df64<10>(ctx, A, m, partials); break;
            default: throw Error(MGLDG_ERR_UNSUPPORTED, "double-float product: unsupported block size");
        }
    }
    check_launch();
}

static void drop_pcg_graph(mgldg_mg* m) {
    if (m->pg.exec) cudaGraphExecDestroy(m->pg.exec);
    m->pg = mgldg_mg::PcgGraph();
}

static void ensure_pcg(mgldg_mg* m, mgldg_ctx* ctx, int64_t n, int maxit) {
    if (m->pcg_n != n || m->pcg_maxit < maxit) drop_pcg_graph(m);
    if (m->pcg_n != n) {
        dfree(m->r); dfree(m->d); dfree(m->q); dfree(m->s); dfree(m->dhi); dfree(m->dlo);
        m->dhi = m->dlo = nullptr;
        m->r = dalloc<double>(n); m->d = dalloc<double>(n); m->q = dalloc<double>(n); m->s = dalloc<double>(n);
        if (m->p.precision != MGLDG_PREC_FP64) {
            m->dhi = dalloc<float>(n);
            m->dlo = dalloc<float>(n);
        }
        m->pcg_n = n;
    }
    if (m->pcg_maxit < maxit) {
        dfree(m->hist);
        m->hist = dalloc<double>(std::max(1, maxit));
        m->pcg_maxit = maxit;
    }
    if (!m->sc) {
        m->sc = dalloc<PcgScalars>(1);
        MG_CHECK_CUDA(cudaMallocHost(&m->h_sc, sizeof(PcgScalars)));
    }
}

// Captures one preconditioner application (x = 0, b = r, V-cycle, s = x) as
// a CUDA graph.  Returns null (and stops trying) if the capture is refused.
static mgldg_mg::Graph* capture_precon(mgldg_mg* m, const double* r, double* s, double* part) {
    mgldg_ctx* ctx = m->ctx;
    mgldg_mg::Graph& g = m->graphs[m->next_graph];
    m->next_graph ^= 1;
    if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
    }
    int64_t before[MGLDG_K_NCLASS];
    std::memcpy(before, ctx->launches, sizeof before);
    cudaGraph_t graph = nullptr;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        m->graphs_off = true;
        return nullptr;
    }
    bool ok = true;
    try {
        vcycle_dev(m, r, s, true, part);
    } catch (...) {
        ok = false;
    }
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &graph);
    if (e != cudaSuccess || !ok || !graph) ok = false;
    if (ok && cudaGraphInstantiate(&g.exec, graph, 0) != cudaSuccess) {
        g.exec = nullptr;
        ok = false;
    }
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    for (int k = 0; k < MGLDG_K_NCLASS; ++k) {
        g.launches[k] = ctx->launches[k] - before[k];
        ctx->launches[k] = before[k];   // captured, not run
    }
    if (!ok) {
        m->graphs_off = true;
        return nullptr;
    }
    g.in = r;
    g.out = s;
    g.part = part;
    return &g;
}

// s = M(r); with `part`, also the partial sums of r.s (reduce_grid(n) of them)
static void precon(mgldg_mg* m, const double* r, double* s, double* part = nullptr) {
    mgldg_ctx* ctx = m->ctx;
    if (m->L.empty()) {
        MG_CHECK_CUDA(cudaMemcpyAsync(s, r, m->pcg_n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        return;
    }
    // per-kernel event timing needs eager launches
    if (!ctx->prof && !m->graphs_off) {
        mgldg_mg::Graph* g = nullptr;
        for (auto& c : m->graphs)
            if (c.exec && c.in == r && c.out == s && c.part == part) g = &c;
        if (!g) g = capture_precon(m, r, s, part);
        if (g) {
            MG_CHECK_CUDA(cudaGraphLaunch(g->exec, ctx->stream));
            for (int k = 0; k < MGLDG_K_NCLASS; ++k) ctx->launches[k] += g->launches[k];
            return;
        }
    }
    vcycle_dev(m, r, s, true, part);
}

void mg_precon(mgldg_mg* m, const double* r, double* s) { precon(m, r, s); }
void mg_precon_eager(mgldg_mg* m, const double* r, double* s) {
    if (m->L.empty()) precon(m, r, s);
    else vcycle_dev(m, r, s, true);
}
void mg_take_errors(mgldg_mg* m) { take_errors(m); }

// One PCG iteration (krylov.h:43-61) on the context's stream: q = A d,
// alpha, x += alpha d with r -= alpha q (or, when `replace`, r = b - A x),
// ||r|| into the history at the device-side iteration index, s = M(r),
// delta_new = r.s, beta (which advances the iteration counter), d = s + beta d.
// `eager`: the preconditioner's launches are issued directly (inside a graph
// capture) instead of replaying its own graph.
static void pcg_iteration(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, const double* b, double* x, int64_t n,
                          bool df, int grid_vec, bool replace, bool eager) {
    double* part = ctx->d_partials;
    int np = 0;
    // q = A d ; alpha = delta_new / d.q
    if (df) spmv_df64(ctx, A, m, part, &np);
    else spmv<double>(ctx, A, 1.0, m->d, 0.0, nullptr, m->q, m->d, part, &np);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_pcg_alpha<<<1, 256, 0, ctx->stream>>>(m->sc, part, np);
    }
    check_launch();
    if (replace) {
        // x += alpha d ; r = b - A x (residual replacement)
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_pcg_update<<<grid_vec, 256, 0, ctx->stream>>>(n, m->sc, m->d, m->q, x, m->r, 0, part);
        }
        check_launch();
        spmv<double>(ctx, A, -1.0, x, 1.0, b, m->r, m->r, part, &np);
    } else {
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_pcg_update<<<grid_vec, 256, 0, ctx->stream>>>(n, m->sc, m->d, m->q, x, m->r, 1, part);
        }
        check_launch();
        np = grid_vec;
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_pcg_rr<<<1, 256, 0, ctx->stream>>>(m->sc, part, np, m->hist, -1);
    }
    check_launch();
    // s = M(r) ; delta_new = r.s (summed by the V-cycle's output kernel) ;
    // beta ; d = s + beta d
    if (m->L.empty()) {
        precon(m, m->r, m->s);
        dot_partials<double>(ctx, (int)n, m->r, m->s, part, &np);
    } else {
        if (eager) vcycle_dev(m, m->r, m->s, true, part);
        else precon(m, m->r, m->s, part);
        np = reduce_grid((int)std::min<int64_t>(n, 1 << 30));
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_pcg_beta<<<1, 256, 0, ctx->stream>>>(m->sc, part, np);
    }
    check_launch();
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        if (df) k_pcg_dir_split<<<grid_vec, 256, 0, ctx->stream>>>(n, m->sc, m->s, m->d, m->dhi, m->dlo);
        else k_pcg_dir<<<grid_vec, 256, 0, ctx->stream>>>(n, m->sc, m->s, m->d);
    }
    check_launch();
}

// Captures a block of iterations as one CUDA graph: the residual-replacement
// iteration, then a device-side while loop (a conditional graph node) over
// ordinary iterations whose condition k_pcg_cond sets after each one.  The
// host looks at the scalars once per block (at most every 50 iterations)
// instead of after every iteration.  Returns false (and stops trying for
// this multigrid object) if the runtime refuses any step.
static bool build_pcg_graph(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, const double* b, double* x, int64_t n,
                            bool df, int grid_vec, double tol, int maxit) {
    drop_pcg_graph(m);
    int64_t before[MGLDG_K_NCLASS];
    std::memcpy(before, ctx->launches, sizeof before);
    cudaGraph_t graph = nullptr;
    bool ok = true;
    mgldg_mg::PcgGraph G;
    const double tol2 = tol * tol;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    cudaGraph_t body = nullptr;
    try {
        pcg_iteration(ctx, m, A, b, x, n, df, grid_vec, true, true);
        for (int k = 0; k < MGLDG_K_NCLASS; ++k) G.pro_launches[k] = ctx->launches[k] - before[k];
        cudaStreamCaptureStatus st;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        MG_CHECK_CUDA(cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, nullptr, &ndeps));
        cudaGraphConditionalHandle h;
        MG_CHECK_CUDA(cudaGraphConditionalHandleCreate(&h, cg, 0, 0));
        // the loop's first test, then the loop node itself
        k_pcg_cond<<<1, 1, 0, ctx->stream>>>(m->sc, tol2, maxit, h);
        check_launch();
        MG_CHECK_CUDA(cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, nullptr, &ndeps));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t wnode;
        MG_CHECK_CUDA(cudaGraphAddNode(&wnode, cg, deps, nullptr, ndeps, &cp));
        body = cp.conditional.phGraph_out[0];
        MG_CHECK_CUDA(cudaStreamUpdateCaptureDependencies(ctx->stream, &wnode, nullptr, 1,
                                                          cudaStreamSetCaptureDependencies));
        if (cudaStreamEndCapture(ctx->stream, &graph) != cudaSuccess || !graph) ok = false;
        if (ok) {
            // the loop body: one ordinary iteration and the next test
            int64_t b2[MGLDG_K_NCLASS];
            std::memcpy(b2, ctx->launches, sizeof b2);
            MG_CHECK_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0,
                                                        cudaStreamCaptureModeThreadLocal));
            pcg_iteration(ctx, m, A, b, x, n, df, grid_vec, false, true);
            k_pcg_cond<<<1, 1, 0, ctx->stream>>>(m->sc, tol2, maxit, h);
            check_launch();
            cudaGraph_t bg = nullptr;
            if (cudaStreamEndCapture(ctx->stream, &bg) != cudaSuccess) ok = false;
            for (int k = 0; k < MGLDG_K_NCLASS; ++k) G.body_launches[k] = ctx->launches[k] - b2[k];
        }
    } catch (...) {
        ok = false;
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(ctx->stream, &junk);
        if (junk) cudaGraphDestroy(junk);
    }
    if (ok && cudaGraphInstantiate(&G.exec, graph, 0) != cudaSuccess) {
        G.exec = nullptr;
        ok = false;
    }
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    std::memcpy(ctx->launches, before, sizeof before);   // captured, not run
    if (!ok) return false;
    G.A = A;
    G.b = b;
    G.x = x;
    G.tol = tol;
    G.maxit = maxit;
    m->pg = G;
    return true;
}

// pcg on device vectors (krylov.h:22-68)
static void pcg_dev(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, const double* b, double* x, double tol,
                    int maxit, int* iters, double* res_hist) {
    const int64_t n = (int64_t)A->nbr * A->br;
    const int grid_vec = reduce_grid((int)std::min<int64_t>(n, 1 << 30));
    ensure_pcg(m, ctx, n, std::max(1, maxit));
    double* part = ctx->d_partials;
    int np = 0;
    // r = b - A x ; d = M(r) ; delta_new = delta_0 = r.d
    const bool df = df64_ok(m, A) && m->dhi;
    spmv<double>(ctx, A, -1.0, x, 1.0, b, m->r);
    if (m->L.empty()) {
        precon(m, m->r, m->d);
        dot_partials<double>(ctx, (int)n, m->r, m->d, part, &np);
    } else {
        precon(m, m->r, m->d, part);
        np = grid_vec;
    }
    if (df) {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_split<<<grid_vec, 256, 0, ctx->stream>>>(n, m->d, m->dhi, m->dlo);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_pcg_init<<<1, 256, 0, ctx->stream>>>(m->sc, part, np);
    }
    check_launch();
    MG_CHECK_CUDA(cudaMemcpyAsync(m->h_sc, m->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, ctx->stream));
    sync(ctx);
    take_errors(m);
    const double tol2 = tol * tol;
    int i = 0;
    bool broke = m->h_sc->breakdown != 0;
    if (broke) maxit = 0;
    // blocks of iterations as graphs (per-kernel event timing needs eager
    // launches; MGLDG_PCG_HOST_LOOP=1 keeps the host loop for profilers that
    // cannot see kernels under a conditional graph node)
    static const bool host_loop = std::getenv("MGLDG_PCG_HOST_LOOP") != nullptr;
    const bool use_graph = !ctx->prof && !m->pcg_graph_off && !host_loop;
    while (i < maxit && m->h_sc->delta_new > tol2 * m->h_sc->delta0) {
        if (use_graph && !m->pcg_graph_off) {
            mgldg_mg::PcgGraph& G = m->pg;
            if (!(G.exec && G.A == A && G.b == b && G.x == x && G.tol == tol && G.maxit == maxit) &&
                !build_pcg_graph(ctx, m, A, b, x, n, df, grid_vec, tol, maxit))
                m->pcg_graph_off = true;
            if (!m->pcg_graph_off && cudaGraphLaunch(m->pg.exec, ctx->stream) != cudaSuccess) {
                // refused at launch: nothing ran; iterate from the host
                cudaGetLastError();
                drop_pcg_graph(m);
                m->pcg_graph_off = true;
            }
            if (!m->pcg_graph_off) {
                MG_CHECK_CUDA(cudaMemcpyAsync(m->h_sc, m->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost,
                                              ctx->stream));
                sync(ctx);
                const int done = m->h_sc->it - i;   // the replacement iteration + the loop's
                for (int k = 0; k < MGLDG_K_NCLASS; ++k)
                    ctx->launches[k] += m->pg.pro_launches[k] + (int64_t)(done - 1) * m->pg.body_launches[k];
                i = m->h_sc->it;
                if (m->h_sc->breakdown) { broke = true; break; }
                continue;
            }
        }
        pcg_iteration(ctx, m, A, b, x, n, df, grid_vec, i % 50 == 0, false);
        MG_CHECK_CUDA(cudaMemcpyAsync(m->h_sc, m->sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, ctx->stream));
        sync(ctx);
        ++i;
        if (m->h_sc->breakdown) { broke = true; break; }
    }
    take_errors(m);
    if (iters) *iters = i;
    if (res_hist && i > 0) {
        download(ctx, res_hist, m->hist, i);
        sync(ctx);
    }
    if (broke) throw Error(MGLDG_ERR_BREAKDOWN, "pcg breakdown (d.q <= 0, r.z < 0 or a non-finite scalar)");
}

}  // namespace mg

mgldg_mg::~mgldg_mg() {
    if (ctx) cudaSetDevice(ctx->device);
    for (auto& g : graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (pg.exec) cudaGraphExecDestroy(pg.exec);
    for (auto& L : this->L) {
        if (L.owns_ops) delete L.ops;
        dfree(L.Dinv); dfree(L.Dinv32);
        if (L.has_sched) sched_free(L.sched);
        dfree(L.x); dfree(L.bb); dfree(L.r); dfree(L.xt);
        dfree(L.x32); dfree(L.b32); dfree(L.r32); dfree(L.xt32);
        delete L.T;
        delete L.Tt;
    }
    dfree(Cinv);
    dfree(r); dfree(d); dfree(q); dfree(s); dfree(hist); dfree(dhi); dfree(dlo);
    dfree(host_b); dfree(host_x);
    dfree(tail_count);
    dfree(sc);
    if (h_sc) cudaFreeHost(h_sc);
    mg::batch_free(batch);
    mg::seg_free(seg);
}

// ================================================================== C ABI ==
extern "C" void mgldg_mg_params_default(mgldg_mg_params* p) {
    if (!p) return;
    p->relaxation = MGLDG_RELAX_GAUSS_SEIDEL;
    p->omega = 0.8;
    p->solver = MGLDG_COARSE_CHOLESKY;
    p->npre = 3;
    p->npost = 3;
    p->restriction = MGLDG_RESTRICT_RATRAT;
    p->precision = MGLDG_PREC_FP64;
    p->max_levels = 0;
    p->mean_project = 1;
}

static void level_alloc(mgldg_ctx* ctx, mgldg_mg* m, LevelData& L, bool need_sched) {
    L.A = L.ops->A;
    L.ne = L.A->nbr;
    L.b = L.A->br;
    L.n = (int64_t)L.ne * L.b;
    bsr_build_diag(const_cast<mgldg_bsr*>(L.A));
    for (int i = 0; i < L.ne; ++i)
        MG_REQUIRE(L.A->h_diag[i] >= 0, MGLDG_ERR_SHAPE, "level matrix lacks a diagonal block");
    // inverse diagonal blocks (the reference's Dinv LDL^T factors)
    int* dstatus = dalloc<int>(1);
    try {
        MG_CHECK_CUDA(cudaMemsetAsync(dstatus, 0, sizeof(int), ctx->stream));
        L.Dinv = dalloc<double>((size_t)L.ne * L.b * L.b);
        block_inverse(ctx, L.A, L.Dinv, dstatus);
        int h = 0;
        download(ctx, &h, dstatus, 1);
        sync(ctx);
        MG_REQUIRE(h == 0, MGLDG_ERR_NOT_SPD, "singular diagonal block in a level matrix");
    } catch (...) {
        dfree(dstatus);
        throw;
    }
    dfree(dstatus);
    const bool mixed = m->p.precision != MGLDG_PREC_FP64;
    if (mixed) {
        bsr_ensure_fp32(const_cast<mgldg_bsr*>(L.A));
        if (m->p.precision == MGLDG_PREC_MIXED_F16 && !L.A->blk && f16_shape(L.A->br, L.A->bc))
            bsr_ensure_f16(const_cast<mgldg_bsr*>(L.A));
        // the finest operator is the outer CG's: its double-float split
        // (single-RHS products use it for 16 x 16 blocks, multi-RHS ones for
        // square blocks 4..16)
        if (&L == &m->L[0] && !L.A->blk) bsr_ensure_lo32(const_cast<mgldg_bsr*>(L.A));
        L.Dinv32 = dalloc<float>((size_t)L.ne * L.b * L.b);
        convert<double, float>(ctx, (int64_t)L.ne * L.b * L.b, L.Dinv, L.Dinv32);
        L.x32 = dalloc<float>(L.n); L.b32 = dalloc<float>(L.n); L.r32 = dalloc<float>(L.n); L.xt32 = dalloc<float>(L.n);
    } else {
        L.x = dalloc<double>(L.n); L.bb = dalloc<double>(L.n); L.r = dalloc<double>(L.n); L.xt = dalloc<double>(L.n);
    }
    if (need_sched) {
        sched_build(ctx, L.A, L.sched);
        L.has_sched = true;
    }
}

extern "C" int mgldg_mg_create(mgldg_ctx* ctx, const mgldg_ops* fine, const mgldg_bsr* const* T, int nT,
                               const mgldg_mg_params* params, mgldg_mg** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(out && fine && params && nT >= 0 && (nT == 0 || T), MGLDG_ERR_ARG, "bad multigrid arguments");
    *out = nullptr;
    const mgldg_mg_params& p = *params;
    MG_REQUIRE(p.relaxation == MGLDG_RELAX_JACOBI || p.relaxation == MGLDG_RELAX_GAUSS_SEIDEL, MGLDG_ERR_ARG,
               "Unknown relaxation method.");
    MG_REQUIRE(p.solver == MGLDG_COARSE_CHOLESKY || p.solver == MGLDG_COARSE_RELAXATION ||
                   p.solver == MGLDG_COARSE_DENSE, MGLDG_ERR_ARG, "Unknown coarse solver.");
    MG_REQUIRE(p.restriction == MGLDG_RESTRICT_RAT || p.restriction == MGLDG_RESTRICT_RATRAT, MGLDG_ERR_ARG,
               "Unknown restriction method.");
    MG_REQUIRE(p.precision == MGLDG_PREC_FP64 || p.precision == MGLDG_PREC_MIXED ||
                   p.precision == MGLDG_PREC_MIXED_F16 || p.precision == MGLDG_PREC_MIXED_TF32,
               MGLDG_ERR_ARG, "Unknown precision.");
    MG_REQUIRE(p.npre >= 0 && p.npost >= 0, MGLDG_ERR_ARG, "negative smoothing count");
    MG_REQUIRE(fine->A != nullptr, MGLDG_ERR_ARG, "fine operators lack A (call construct_laplacian)");
    mgldg_mg* m = new mgldg_mg();
    m->ctx = ctx;
    m->p = p;
    // MGLDG_SETUP_TRACE=1: phase times of the setup on stderr
    static const bool trace = std::getenv("MGLDG_SETUP_TRACE") != nullptr;
    auto t_last = std::chrono::steady_clock::now();
    auto phase = [&](const char* what, int level) {
        if (!trace) return;
        sync(ctx);
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[mgldg setup] level %d %-12s %8.1f ms\n", level, what,
                     std::chrono::duration<double, std::milli>(now - t_last).count());
        t_last = now;
    };
    try {
        const int use = (p.max_levels <= 0) ? nT : std::min(nT, p.max_levels - 1);
        m->L.resize(use + 1);
        m->L[0].ops = const_cast<mgldg_ops*>(fine);
        m->L[0].owns_ops = false;
        for (int i = 0; i < use; ++i) {
            const mgldg_bsr* Ti = T[i];
            MG_REQUIRE(Ti != nullptr, MGLDG_ERR_ARG, "null interpolation operator");
            const mgldg_ops* f = m->L[i].ops;
            MG_REQUIRE(Ti->nbr == f->A->nbr && Ti->br == f->A->br, MGLDG_ERR_SHAPE,
                       "interpolation rows do not match the finer level");
            // transfers: private copy with repeated blocks collapsed, and its transpose
            mgldg_bsr* Tc = bsr_clone(ctx, Ti);
            m->L[i].T = Tc;
            bsr_dedupe(ctx, Tc);
            phase("dedupe", i);
            m->L[i].Tt = bsr_transpose(ctx, Tc);
            phase("transpose", i);
            mgldg_ops* c = (p.restriction == MGLDG_RESTRICT_RATRAT) ? galerkin_ratrat(ctx, f, Tc) : galerkin_rat(ctx, f, Tc);
            m->L[i + 1].ops = c;
            m->L[i + 1].owns_ops = true;
            phase("galerkin", i);
            if (trace) {
                double pl = 0, pr = 0;
                setup_clock_take(&pl, &pr);
                std::fprintf(stderr, "[mgldg setup] level %d   symbolic plans %.1f ms, numeric products %.1f ms\n", i, pl, pr);
            }
            if (p.precision != MGLDG_PREC_FP64) {
                bsr_ensure_fp32(Tc);
                bsr_ensure_fp32(m->L[i].Tt);
            }
        }
        const int last = use;
        for (int i = 0; i <= last; ++i) {
            bool sched = p.relaxation == MGLDG_RELAX_GAUSS_SEIDEL && (i < last || p.solver == MGLDG_COARSE_RELAXATION);
            level_alloc(ctx, m, m->L[i], sched);
            phase("smoother", i);
        }
        if (p.solver != MGLDG_COARSE_RELAXATION) {
            const mgldg_bsr* Ac = m->L[last].A;
            if (p.solver == MGLDG_COARSE_CHOLESKY)
                MG_REQUIRE(Ac->nbr == 1, MGLDG_ERR_ARG,
                           "Cholesky coarse solve needs a one-element coarsest level (use MGLDG_COARSE_DENSE)");
            m->nc = Ac->nbr * Ac->br;
            MG_REQUIRE(m->nc <= 4096, MGLDG_ERR_UNSUPPORTED, "dense coarsest solve limited to 4096 unknowns");
            m->Cinv = dalloc<double>((size_t)m->nc * m->nc);
            dense_spd_inverse(ctx, Ac, m->Cinv);
            phase("coarse", last);
        }
        // the coarse tail (opt-in): from the first level of at most
        // MGLDG_VTAIL_ROWS block rows.  Off by default: on the 512^2 Q3
        // solve it cut the event-timed coarse levels from 5.5 to 3.7 ms per
        // solve, but the graph-replayed solve went from 53.2 to 54.5 ms --
        // its ~28 grid barriers cost about what the replayed launches did.
        {
            const char* env = std::getenv("MGLDG_VTAIL_ROWS");
            const long rows = env ? std::strtol(env, nullptr, 10) : 0;
            for (int i = 1; rows > 0 && i < last; ++i)
                if (m->L[i].ne <= rows) {
                    if (tail_supported(m, i)) {
                        m->tail_count = dalloc<unsigned>(1);
                        m->tail_start = i;
                    }
                    break;
                }
        }
        sync(ctx);
    } catch (...) {
        delete m;
        throw;
    }
    *out = m;
    MG_API_END
}

extern "C" int mgldg_mg_destroy(mgldg_mg* m) {
    delete m;
    return MGLDG_OK;
}

extern "C" int mgldg_mg_nlevels(const mgldg_mg* m, int* n) {
    if (!m || !n) return MGLDG_ERR_ARG;
    *n = (int)m->L.size();
    return MGLDG_OK;
}

extern "C" int mgldg_mg_level_op(const mgldg_mg* m, int level, int which, const mgldg_bsr** A) {
    if (!m || level < 0 || level >= (int)m->L.size()) return MGLDG_ERR_ARG;
    return mgldg_ops_get(m->L[level].ops, which, A);
}

extern "C" int mgldg_mg_vcycle_dev(mgldg_ctx* ctx, mgldg_mg* m, const double* b, double* x) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(m && b && x, MGLDG_ERR_ARG, "null argument");
    vcycle_dev(m, b, x, false);
    MG_API_END
}

extern "C" int mgldg_mg_vcycle(mgldg_ctx* ctx, mgldg_mg* m, const double* b, double* x) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(m && b && x, MGLDG_ERR_ARG, "null argument");
    const int64_t n = m->L[0].n;
    double *db = nullptr, *dx = nullptr;
    try {
        db = dalloc<double>(n);
        dx = dalloc<double>(n);
        upload(ctx, db, b, n);
        upload(ctx, dx, x, n);
        vcycle_dev(m, db, dx, false);
        download(ctx, x, dx, n);
        sync(ctx);
        take_errors(m);
    } catch (...) {
        dfree(db);
        dfree(dx);
        throw;
    }
    dfree(db);
    dfree(dx);
    MG_API_END
}

extern "C" int mgldg_mg_relax(mgldg_ctx* ctx, mgldg_mg* m, int level, int n, int reverse, const double* b, double* x) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(m && b && x && level >= 0 && level < (int)m->L.size() && n >= 0, MGLDG_ERR_ARG, "bad relax arguments");
    LevelData& L = m->L[level];
    MG_REQUIRE(m->p.relaxation == MGLDG_RELAX_JACOBI || L.has_sched, MGLDG_ERR_ARG, "no smoother schedule on this level");
    double *db = nullptr, *dx = nullptr;
    try {
        db = dalloc<double>(L.n);
        dx = dalloc<double>(L.n);
        upload(ctx, db, b, L.n);
        upload(ctx, dx, x, L.n);
        if (m->p.precision != MGLDG_PREC_FP64) {
            convert<double, float>(ctx, L.n, db, L.b32);
            convert<double, float>(ctx, L.n, dx, L.x32);
            relax<float>(m, level, n, reverse != 0);
            convert<float, double>(ctx, L.n, L.x32, dx);
        } else {
            MG_CHECK_CUDA(cudaMemcpyAsync(L.bb, db, L.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
            MG_CHECK_CUDA(cudaMemcpyAsync(L.x, dx, L.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
            relax<double>(m, level, n, reverse != 0);
            MG_CHECK_CUDA(cudaMemcpyAsync(dx, L.x, L.n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        }
        download(ctx, x, dx, L.n);
        sync(ctx);
        take_errors(m);
    } catch (...) {
        dfree(db);
        dfree(dx);
        throw;
    }
    dfree(db);
    dfree(dx);
    MG_API_END
}

extern "C" int mgldg_pcg_dev(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, const double* b, double* x, double tol,
                             int maxit, int* iters, double* res_hist) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && b && x && maxit >= 0, MGLDG_ERR_ARG, "bad pcg arguments");
    MG_REQUIRE(A->br == A->bc && A->nbr == A->nbc, MGLDG_ERR_SHAPE, "pcg needs a square matrix");
    if (m) MG_REQUIRE(m->L[0].n == (int64_t)A->nbr * A->br, MGLDG_ERR_SHAPE, "preconditioner size mismatch");
    if (m) {
        pcg_dev(ctx, m, A, b, x, tol, maxit, iters, res_hist);
    } else {
        // unpreconditioned overload (krylov.h:78-82): a level-free holder
        // owns the work space for this call only
        mgldg_mg plain;
        plain.ctx = ctx;
        mgldg_mg_params_default(&plain.p);
        pcg_dev(ctx, &plain, A, b, x, tol, maxit, iters, res_hist);
    }
    MG_API_END
}

extern "C" int mgldg_pcg(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, const double* b, double* x, double tol,
                         int maxit, int* iters, double* res_hist) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && b && x && maxit >= 0, MGLDG_ERR_ARG, "bad pcg arguments");
    MG_REQUIRE(A->br == A->bc && A->nbr == A->nbc, MGLDG_ERR_SHAPE, "pcg needs a square matrix");
    if (m) MG_REQUIRE(m->L[0].n == (int64_t)A->nbr * A->br, MGLDG_ERR_SHAPE, "preconditioner size mismatch");
    const int64_t n = (int64_t)A->nbr * A->br;
    if (m) {
        // the multigrid object keeps the device copies between calls
        if (m->host_n != n) {
            dfree(m->host_b);
            dfree(m->host_x);
            m->host_b = m->host_x = nullptr;
            m->host_n = 0;
            m->host_b = dalloc<double>(n);
            m->host_x = dalloc<double>(n);
            m->host_n = n;
        }
        upload(ctx, m->host_b, b, n);
        upload(ctx, m->host_x, x, n);
        pcg_dev(ctx, m, A, m->host_b, m->host_x, tol, maxit, iters, res_hist);
        download(ctx, x, m->host_x, n);
        sync(ctx);
        return MGLDG_OK;
    }
    double *db = nullptr, *dx = nullptr;
    try {
        db = dalloc<double>(n);
        dx = dalloc<double>(n);
        upload(ctx, db, b, n);
        upload(ctx, dx, x, n);
        {
            mgldg_mg plain;
            plain.ctx = ctx;
            mgldg_mg_params_default(&plain.p);
            pcg_dev(ctx, &plain, A, db, dx, tol, maxit, iters, res_hist);
        }
        download(ctx, x, dx, n);
        sync(ctx);
    } catch (...) {
        dfree(db);
        dfree(dx);
        throw;
    }
    dfree(db);
    dfree(dx);
    MG_API_END
}

// ======================================================= allocation-free CG ==
// mgldg_cg_noalloc_dev: the unpreconditioned CG of mgldg_pcg_dev(ctx, NULL,
// ...) for callers that must not allocate device memory during a solve --
// for example a host framework whose caching allocator already owns the
// device memory, or a caller held to a fixed memory budget set at start-up.
// The existing entry point allocates four work vectors, a history buffer and
// pinned scalars on every call; this one uses the fixed scratch array below
// instead and calls no allocating routine (with kernel profiling off, the
// default).  The array is carved into r, d, q, s (kCgMaxN doubles each), the
// reduction partials, the residual history and the scalar block.
namespace {
constexpr int64_t kCgMaxN = 131072;    // largest system: 131,072 unknowns
constexpr int kCgMaxIt = 1024;         // largest iteration limit
constexpr int kCgParts = 8192;         // CTA partial sums (>= ctx->n_partials)
constexpr int64_t kCgScalarOff = 4 * kCgMaxN + kCgParts + kCgMaxIt;
constexpr int64_t kCgScratchDoubles = kCgScalarOff + 32;   // ~4.1 MiB per GPU
static_assert(sizeof(mg::PcgScalars) <= 32 * sizeof(double), "scalar block too small");
static_assert((kCgScalarOff * sizeof(double)) % 256 == 0, "scalar block alignment");
}  // namespace

// One copy per GPU that loads this library, held until the process exits;
// every call on that GPU shares it.
static __device__ __align__(256) double g_cg_scratch[kCgScratchDoubles];

static std::mutex g_cg_scratch_mu;
static double* g_cg_scratch_addr[64] = {nullptr};

// Device address of g_cg_scratch on `device` (which must be current).  Host
// code cannot use the symbol's name as a device pointer; the address is
// looked up once per device, on the first call made on that device, in the
// device's primary context (the one the runtime API uses).  The cached
// address belongs to that context: a process that resets the device
// (cudaDeviceReset) after the first call must not call the entry point again.
static double* cg_scratch(int device) {
    MG_REQUIRE(device >= 0 && device < 64, MGLDG_ERR_ARG, "device index out of range for the scratch table");
    std::lock_guard<std::mutex> lock(g_cg_scratch_mu);
    if (!g_cg_scratch_addr[device]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_cg_scratch);
        if (e != cudaSuccess)
            throw Error(MGLDG_ERR_CUDA, std::string("cudaGetSymbolAddress(g_cg_scratch): ") + cudaGetErrorString(e));
        g_cg_scratch_addr[device] = static_cast<double*>(p);
    }
    return g_cg_scratch_addr[device];
}

extern "C" int mgldg_cg_noalloc_dev(mgldg_ctx* ctx, const mgldg_bsr* A, const double* b, double* x, double tol,
                                    int maxit, int* iters, double* res_hist) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && b && x && maxit >= 0, MGLDG_ERR_ARG, "bad cg arguments");
    MG_REQUIRE(A->br == A->bc && A->nbr == A->nbc, MGLDG_ERR_SHAPE, "cg needs a square matrix");
    const int64_t n = (int64_t)A->nbr * A->br;
    MG_REQUIRE(n <= kCgMaxN, MGLDG_ERR_ARG,
               "mgldg_cg_noalloc_dev: system has " + std::to_string(n) + " unknowns, the fixed scratch holds at most " +
                   std::to_string(kCgMaxN) + " (use mgldg_pcg_dev)");
    MG_REQUIRE(maxit <= kCgMaxIt, MGLDG_ERR_ARG,
               "mgldg_cg_noalloc_dev: maxit " + std::to_string(maxit) + " exceeds " + std::to_string(kCgMaxIt));
    MG_REQUIRE(ctx->n_partials <= kCgParts, MGLDG_ERR_ARG, "context reduction width exceeds the scratch");
    double* base = cg_scratch(ctx->device);
    double* r = base;
    double* d = base + kCgMaxN;
    double* q = base + 2 * kCgMaxN;
    double* s = base + 3 * kCgMaxN;
    double* part = base + 4 * kCgMaxN;
    double* hist = part + kCgParts;
    PcgScalars* sc = reinterpret_cast<PcgScalars*>(base + kCgScalarOff);
    // the scratch keeps the previous call's contents: start the scalars at zero
    MG_CHECK_CUDA(cudaMemsetAsync(sc, 0, sizeof(PcgScalars), ctx->stream));
    const int grid_vec = reduce_grid((int)n);
    PcgScalars h{};
    int np = 0;
    // r = b - A x ; d = r ; delta_new = delta_0 = r.d   (krylov.h:35-38, identity preconditioner)
    spmv<double>(ctx, A, -1.0, x, 1.0, b, r);
    MG_CHECK_CUDA(cudaMemcpyAsync(d, r, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    dot_partials<double>(ctx, (int)n, r, d, part, &np);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_pcg_init<<<1, 256, 0, ctx->stream>>>(sc, part, np);
    }
    check_launch();
    MG_CHECK_CUDA(cudaMemcpyAsync(&h, sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, ctx->stream));
    sync(ctx);
    const double tol2 = tol * tol;
    int i = 0;
    // a non-finite r.r (NaN or inf in b or x) is a breakdown before the
    // first iteration, reported as mgldg_pcg_dev reports it
    bool broke = h.breakdown != 0;
    if (broke) maxit = 0;
    while (i < maxit && h.delta_new > tol2 * h.delta0) {
        spmv<double>(ctx, A, 1.0, d, 0.0, nullptr, q, d, part, &np);
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_pcg_alpha<<<1, 256, 0, ctx->stream>>>(sc, part, np);
        }
        check_launch();
        if (i % 50 == 0) {
            {
                Launch L(ctx, MGLDG_K_VECTOR);
                k_pcg_update<<<grid_vec, 256, 0, ctx->stream>>>(n, sc, d, q, x, r, 0, part);
            }
            check_launch();
            spmv<double>(ctx, A, -1.0, x, 1.0, b, r, r, part, &np);
        } else {
            {
                Launch L(ctx, MGLDG_K_VECTOR);
                k_pcg_update<<<grid_vec, 256, 0, ctx->stream>>>(n, sc, d, q, x, r, 1, part);
            }
            check_launch();
            np = grid_vec;
        }
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_pcg_rr<<<1, 256, 0, ctx->stream>>>(sc, part, np, hist, i);
        }
        check_launch();
        MG_CHECK_CUDA(cudaMemcpyAsync(s, r, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        dot_partials<double>(ctx, (int)n, r, s, part, &np);
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_pcg_beta<<<1, 256, 0, ctx->stream>>>(sc, part, np);
        }
        check_launch();
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_pcg_dir<<<grid_vec, 256, 0, ctx->stream>>>(n, sc, s, d);
        }
        check_launch();
        MG_CHECK_CUDA(cudaMemcpyAsync(&h, sc, sizeof(PcgScalars), cudaMemcpyDeviceToHost, ctx->stream));
        sync(ctx);
        ++i;
        if (h.breakdown) { broke = true; break; }
    }
    if (iters) *iters = i;
    if (res_hist && i > 0) {
        MG_CHECK_CUDA(cudaMemcpyAsync(res_hist, hist, i * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        sync(ctx);
    }
    if (broke) throw Error(MGLDG_ERR_BREAKDOWN, "cg breakdown (d.q <= 0 or a non-finite scalar)");
    MG_API_END
}

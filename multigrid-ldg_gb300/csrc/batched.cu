// batched.cu -- many right-hand sides per operator: block SpMM, the
// multi-RHS V-cycle and a lock-step block PCG.
//
// The reference solves one right-hand side at a time (pcg, krylov.h:22-68;
// vcycle, multigrid.h:361-383).  Here k right-hand sides share every sweep
// over the operator: a multi-vector of k columns over n unknowns is stored
// row-major, X[u*k + c], so the k values of one unknown are contiguous and a
// warp reads them with coalesced vector loads while one block of A, staged
// once in shared memory, is applied to all k columns.  Each column keeps its
// own CG scalars (alpha, beta, delta) and stops on its own criterion
// delta_c <= tol^2 delta0_c; a stopped column is frozen (no further updates)
// while the others continue, so column c reproduces the single-RHS pcg of
// b_c.  The smoother is block Jacobi (the exact Gauss-Seidel order is a
// single-RHS dataflow kernel, smooth.cu).
//
// Tile widths: a warp covers 32*V columns (V = 1, 2 or 4 consecutive columns
// per lane); the best V for each level operator and kernel is picked by
// timing every valid candidate once when the work space is set up.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <map>

#include "api.cuh"
#include "mg.cuh"

using namespace mg;

namespace mg {

constexpr int kMaxCols = 1024;

template <class T>
struct SpmmArgs {
    int nbr;
    const int* row_ptr;
    const int* col_idx;
    const T* val;
    const int* blk;
    T alpha, beta;
    const T* X;
    const T* Yin;
    T* Y;
    int k;
    // Jacobi epilogue: Y = X + omega * Dinv_i (B_i - (A X)_i)
    const T* Dinv;
    const T* B;
    T omega;
    // Jacobi from X = 0: neither X nor A is read ((A 0)_i is +0, so the
    // values are the full sweep's bit for bit)
    int xzero;
};

template <class T, int V>
struct VecIO;
template <class T>
struct VecIO<T, 1> {
    static __device__ __forceinline__ void ld(const T* p, T (&v)[1]) { v[0] = p[0]; }
    static __device__ __forceinline__ void st(T* p, const T (&v)[1]) { p[0] = v[0]; }
};
template <>
struct VecIO<float, 2> {
    static __device__ __forceinline__ void ld(const float* p, float (&v)[2]) {
        float2 t = *reinterpret_cast<const float2*>(p);
        v[0] = t.x; v[1] = t.y;
    }
    static __device__ __forceinline__ void st(float* p, const float (&v)[2]) {
        *reinterpret_cast<float2*>(p) = make_float2(v[0], v[1]);
    }
};
template <>
struct VecIO<float, 4> {
    static __device__ __forceinline__ void ld(const float* p, float (&v)[4]) {
        float4 t = *reinterpret_cast<const float4*>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    static __device__ __forceinline__ void st(float* p, const float (&v)[4]) {
        *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
    }
};
template <>
struct VecIO<double, 2> {
    static __device__ __forceinline__ void ld(const double* p, double (&v)[2]) {
        double2 t = *reinterpret_cast<const double2*>(p);
        v[0] = t.x; v[1] = t.y;
    }
    static __device__ __forceinline__ void st(double* p, const double (&v)[2]) {
        *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    }
};

// shared-memory staging of one b x b block, stored transposed (column cc of
// the block is contiguous) with the column padded to a multiple of 4 values
template <int BR, int BC>
struct Stage {
    static constexpr int BRP = (BR + 3) / 4 * 4;
    static constexpr int SIZE = BC * BRP;
    static constexpr int PER = (BR * BC + 31) / 32;
};

template <class T, int BR, int BC>
__device__ __forceinline__ void stage_fetch(const T* __restrict__ src, int lane, T (&dst)[Stage<BR, BC>::PER]) {
#pragma unroll
    for (int p = 0; p < Stage<BR, BC>::PER; ++p) {
        const int idx = lane + 32 * p;
        if (idx < BR * BC) dst[p] = src[idx];
    }
}

template <class T, int BR, int BC>
__device__ __forceinline__ void stage_store(T* s, int lane, const T (&src)[Stage<BR, BC>::PER]) {
#pragma unroll
    for (int p = 0; p < Stage<BR, BC>::PER; ++p) {
        const int idx = lane + 32 * p;
        if (idx < BR * BC) s[(idx % BC) * Stage<BR, BC>::BRP + idx / BC] = src[p];
    }
}

// acc[r][v] += sum_cc S[cc][r] * x[cc][v] with S the transposed staged block
template <class T, int BR, int BC, int V>
__device__ __forceinline__ void block_apply(const T* __restrict__ S, const T* __restrict__ xb, int k, T (&acc)[BR][V]) {
    constexpr int BRP = Stage<BR, BC>::BRP;
#pragma unroll
    for (int cc = 0; cc < BC; ++cc) {
        T xv[V];
        VecIO<T, V>::ld(xb + (size_t)cc * k, xv);
        const T* col = S + cc * BRP;
        if constexpr (sizeof(T) == 4) {
#pragma unroll
            for (int r = 0; r < BR; r += 4) {
                const float4 a4 = *reinterpret_cast<const float4*>(col + r);
                const float av[4] = {a4.x, a4.y, a4.z, a4.w};
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (r + q < BR)
#pragma unroll
                        for (int v = 0; v < V; ++v) acc[r + q][v] = fmaf(av[q], xv[v], acc[r + q][v]);
            }
        } else {
#pragma unroll
            for (int r = 0; r < BR; r += 2) {
                const double2 a2 = *reinterpret_cast<const double2*>(col + r);
                const double av[2] = {a2.x, a2.y};
#pragma unroll
                for (int q = 0; q < 2; ++q)
                    if (r + q < BR)
#pragma unroll
                        for (int v = 0; v < V; ++v) acc[r + q][v] = fma(av[q], xv[v], acc[r + q][v]);
            }
        }
    }
}

// One warp per block row; the lane owns columns c .. c+V-1 of the column
// tile blockIdx.y.  MODE 0: Y = alpha A X + beta Yin.  MODE 1 (square blocks):
// Y = X + omega Dinv_i (B_i - (A X)_i).
template <class T, int BR, int BC, int V, int MODE>
__global__ void __launch_bounds__(256) k_spmm(const SpmmArgs<T> a) {
    using S = Stage<BR, BC>;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    T* st = reinterpret_cast<T*>(smraw) + (size_t)warp * S::SIZE;
    const int c = (blockIdx.y * 32 + lane) * V;
    const bool cok = c < a.k;
    const int k = a.k;
    for (int i = blockIdx.x * wpb + warp; i < a.nbr; i += gridDim.x * wpb) {
        T acc[BR][V];
#pragma unroll
        for (int r = 0; r < BR; ++r)
#pragma unroll
            for (int v = 0; v < V; ++v) acc[r][v] = T(0);
        const int k0 = a.row_ptr[i], k1 = (MODE == 1 && a.xzero) ? k0 : a.row_ptr[i + 1];
        T pre[S::PER];
        if (k0 < k1) stage_fetch<T, BR, BC>(a.val + (size_t)(a.blk ? a.blk[k0] : k0) * (BR * BC), lane, pre);
        for (int kk = k0; kk < k1; ++kk) {
            const int j = a.col_idx[kk];
            __syncwarp();
            stage_store<T, BR, BC>(st, lane, pre);
            __syncwarp();
            if (kk + 1 < k1)
                stage_fetch<T, BR, BC>(a.val + (size_t)(a.blk ? a.blk[kk + 1] : kk + 1) * (BR * BC), lane, pre);
            if (cok) block_apply<T, BR, BC, V>(st, a.X + (size_t)j * BC * k + c, k, acc);
        }
        const size_t y0 = (size_t)i * BR * k + c;
        if constexpr (MODE == 0) {
            if (cok) {
#pragma unroll
                for (int r = 0; r < BR; ++r) {
                    T out[V];
                    if (a.beta != T(0)) {
                        T yv[V];
                        VecIO<T, V>::ld(a.Yin + y0 + (size_t)r * k, yv);
#pragma unroll
                        for (int v = 0; v < V; ++v) out[v] = a.alpha * acc[r][v] + a.beta * yv[v];
                    } else {
#pragma unroll
                        for (int v = 0; v < V; ++v) out[v] = a.alpha * acc[r][v];
                    }
                    VecIO<T, V>::st(a.Y + y0 + (size_t)r * k, out);
                }
            }
        } else {
            // stage Dinv_i, then t = B_i - acc ; Y_i = X_i + omega Dinv_i t
            T pd[S::PER];
            stage_fetch<T, BR, BC>(a.Dinv + (size_t)i * (BR * BC), lane, pd);
            __syncwarp();
            stage_store<T, BR, BC>(st, lane, pd);
            __syncwarp();
            if (cok) {
#pragma unroll
                for (int r = 0; r < BR; ++r) {
                    T bv[V];
                    VecIO<T, V>::ld(a.B + y0 + (size_t)r * k, bv);
#pragma unroll
                    for (int v = 0; v < V; ++v) acc[r][v] = bv[v] - acc[r][v];
                }
                T out[BR][V];
#pragma unroll
                for (int r = 0; r < BR; ++r)
#pragma unroll
                    for (int v = 0; v < V; ++v) out[r][v] = T(0);
                // out += Dinv t, the same staged-column product on registers
#pragma unroll
                for (int cc = 0; cc < BC; ++cc) {
                    const T* col = st + cc * S::BRP;
#pragma unroll
                    for (int r = 0; r < BR; ++r)
#pragma unroll
                        for (int v = 0; v < V; ++v) out[r][v] = fma(col[r], acc[cc][v], out[r][v]);
                }
#pragma unroll
                for (int r = 0; r < BR; ++r) {
                    T xv[V];
                    if (a.xzero) {
#pragma unroll
                        for (int v = 0; v < V; ++v) xv[v] = T(0);
                    } else {
                        VecIO<T, V>::ld(a.X + y0 + (size_t)r * k, xv);
                    }
#pragma unroll
                    for (int v = 0; v < V; ++v) xv[v] = xv[v] + a.omega * out[r][v];
                    VecIO<T, V>::st(a.Y + y0 + (size_t)r * k, xv);
                }
            }
        }
    }
}

// any block shape: one thread per (block row, column), rows of the block in
// a loop (MODE 1 needs br <= 64)
template <class T, int MODE>
__global__ void __launch_bounds__(256) k_spmm_generic(const SpmmArgs<T> a, int br, int bc) {
    const int64_t total = (int64_t)a.nbr * a.k;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(t / a.k), c = (int)(t % a.k);
        const int k0 = a.row_ptr[i], k1 = (MODE == 1 && a.xzero) ? k0 : a.row_ptr[i + 1];
        T tv[64];
        for (int r = 0; r < br; ++r) {
            T s = 0;
            for (int kk = k0; kk < k1; ++kk) {
                const T* blkp = a.val + (size_t)(a.blk ? a.blk[kk] : kk) * br * bc + (size_t)r * bc;
                const T* xb = a.X + (size_t)a.col_idx[kk] * bc * a.k + c;
                for (int cc = 0; cc < bc; ++cc) s = fma(blkp[cc], xb[(size_t)cc * a.k], s);
            }
            const size_t o = ((size_t)i * br + r) * a.k + c;
            if (MODE == 0) {
                a.Y[o] = a.alpha * s + (a.beta != T(0) ? a.beta * a.Yin[o] : T(0));
            } else {
                tv[r] = a.B[o] - s;
            }
        }
        if (MODE == 1) {
            for (int r = 0; r < br; ++r) {
                T s = 0;
                for (int cc = 0; cc < br; ++cc) s = fma(a.Dinv[(size_t)i * br * br + r * br + cc], tv[cc], s);
                const size_t o = ((size_t)i * br + r) * a.k + c;
                a.Y[o] = (a.xzero ? T(0) : a.X[o]) + a.omega * s;
            }
        }
    }
}

struct TileCfg {
    int V = 1;
    int wpb = 8;
    bool mma = false;   // tensor-core kernel (k_spmm_mma), MGLDG_PREC_MIXED_TF32 only
};

// ------------------------------------------------ tensor-core block SpMM --
// The FP32 multi-RHS products on the tensor pipes: mma.sync m16n8k8 with
// TF32 operands and FP32 accumulation, each FP32 value split into a high and
// a low TF32 part (x = hi + lo, lo = tf32(x - hi)) and each product formed as
// lo*hi + hi*lo + hi*hi ("3xTF32", about 2^-21 relative per product, the
// accuracy class of FP32).  One warp owns block row i and a tile of 64
// columns: the b x b block (b <= 16) is the 16 x 16 A operand (rows and
// columns beyond b are zero), the 64 columns of X_j eight 8-column B
// operands; the 16 x 64 accumulator tile stays in registers across the row's
// blocks.  MODE 1 (Jacobi) stages t = B_i - (A X)_i in shared memory and
// applies Dinv_i with the same split products.
__device__ __forceinline__ unsigned f2tf32(float x) {
    unsigned r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ void split_tf32(float x, unsigned& hi, unsigned& lo) {
    hi = f2tf32(x);
    lo = f2tf32(x - __uint_as_float(hi));
}
__device__ __forceinline__ void mma_tf32(float (&d)[4], const unsigned (&a)[4], const unsigned (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ void mma_3xtf32(float (&d)[4], const unsigned (&ah)[4], const unsigned (&al)[4],
                                           const unsigned (&bh)[2], const unsigned (&bl)[2]) {
    mma_tf32(d, al, bh);
    mma_tf32(d, ah, bl);
    mma_tf32(d, ah, bh);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// per-warp shared-memory stages of k_spmm_mma: the b x b block (16 x AS,
// zero beyond b) and the block's 16 x 64 slice of X (rows beyond b zero),
// twice (double buffering)
constexpr int kMmaWarps = 4;
constexpr int kMmaXS = 72;   // X row stride: conflict-free B-operand reads
constexpr int kMmaAS = 20;   // A row stride: conflict-free A-operand reads
struct MmaStage {
    float x[2][16 * kMmaXS];
    float a[2][16 * kMmaAS];
};

// issues the copies of block kk (its values and its X slice) into stage buf
template <int B>
__device__ __forceinline__ void mma_prefetch(const SpmmArgs<float>& a, int kk, int c0, MmaStage& st, int buf,
                                             int lane) {
    const float* A = a.val + (size_t)(a.blk ? a.blk[kk] : kk) * (B * B);
    for (int q = lane; q < B * B; q += 32) cp_async4(&st.a[buf][(q / B) * kMmaAS + q % B], A + q);
    const float* xb = a.X + (size_t)a.col_idx[kk] * B * a.k + c0;
    const int ncols = min(64, a.k - c0);   // a multiple of 4
    for (int q = lane; q < B * 16; q += 32) {
        const int r = q >> 4, c4 = (q & 15) * 4;
        if (c4 < ncols) cp_async16(&st.x[buf][r * kMmaXS + c4], xb + (size_t)r * a.k + c4);
    }
}

// A operand (rows g, g+8; columns 8 s + t, + 4) from a staged 16 x AS block
template <bool SPLIT>
__device__ __forceinline__ void a_frag_s(const float* As, int s, int g, int t, unsigned (&ah)[4], unsigned (&al)[4]) {
    const int ka = s * 8 + t;
    float v[4];
    v[0] = As[g * kMmaAS + ka];
    v[1] = As[(g + 8) * kMmaAS + ka];
    v[2] = As[g * kMmaAS + ka + 4];
    v[3] = As[(g + 8) * kMmaAS + ka + 4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if constexpr (SPLIT) split_tf32(v[q], ah[q], al[q]);
        else ah[q] = f2tf32(v[q]);
    }
}

// one k-step x n-tile product: split (3xTF32) or plain TF32
template <bool SPLIT>
__device__ __forceinline__ void mma_step(float (&d)[4], const unsigned (&ah)[4], const unsigned (&al)[4], float x0,
                                         float x1) {
    unsigned bh[2], bl[2];
    if constexpr (SPLIT) {
        split_tf32(x0, bh[0], bl[0]);
        split_tf32(x1, bh[1], bl[1]);
        mma_3xtf32(d, ah, al, bh, bl);
    } else {
        bh[0] = f2tf32(x0);
        bh[1] = f2tf32(x1);
        mma_tf32(d, ah, bh);
    }
}

template <int B, int MODE, bool SPLIT>
__global__ void __launch_bounds__(kMmaWarps * 32) k_spmm_mma(const SpmmArgs<float> a) {
    static_assert(B >= 1 && B <= 16, "tensor-core SpMM takes blocks up to 16 x 16");
    constexpr int KS = (B + 7) / 8;   // k-steps of 8
    __shared__ __align__(16) MmaStage stages[kMmaWarps];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, t = lane & 3;
    const int k = a.k;
    const int c0 = blockIdx.y * 64;
    MmaStage& st = stages[warp];
    // zero both stages once: rows and columns beyond b stay zero (finite)
    for (int q = lane; q < 2 * 16 * kMmaXS; q += 32) (&st.x[0][0])[q] = 0.f;
    for (int q = lane; q < 2 * 16 * kMmaAS; q += 32) (&st.a[0][0])[q] = 0.f;
    __syncwarp();
    for (int i = blockIdx.x * kMmaWarps + warp; i < a.nbr; i += gridDim.x * kMmaWarps) {
        float acc[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
            for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
        const int k0 = a.row_ptr[i], k1 = (MODE == 1 && a.xzero) ? k0 : a.row_ptr[i + 1];
        if (k0 < k1) mma_prefetch<B>(a, k0, c0, st, 0, lane);
        cp_async_commit();
        for (int kk = k0; kk < k1; ++kk) {
            const int buf = (kk - k0) & 1;
            if (kk + 1 < k1) mma_prefetch<B>(a, kk + 1, c0, st, buf ^ 1, lane);
            cp_async_commit();
            cp_async_wait<1>();   // block kk has landed (kk + 1 may be in flight)
            __syncwarp();
            const float* As = st.a[buf];
            const float* Xs = st.x[buf];
#pragma unroll
            for (int s = 0; s < KS; ++s) {
                unsigned ah[4], al[4];
                a_frag_s<SPLIT>(As, s, g, t, ah, al);
                const int ka = s * 8 + t;
#pragma unroll
                for (int nt = 0; nt < 8; ++nt)
                    mma_step<SPLIT>(acc[nt], ah, al, Xs[ka * kMmaXS + nt * 8 + g], Xs[(ka + 4) * kMmaXS + nt * 8 + g]);
            }
            __syncwarp();   // stage buf is rewritten by the prefetch two blocks on
        }
        cp_async_wait<0>();
        __syncwarp();
        const size_t y0 = (size_t)i * B * k;
        if constexpr (MODE == 0) {
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const int row = g + 8 * h, col = c0 + nt * 8 + 2 * t + e;
                        if (row < B && col < k) {
                            const size_t idx = y0 + (size_t)row * k + col;
                            float v = a.alpha * acc[nt][2 * h + e];
                            if (a.beta != 0.f) v += a.beta * a.Yin[idx];
                            a.Y[idx] = v;
                        }
                    }
        } else {
            // t = B_i - (A X)_i into stage 0's X slice (rows beyond b stay
            // zero), Dinv_i into stage 0's block, then Y_i = X_i + omega Dinv_i t
            float* T = st.x[0];
            float* Ds = st.a[0];
            const float* D = a.Dinv + (size_t)i * B * B;
            for (int q = lane; q < B * B; q += 32) Ds[(q / B) * kMmaAS + q % B] = __ldg(D + q);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const int row = g + 8 * h, cl = nt * 8 + 2 * t + e, col = c0 + cl;
                        if (row < B) T[row * kMmaXS + cl] = (col < k) ? a.B[y0 + (size_t)row * k + col] - acc[nt][2 * h + e] : 0.f;
                    }
            __syncwarp();
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int q = 0; q < 4; ++q) acc[nt][q] = 0.f;
#pragma unroll
            for (int s = 0; s < KS; ++s) {
                unsigned ah[4], al[4];
                a_frag_s<SPLIT>(Ds, s, g, t, ah, al);
                const int ka = s * 8 + t;
#pragma unroll
                for (int nt = 0; nt < 8; ++nt)
                    mma_step<SPLIT>(acc[nt], ah, al, T[ka * kMmaXS + nt * 8 + g], T[(ka + 4) * kMmaXS + nt * 8 + g]);
            }
            __syncwarp();
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int e = 0; e < 2; ++e) {
                        const int row = g + 8 * h, col = c0 + nt * 8 + 2 * t + e;
                        if (row < B && col < k) {
                            const size_t idx = y0 + (size_t)row * k + col;
                            a.Y[idx] = (a.xzero ? 0.f : a.X[idx]) + a.omega * acc[nt][2 * h + e];
                        }
                    }
        }
    }
}

static bool mma_shape(int br, int bc) { return br == bc && (br == 4 || br == 6 || br == 9 || br == 10 || br == 16); }

template <int B, int MODE, bool SPLIT>
static void launch_mma_t(mgldg_ctx* ctx, const SpmmArgs<float>& a, int kclass) {
    const int ncolt = (a.k + 63) / 64;
    int per_sm = 0;
    MG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmm_mma<B, MODE, SPLIT>, kMmaWarps * 32, 0));
    per_sm = std::max(1, per_sm);
    const int want = (a.nbr + kMmaWarps - 1) / kMmaWarps;
    const int gx = std::max(1, std::min(want, ctx->sm_count * per_sm * 4 / std::max(1, ncolt) + 1));
    {
        Launch L(ctx, kclass);
        k_spmm_mma<B, MODE, SPLIT><<<dim3(gx, ncolt), kMmaWarps * 32, 0, ctx->stream>>>(a);
    }
    check_launch();
}

// (the plain-TF32 instantiation, SPLIT = false, measured slower per sweep
// than the CUDA-core kernel as well and needed 10-30% more iterations; the
// form uses the split products)
template <int B, int MODE>
static void launch_mma(mgldg_ctx* ctx, const SpmmArgs<float>& a, int kclass) {
    launch_mma_t<B, MODE, true>(ctx, a, kclass);
}

static void spmm_mma(mgldg_ctx* ctx, int b, const SpmmArgs<float>& a, int mode, int kclass) {
#define MG_M(B)                                             \
    if (b == B) {                                           \
        if (mode == 0) launch_mma<B, 0>(ctx, a, kclass);   \
        else launch_mma<B, 1>(ctx, a, kclass);             \
        return;                                             \
    }
    MG_M(4) MG_M(6) MG_M(9) MG_M(10) MG_M(16)
#undef MG_M
    throw Error(MGLDG_ERR_UNSUPPORTED, "tensor-core SpMM: unsupported block size");
}

template <class T, int BR, int BC, int V, int MODE>
static void launch_tiled(mgldg_ctx* ctx, const SpmmArgs<T>& a, int wpb, int kclass) {
    const int ncolt = (a.k + 32 * V - 1) / (32 * V);
    const size_t smem = (size_t)wpb * Stage<BR, BC>::SIZE * sizeof(T);
    int per_sm = 0;
    MG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmm<T, BR, BC, V, MODE>, wpb * 32, smem));
    per_sm = std::max(1, per_sm);
    const int want = (a.nbr + wpb - 1) / wpb;
    const int gx = std::max(1, std::min(want, ctx->sm_count * per_sm * 4 / std::max(1, ncolt) + 1));
    dim3 grid(gx, ncolt);
    {
        Launch L(ctx, kclass);
        k_spmm<T, BR, BC, V, MODE><<<grid, wpb * 32, smem, ctx->stream>>>(a);
    }
    check_launch();
}

template <class T, int B, int MODE>
static bool dispatch_v(mgldg_ctx* ctx, const SpmmArgs<T>& a, const TileCfg& cfg, int kclass) {
    switch (cfg.V) {
        case 1: launch_tiled<T, B, B, 1, MODE>(ctx, a, cfg.wpb, kclass); return true;
        case 2: launch_tiled<T, B, B, 2, MODE>(ctx, a, cfg.wpb, kclass); return true;
        case 4:
            if constexpr (sizeof(T) == 4) {
                launch_tiled<T, B, B, 4, MODE>(ctx, a, cfg.wpb, kclass);
                return true;
            }
            return false;
        default: return false;
    }
}

static bool is_tiled_shape(int br, int bc) {
    return br == bc && (br == 4 || br == 6 || br == 9 || br == 10 || br == 16 || br == 25);
}

static bool aligned(const void* p, size_t a) { return p == nullptr || ((uintptr_t)p % a) == 0; }

// can this tile be used with these pointers and k
template <class T>
static bool tile_valid(const SpmmArgs<T>& a, int V) {
    if (a.k % V) return false;
    if (V == 4 && sizeof(T) != 4) return false;
    const size_t al = V * sizeof(T);
    return aligned(a.X, al) && aligned(a.Yin, al) && aligned(a.Y, al) && aligned(a.B, al);
}

template <class T>
static void spmm_launch(mgldg_ctx* ctx, int br, int bc, const SpmmArgs<T>& a, int mode, TileCfg cfg, int kclass) {
    if (a.nbr == 0 || a.k == 0) return;
    if constexpr (sizeof(T) == 4) {
        if (cfg.mma && mma_shape(br, bc) && a.k % 4 == 0 && aligned(a.X, 16)) {
            spmm_mma(ctx, br, a, mode, kclass);
            return;
        }
    }
    if (is_tiled_shape(br, bc) && tile_valid(a, cfg.V)) {
        bool ok = false;
#define MG_B(B)                                                                                        \
    if (br == B) ok = mode == 0 ? dispatch_v<T, B, 0>(ctx, a, cfg, kclass) : dispatch_v<T, B, 1>(ctx, a, cfg, kclass);
        MG_B(4) MG_B(6) MG_B(9) MG_B(10) MG_B(16) MG_B(25)
#undef MG_B
        if (ok) return;
    }
    MG_REQUIRE(mode == 0 || (br == bc && br <= 64), MGLDG_ERR_UNSUPPORTED, "Jacobi block size above 64");
    const int64_t total = (int64_t)a.nbr * a.k;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>((total + 255) / 256, ctx->sm_count * 16));
    {
        Launch L(ctx, kclass);
        if (mode == 0) k_spmm_generic<T, 0><<<g, 256, 0, ctx->stream>>>(a, br, bc);
        else k_spmm_generic<T, 1><<<g, 256, 0, ctx->stream>>>(a, br, bc);
    }
    check_launch();
}

template <class T>
static SpmmArgs<T> args_of(const mgldg_bsr* A, const T* vals, int k) {
    SpmmArgs<T> a{};
    a.nbr = A->nbr;
    a.row_ptr = A->row_ptr;
    a.col_idx = A->col_idx;
    a.val = vals;
    a.blk = A->blk;
    a.k = k;
    return a;
}

static TileCfg default_cfg(int k, size_t elem) {
    TileCfg c;
    c.V = (k % 2 == 0 && k >= 64) ? 2 : 1;
    (void)elem;
    return c;
}

// -------------------------------------------------------- column reductions
// partials[blockIdx.x * k + c] = sum over this CTA's rows of a[u,c] * b[u,c]
template <class T>
__global__ void __launch_bounds__(256) k_coldot(int64_t n, int k, const T* __restrict__ a, const T* __restrict__ b,
                                               double* __restrict__ partials) {
    __shared__ double sm[256];
    const int c0 = blockIdx.y * 256;
    const int kc = min(256, k - c0);
    const int rp = max(1, 256 / kc);          // rows per pass
    const int col = c0 + threadIdx.x % kc, ro = threadIdx.x / kc;
    double s = 0;
    if (ro < rp) {
        // four rows per round: their loads are in flight together
        const int64_t step = (int64_t)gridDim.x * rp;
        int64_t u = (int64_t)blockIdx.x * rp + ro;
        for (; u + 3 * step < n; u += 4 * step) {
            const double p0 = (double)a[u * k + col] * (double)b[u * k + col];
            const double p1 = (double)a[(u + step) * k + col] * (double)b[(u + step) * k + col];
            const double p2 = (double)a[(u + 2 * step) * k + col] * (double)b[(u + 2 * step) * k + col];
            const double p3 = (double)a[(u + 3 * step) * k + col] * (double)b[(u + 3 * step) * k + col];
            s += p0;
            s += p1;
            s += p2;
            s += p3;
        }
        for (; u < n; u += step) s += (double)a[u * k + col] * (double)b[u * k + col];
    }
    sm[threadIdx.x] = s;
    __syncthreads();
    if ((int)threadIdx.x < kc) {
        double t = 0;
        for (int q = 0; q < rp; ++q) t += sm[q * kc + threadIdx.x];
        partials[(size_t)blockIdx.x * k + c0 + threadIdx.x] = t;
    }
}

static int coldot_grid(mgldg_ctx* ctx, int64_t n) {
    return (int)std::max<int64_t>(1, std::min<int64_t>(n / 8 + 1, ctx->sm_count * 4));
}

template <class T>
static void coldot(mgldg_ctx* ctx, int64_t n, int k, const T* a, const T* b, double* partials, int* np) {
    const int g = coldot_grid(ctx, n);
    dim3 grid(g, (k + 255) / 256);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_coldot<T><<<grid, 256, 0, ctx->stream>>>(n, k, a, b, partials);
    }
    check_launch();
    *np = g;
}

// ------------------------------------------------------------ block PCG ----
struct BatchScalars {
    double *delta_new, *delta_old, *delta0, *alpha, *beta;
    int *active, *iters, *broken;
    int* counter;   // [0] = active columns after the iteration, [1] = broken,
                    // [2] = completed iterations (segmented PCG only)
};

__device__ double col_total(const double* partials, int np, int k, int c) {
    double s = 0;
    for (int p = 0; p < np; ++p) s += partials[(size_t)p * k + c];
    return s;
}

__global__ void k_bpcg_init(int k, BatchScalars sc, const double* partials, int np, double tol2, int maxit) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c == 0) { sc.counter[0] = 0; sc.counter[1] = 0; }
    if (c >= k) return;
    const double d = col_total(partials, np, k, c);
    sc.delta_new[c] = d;
    sc.delta0[c] = d;
    sc.iters[c] = 0;
    // r.z < 0 or NaN/inf: the preconditioner is not positive definite or failed
    sc.broken[c] = (d < 0.0 || !isfinite(d)) ? 1 : 0;
    sc.active[c] = (maxit > 0 && d > tol2 * d && !sc.broken[c]) ? 1 : 0;
}

__global__ void k_bpcg_count(int k, BatchScalars sc) {
    __shared__ int cnt[2];
    if (threadIdx.x < 2) cnt[threadIdx.x] = 0;
    __syncthreads();
    for (int c = threadIdx.x; c < k; c += blockDim.x) {
        if (sc.active[c]) atomicAdd(&cnt[0], 1);
        if (sc.broken[c]) atomicAdd(&cnt[1], 1);
    }
    __syncthreads();
    if (threadIdx.x < 2) sc.counter[threadIdx.x] = cnt[threadIdx.x];
}

__global__ void k_bpcg_alpha(int k, BatchScalars sc, const double* partials, int np) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    double a = 0;
    if (sc.active[c]) {
        const double dq = col_total(partials, np, k, c);
        a = sc.delta_new[c] / dq;
        if (!(dq > 0.0) || !isfinite(a)) {
            sc.broken[c] = 1;
            sc.active[c] = 0;
            a = 0;
        }
    }
    sc.alpha[c] = a;
}

// x += alpha d ; r -= alpha q (update_r), active columns only
__global__ void __launch_bounds__(256) k_bpcg_update(int64_t nk, int k, BatchScalars sc, const double* __restrict__ d,
                                                     const double* __restrict__ q, double* __restrict__ x,
                                                     double* __restrict__ r, int update_r) {
    const int64_t stride = (int64_t)gridDim.x * 256;
    const int dc = (int)(stride % k);
    int64_t e = (int64_t)blockIdx.x * 256 + threadIdx.x;
    int c = (int)(e % k);
    for (; e < nk; e += stride, c = (c + dc >= k) ? c + dc - k : c + dc) {
        if (!sc.active[c]) continue;
        const double al = sc.alpha[c];
        x[e] += al * d[e];
        if (update_r) r[e] -= al * q[e];
    }
}

// it < 0: the iteration index is the device-side counter[2]
__global__ void k_bpcg_rr(int k, BatchScalars sc, const double* partials, int np, double* hist, int maxit, int it) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k || !sc.active[c]) return;
    hist[(size_t)c * maxit + (it >= 0 ? it : sc.counter[2])] = sqrt(col_total(partials, np, k, c));
}

__global__ void k_bpcg_beta(int k, BatchScalars sc, const double* partials, int np) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= k) return;
    double b = 0;
    if (sc.active[c]) {
        const double rs = col_total(partials, np, k, c);
        sc.delta_old[c] = sc.delta_new[c];
        sc.delta_new[c] = rs;
        b = rs / sc.delta_old[c];
        if (!isfinite(b) || rs < 0.0) {   // r.z < 0: preconditioner not positive definite
            sc.broken[c] = 1;
            sc.active[c] = 0;
            b = 0;
        }
    }
    sc.beta[c] = b;
}

// d = s + beta d (active columns)
__global__ void __launch_bounds__(256) k_bpcg_dir(int64_t nk, int k, BatchScalars sc, const double* __restrict__ s,
                                                  double* __restrict__ d) {
    const int64_t stride = (int64_t)gridDim.x * 256;
    const int dc = (int)(stride % k);
    int64_t e = (int64_t)blockIdx.x * 256 + threadIdx.x;
    int c = (int)(e % k);
    for (; e < nk; e += stride, c = (c + dc >= k) ? c + dc - k : c + dc) {
        if (sc.active[c]) d[e] = s[e] + sc.beta[c] * d[e];
    }
}

__global__ void k_bpcg_end(int k, BatchScalars sc, double tol2, int maxit, int it) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (it < 0) it = sc.counter[2];
    if (c >= k || !sc.active[c]) return;
    sc.iters[c] = it + 1;
    sc.active[c] = (it + 1 < maxit && sc.delta_new[c] > tol2 * sc.delta0[c]) ? 1 : 0;
}

// ---------------------------------------------------- multi-RHS coarse solve
// one CTA per column: (b -= mean(b)); x = Cinv b, FP64 accumulation
template <class T>
__global__ void __launch_bounds__(256) k_bcoarse(int n, int k, T* b, T* x, const double* __restrict__ Cinv,
                                                int mean_project, int solve) {
    extern __shared__ double sb[];   // n doubles when solving, unused otherwise
    __shared__ double red[8];
    const int c = blockIdx.x;
    double s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const double v = (double)b[(size_t)i * k + c];
        if (solve) sb[i] = v;
        s += v;
    }
    if (mean_project) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
        __syncthreads();
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        const double mean = t / n;
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            const double v = (solve ? sb[i] : (double)b[(size_t)i * k + c]) - mean;
            if (solve) sb[i] = v;
            b[(size_t)i * k + c] = (T)v;
        }
    }
    __syncthreads();
    if (!solve) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int row = w; row < n; row += nw) {
        double a = 0;
        for (int cc = lane; cc < n; cc += 32) a += Cinv[(size_t)row * n + cc] * sb[cc];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) x[(size_t)row * k + c] = (T)a;
    }
}

template <class A, class B>
__global__ void k_bconvert(int64_t n, const A* __restrict__ a, B* __restrict__ b) {
    for (int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x; i < n; i += (int64_t)gridDim.x * 256) b[i] = (B)a[i];
}

// --------------------------------------------------------------- work space
struct BatchLevel {
    double *x = nullptr, *b = nullptr, *r = nullptr, *xt = nullptr;
    float *x32 = nullptr, *b32 = nullptr, *r32 = nullptr, *xt32 = nullptr;
    TileCfg spmm, jac, restrict_, prolong;
};

struct Batch {
    int k = 0;
    std::vector<BatchLevel> L;
    TileCfg outer;   // FP64 SpMM of the outer CG
    const mgldg_bsr* outer_A = nullptr;
    bool tuned = false;
    // block PCG
    double *R = nullptr, *D = nullptr, *Q = nullptr, *S = nullptr, *hist = nullptr;
    float *Dhi = nullptr, *Dlo = nullptr;   // D as float pairs (mixed forms' double-float Q = A D)
    int64_t pcg_nk = 0;
    int hist_len = 0;
    double* partials = nullptr;
    int partials_len = 0;
    BatchScalars sc{};
    double* sc_mem = nullptr;
    int* sc_int = nullptr;
    int* h_counter = nullptr;   // pinned
};

template <class T>
struct BL;
template <>
struct BL<double> {
    static double*& x(BatchLevel& L) { return L.x; }
    static double*& b(BatchLevel& L) { return L.b; }
    static double*& r(BatchLevel& L) { return L.r; }
    static double*& xt(BatchLevel& L) { return L.xt; }
    static const double* D(LevelData& L) { return L.Dinv; }
};
template <>
struct BL<float> {
    static float*& x(BatchLevel& L) { return L.x32; }
    static float*& b(BatchLevel& L) { return L.b32; }
    static float*& r(BatchLevel& L) { return L.r32; }
    static float*& xt(BatchLevel& L) { return L.xt32; }
    static const float* D(LevelData& L) { return L.Dinv32; }
};

void batch_free(Batch* b) {
    if (!b) return;
    for (auto& L : b->L) {
        dfree(L.x); dfree(L.b); dfree(L.r); dfree(L.xt);
        dfree(L.x32); dfree(L.b32); dfree(L.r32); dfree(L.xt32);
    }
    dfree(b->R); dfree(b->D); dfree(b->Q); dfree(b->S); dfree(b->hist); dfree(b->Dhi); dfree(b->Dlo);
    dfree(b->partials);
    dfree(b->sc_mem);
    dfree(b->sc_int);
    if (b->h_counter) cudaFreeHost(b->h_counter);
    delete b;
}

// times fn() (one launch sequence) on the library stream, best of 3
template <class F>
static float time_best(mgldg_ctx* ctx, F fn) {
    cudaEvent_t e0, e1;
    MG_CHECK_CUDA(cudaEventCreate(&e0));
    MG_CHECK_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    try {
        fn();   // warm-up (and first-use setup)
        for (int rep = 0; rep < 3; ++rep) {
            MG_CHECK_CUDA(cudaEventRecord(e0, ctx->stream));
            fn();
            MG_CHECK_CUDA(cudaEventRecord(e1, ctx->stream));
            MG_CHECK_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            MG_CHECK_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return best;
}

// picks the fastest valid tile for one operator / mode on scratch buffers
template <class T>
static TileCfg autotune(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, int k, int mode, const T* X, T* Y,
                        const T* Dinv, const T* B) {
    SpmmArgs<T> a = args_of<T>(A, vals, k);
    a.alpha = T(1);
    a.beta = T(0);
    a.X = X;
    a.Y = Y;
    a.Dinv = Dinv;
    a.B = B;
    a.omega = T(0.5);
    TileCfg best = default_cfg(k, sizeof(T));
    if (!is_tiled_shape(A->br, A->bc) || A->nbr == 0) return best;
    float tbest = 1e30f;
    const bool prof = ctx->prof;
    ctx->prof = false;   // tuning launches are not solver work
    int64_t saved[MGLDG_K_NCLASS];
    std::memcpy(saved, ctx->launches, sizeof saved);
    try {
        for (int V : {1, 2, 4}) {
            if (!tile_valid(a, V)) continue;
            if (V > 1 && 32 * V > (k + 31) / 32 * 32) continue;   // a tile wider than the columns
            for (int wpb : {4, 8}) {
                TileCfg c;
                c.V = V;
                c.wpb = wpb;
                float t = time_best(ctx, [&] { spmm_launch<T>(ctx, A->br, A->bc, a, mode, c, MGLDG_K_SETUP); });
                if (t < tbest) {
                    tbest = t;
                    best = c;
                }
            }
        }
    } catch (...) {
        ctx->prof = prof;
        std::memcpy(ctx->launches, saved, sizeof saved);
        throw;
    }
    ctx->prof = prof;
    std::memcpy(ctx->launches, saved, sizeof saved);
    return best;
}

static void ensure_batch(mgldg_mg* m, int k, const mgldg_bsr* A_outer) {
    mgldg_ctx* ctx = m->ctx;
    if (m->batch && m->batch->k != k) {
        batch_free(m->batch);
        m->batch = nullptr;
    }
    if (!m->batch) {
        Batch* b = new Batch();
        b->k = k;
        m->batch = b;
        b->L.resize(m->L.size());
        const bool mixed = m->p.precision != MGLDG_PREC_FP64;
        for (size_t l = 0; l < m->L.size(); ++l) {
            const int64_t nk = std::max<int64_t>(1, m->L[l].n * k);
            BatchLevel& B = b->L[l];
            if (mixed) {
                B.x32 = dalloc<float>(nk); B.b32 = dalloc<float>(nk);
                B.r32 = dalloc<float>(nk); B.xt32 = dalloc<float>(nk);
                MG_CHECK_CUDA(cudaMemsetAsync(B.x32, 0, nk * sizeof(float), ctx->stream));
                MG_CHECK_CUDA(cudaMemsetAsync(B.b32, 0, nk * sizeof(float), ctx->stream));
            } else {
                B.x = dalloc<double>(nk); B.b = dalloc<double>(nk);
                B.r = dalloc<double>(nk); B.xt = dalloc<double>(nk);
                MG_CHECK_CUDA(cudaMemsetAsync(B.x, 0, nk * sizeof(double), ctx->stream));
                MG_CHECK_CUDA(cudaMemsetAsync(B.b, 0, nk * sizeof(double), ctx->stream));
            }
        }
        b->sc_mem = dalloc<double>(5 * (size_t)k);
        b->sc_int = dalloc<int>(3 * (size_t)k + 2);
        b->sc.delta_new = b->sc_mem;
        b->sc.delta_old = b->sc_mem + k;
        b->sc.delta0 = b->sc_mem + 2 * k;
        b->sc.alpha = b->sc_mem + 3 * k;
        b->sc.beta = b->sc_mem + 4 * k;
        b->sc.active = b->sc_int;
        b->sc.iters = b->sc_int + k;
        b->sc.broken = b->sc_int + 2 * k;
        b->sc.counter = b->sc_int + 3 * k;
        MG_CHECK_CUDA(cudaMallocHost(&b->h_counter, 2 * sizeof(int)));
        b->partials_len = ctx->sm_count * 4 * k;   // coldot_grid partial rows per column
        b->partials = dalloc<double>(b->partials_len);
    }
    Batch* b = m->batch;
    if (!b->tuned) {
        // tile widths per level operator and kernel, on the level buffers
        // (their contents are overwritten before every use)
        const bool mixed = m->p.precision != MGLDG_PREC_FP64;
        for (size_t l = 0; l < m->L.size(); ++l) {
            LevelData& L = m->L[l];
            BatchLevel& B = b->L[l];
            if (mixed) {
                if (m->p.precision == MGLDG_PREC_MIXED_TF32 && !L.A->blk && mma_shape(L.A->br, L.A->bc)) {
                    // the level operator's products on the tensor pipes (no
                    // timing choice: the form fixes the arithmetic)
                    B.spmm.mma = B.jac.mma = true;
                } else {
                    B.spmm = autotune<float>(ctx, L.A, bsr_vals<float>(L.A), k, 0, B.x32, B.r32, nullptr, nullptr);
                    if (L.Dinv32)
                        B.jac = autotune<float>(ctx, L.A, bsr_vals<float>(L.A), k, 1, B.x32, B.xt32, L.Dinv32, B.b32);
                }
                if (l + 1 < m->L.size()) {
                    BatchLevel& C = b->L[l + 1];
                    B.restrict_ = autotune<float>(ctx, L.Tt, bsr_vals<float>(L.Tt), k, 0, B.r32, C.b32, nullptr, nullptr);
                    B.prolong = autotune<float>(ctx, L.T, bsr_vals<float>(L.T), k, 0, C.x32, B.xt32, nullptr, nullptr);
                }
            } else {
                B.spmm = autotune<double>(ctx, L.A, bsr_vals<double>(L.A), k, 0, B.x, B.r, nullptr, nullptr);
                if (L.Dinv) B.jac = autotune<double>(ctx, L.A, bsr_vals<double>(L.A), k, 1, B.x, B.xt, L.Dinv, B.b);
                if (l + 1 < m->L.size()) {
                    BatchLevel& C = b->L[l + 1];
                    B.restrict_ = autotune<double>(ctx, L.Tt, bsr_vals<double>(L.Tt), k, 0, B.r, C.b, nullptr, nullptr);
                    B.prolong = autotune<double>(ctx, L.T, bsr_vals<double>(L.T), k, 0, C.x, B.xt, nullptr, nullptr);
                }
            }
        }
        b->tuned = true;
    }
    if (A_outer && b->outer_A != A_outer) {
        const int64_t nk = (int64_t)A_outer->nbr * A_outer->br * k;
        double* s1 = dalloc<double>(std::max<int64_t>(1, nk));
        double* s2 = dalloc<double>(std::max<int64_t>(1, nk));
        try {
            MG_CHECK_CUDA(cudaMemsetAsync(s1, 0, nk * sizeof(double), ctx->stream));
            b->outer = autotune<double>(ctx, A_outer, bsr_vals<double>(A_outer), k, 0, s1, s2, nullptr, nullptr);
            sync(ctx);
        } catch (...) {
            dfree(s1);
            dfree(s2);
            throw;
        }
        dfree(s1);
        dfree(s2);
        b->outer_A = A_outer;
    }
}

// ------------------------------------------------------- multi-RHS V-cycle
// n Jacobi sweeps on level l; xzero: x is zero and not materialised
template <class T>
static void brelax(mgldg_mg* m, int l, int n, bool xzero = false) {
    LevelData& L = m->L[l];
    BatchLevel& B = m->batch->L[l];
    mgldg_ctx* ctx = m->ctx;
    ctx->cur_level = l;
    MG_REQUIRE(m->p.relaxation == MGLDG_RELAX_JACOBI, MGLDG_ERR_UNSUPPORTED,
               "the multi-RHS V-cycle smooths with block Jacobi only");
    for (int s = 0; s < n; ++s) {
        SpmmArgs<T> a = args_of<T>(L.A, bsr_vals<T>(L.A), m->batch->k);
        a.X = BL<T>::x(B);
        a.Y = BL<T>::xt(B);
        a.Dinv = BL<T>::D(L);
        a.B = BL<T>::b(B);
        a.omega = (T)m->p.omega;
        a.xzero = (xzero && s == 0) ? 1 : 0;
        spmm_launch<T>(ctx, L.A->br, L.A->bc, a, 1, B.jac, MGLDG_K_JACOBI);
        std::swap(BL<T>::x(B), BL<T>::xt(B));
    }
}

template <class T>
static void bcoarse(mgldg_mg* m, int l, bool xzero) {
    LevelData& L = m->L[l];
    BatchLevel& B = m->batch->L[l];
    mgldg_ctx* ctx = m->ctx;
    const int k = m->batch->k;
    ctx->cur_level = l;
    if (m->p.solver == MGLDG_COARSE_RELAXATION) {
        if (m->p.mean_project) {
            Launch K(ctx, MGLDG_K_COARSE);
            k_bcoarse<T><<<k, 256, 0, ctx->stream>>>((int)L.n, k, BL<T>::b(B), BL<T>::x(B), nullptr, 1, 0);
        }
        check_launch();
        brelax<T>(m, l, m->p.npre, xzero);
        brelax<T>(m, l, m->p.npost);
        return;
    }
    {
        Launch K(ctx, MGLDG_K_COARSE);
        k_bcoarse<T><<<k, 256, L.n * sizeof(double), ctx->stream>>>((int)L.n, k, BL<T>::b(B), BL<T>::x(B), m->Cinv,
                                                                    m->p.mean_project, 1);
    }
    check_launch();
}

template <class T>
static void bvcycle(mgldg_mg* m, int l, bool xzero) {
    mgldg_ctx* ctx = m->ctx;
    if (l == (int)m->L.size() - 1) {
        bcoarse<T>(m, l, xzero);
        return;
    }
    LevelData& L = m->L[l];
    BatchLevel& B = m->batch->L[l];
    BatchLevel& C = m->batch->L[l + 1];
    const int k = m->batch->k;
    brelax<T>(m, l, m->p.npre, xzero);
    ctx->cur_level = l;
    {
        // r = b - A x
        SpmmArgs<T> a = args_of<T>(L.A, bsr_vals<T>(L.A), k);
        a.alpha = T(-1);
        a.beta = T(1);
        a.X = BL<T>::x(B);
        a.Yin = BL<T>::b(B);
        a.Y = BL<T>::r(B);
        spmm_launch<T>(ctx, L.A->br, L.A->bc, a, 0, B.spmm, MGLDG_K_SPMV);
    }
    {
        // b_c = T^T r
        SpmmArgs<T> a = args_of<T>(L.Tt, bsr_vals<T>(L.Tt), k);
        a.alpha = T(1);
        a.beta = T(0);
        a.X = BL<T>::r(B);
        a.Y = BL<T>::b(C);
        spmm_launch<T>(ctx, L.Tt->br, L.Tt->bc, a, 0, B.restrict_, MGLDG_K_TRANSFER);
    }
    const bool czero = zero_start(m, l + 1);
    if (!czero) MG_CHECK_CUDA(cudaMemsetAsync(BL<T>::x(C), 0, m->L[l + 1].n * k * sizeof(T), ctx->stream));
    bvcycle<T>(m, l + 1, czero);
    ctx->cur_level = l;
    {
        // x += T x_c
        SpmmArgs<T> a = args_of<T>(L.T, bsr_vals<T>(L.T), k);
        a.alpha = T(1);
        a.beta = T(1);
        a.X = BL<T>::x(C);
        a.Yin = BL<T>::x(B);
        a.Y = BL<T>::x(B);
        spmm_launch<T>(ctx, L.T->br, L.T->bc, a, 0, B.prolong, MGLDG_K_TRANSFER);
    }
    brelax<T>(m, l, m->p.npost);
}

template <class A, class B>
static void bconvert(mgldg_ctx* ctx, int64_t n, const A* a, B* b) {
    if (n == 0) return;
    const int g = (int)std::min<int64_t>((n + 255) / 256, ctx->sm_count * 16);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bconvert<A, B><<<g, 256, 0, ctx->stream>>>(n, a, b);
    }
    check_launch();
}

// S = V-cycle(R) from a zero initial guess (x_is_zero) or from S
static void bprecon(mgldg_mg* m, const double* R, double* S, bool x_is_zero) {
    mgldg_ctx* ctx = m->ctx;
    Batch* b = m->batch;
    const int64_t nk = m->L[0].n * b->k;
    BatchLevel& B = b->L[0];
    struct LevelReset {
        mgldg_ctx* c;
        ~LevelReset() { c->cur_level = -1; }
    } reset{ctx};
    if (m->p.precision != MGLDG_PREC_FP64) {
        bconvert<double, float>(ctx, nk, R, B.b32);
        const bool z = x_is_zero && zero_start(m, 0);
        if (x_is_zero && !z) MG_CHECK_CUDA(cudaMemsetAsync(B.x32, 0, nk * sizeof(float), ctx->stream));
        else if (!x_is_zero) bconvert<double, float>(ctx, nk, S, B.x32);
        bvcycle<float>(m, 0, z);
        bconvert<float, double>(ctx, nk, B.x32, S);
    } else {
        MG_CHECK_CUDA(cudaMemcpyAsync(B.b, R, nk * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        const bool z = x_is_zero && zero_start(m, 0);
        if (x_is_zero && !z) MG_CHECK_CUDA(cudaMemsetAsync(B.x, 0, nk * sizeof(double), ctx->stream));
        else if (!x_is_zero)
            MG_CHECK_CUDA(cudaMemcpyAsync(B.x, S, nk * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
        bvcycle<double>(m, 0, z);
        MG_CHECK_CUDA(cudaMemcpyAsync(S, B.x, nk * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    }
}

// ------------------------------------------- double-float outer SpMM (mixed) --
// Q = A D for the mixed forms on the FP32 pipes: A = val32 + lo32 and D =
// Dhi + Dlo as float pairs, each product exact in its high part (FMA error
// recovery) plus the cross terms, two-sum accumulation with explicitly
// rounded operations (about 2^-44 relative), Q in FP64.  One warp per block
// row, both halves of each block staged (transposed) in shared memory, the
// lane owning V consecutive columns of the column tile.
__device__ __forceinline__ void df_acc(float& sh, float& sl, float ah, float al, float dh, float dl) {
    const float p = __fmul_rn(ah, dh);
    const float pe = fmaf(ah, dh, -p);
    const float t = fmaf(ah, dl, fmaf(al, dh, pe));
    const float s = __fadd_rn(sh, p);
    const float bb = __fsub_rn(s, sh);
    const float e = __fadd_rn(__fsub_rn(sh, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    sh = s;
    sl = __fadd_rn(sl, __fadd_rn(e, t));
}

template <int B, int V>
__global__ void __launch_bounds__(256) k_spmm_df64(int nbr, const int* __restrict__ row_ptr,
                                                   const int* __restrict__ col_idx, const float* __restrict__ ahi,
                                                   const float* __restrict__ alo, const float* __restrict__ Dhi,
                                                   const float* __restrict__ Dlo, int k, double* __restrict__ Q) {
    using S = Stage<B, B>;
    extern __shared__ __align__(16) unsigned char smraw[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    float* sth = reinterpret_cast<float*>(smraw) + (size_t)warp * 2 * S::SIZE;
    float* stl = sth + S::SIZE;
    const int c = (blockIdx.y * 32 + lane) * V;
    const bool cok = c < k;
    for (int i = blockIdx.x * wpb + warp; i < nbr; i += gridDim.x * wpb) {
        float sh[B][V], sl[B][V];
#pragma unroll
        for (int r = 0; r < B; ++r)
#pragma unroll
            for (int v = 0; v < V; ++v) sh[r][v] = sl[r][v] = 0.f;
        const int k0 = row_ptr[i], k1 = row_ptr[i + 1];
        for (int kk = k0; kk < k1; ++kk) {
            const int j = col_idx[kk];
            float ph[S::PER], pl[S::PER];
            stage_fetch<float, B, B>(ahi + (size_t)kk * (B * B), lane, ph);
            stage_fetch<float, B, B>(alo + (size_t)kk * (B * B), lane, pl);
            __syncwarp();
            stage_store<float, B, B>(sth, lane, ph);
            stage_store<float, B, B>(stl, lane, pl);
            __syncwarp();
            if (cok) {
                const size_t xb = (size_t)j * B * k + c;
#pragma unroll
                for (int cc = 0; cc < B; ++cc) {
                    float xh[V], xl[V];
                    VecIO<float, V>::ld(Dhi + xb + (size_t)cc * k, xh);
                    VecIO<float, V>::ld(Dlo + xb + (size_t)cc * k, xl);
#pragma unroll
                    for (int r = 0; r < B; ++r) {
                        const float ah = sth[cc * S::BRP + r], al = stl[cc * S::BRP + r];
#pragma unroll
                        for (int v = 0; v < V; ++v) df_acc(sh[r][v], sl[r][v], ah, al, xh[v], xl[v]);
                    }
                }
            }
        }
        if (cok) {
            const size_t y0 = (size_t)i * B * k + c;
#pragma unroll
            for (int r = 0; r < B; ++r)
#pragma unroll
                for (int v = 0; v < V; ++v) Q[y0 + (size_t)r * k + v] = (double)sh[r][v] + (double)sl[r][v];
        }
    }
}

// float pair of D (all columns, or the active ones after a direction update)
__global__ void __launch_bounds__(256) k_bsplit(int64_t nk, const double* __restrict__ d, float* __restrict__ hi,
                                                float* __restrict__ lo) {
    for (int64_t e = (int64_t)blockIdx.x * 256 + threadIdx.x; e < nk; e += (int64_t)gridDim.x * 256) {
        const double v = d[e];
        const float h = (float)v;
        hi[e] = h;
        lo[e] = (float)(v - (double)h);
    }
}

__global__ void __launch_bounds__(256) k_bpcg_dir_split(int64_t nk, int k, BatchScalars sc, const double* __restrict__ s,
                                                        double* __restrict__ d, float* __restrict__ hi,
                                                        float* __restrict__ lo) {
    const int64_t stride = (int64_t)gridDim.x * 256;
    const int dc = (int)(stride % k);
    int64_t e = (int64_t)blockIdx.x * 256 + threadIdx.x;
    int c = (int)(e % k);
    for (; e < nk; e += stride, c = (c + dc >= k) ? c + dc - k : c + dc) {
        if (sc.active[c]) {
            const double v = s[e] + sc.beta[c] * d[e];
            d[e] = v;
            const float h = (float)v;
            hi[e] = h;
            lo[e] = (float)(v - (double)h);
        }
    }
}

static bool df64_batch_ok(const mgldg_mg* m, const mgldg_bsr* A) {
    const Batch* b = m->batch;
    return m->p.precision != MGLDG_PREC_FP64 && b->Dhi && A->val32 && A->lo32 && !A->blk && A->br == A->bc &&
           (A->br == 4 || A->br == 6 || A->br == 9 || A->br == 10 || A->br == 16);
}

template <int B>
static void launch_spmm_df64(mgldg_ctx* ctx, const mgldg_bsr* A, const float* Dhi, const float* Dlo, int k, double* Q) {
    constexpr int wpb = 8;
    const bool v2 = k % 2 == 0 && k >= 64;
    const int V = v2 ? 2 : 1;
    const int ncolt = (k + 32 * V - 1) / (32 * V);
    const size_t smem = (size_t)wpb * 2 * Stage<B, B>::SIZE * sizeof(float);
    const int gx = std::max(1, std::min((A->nbr + wpb - 1) / wpb, ctx->sm_count * 16 / std::max(1, ncolt) + 1));
    dim3 grid(gx, ncolt);
    {
        Launch L(ctx, MGLDG_K_SPMV);
        if (v2) k_spmm_df64<B, 2><<<grid, wpb * 32, smem, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, A->val32,
                                                                          A->lo32, Dhi, Dlo, k, Q);
        else k_spmm_df64<B, 1><<<grid, wpb * 32, smem, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, A->val32,
                                                                       A->lo32, Dhi, Dlo, k, Q);
    }
    check_launch();
}

static void outer_spmm_df64(mgldg_mg* m, const mgldg_bsr* A, double* Q) {
    const Batch* b = m->batch;
    switch (A->br) {
        case 4: launch_spmm_df64<4>(m->ctx, A, b->Dhi, b->Dlo, b->k, Q); return;
        case 6: launch_spmm_df64<6>(m->ctx, A, b->Dhi, b->Dlo, b->k, Q); return;
        case 9: launch_spmm_df64<9>(m->ctx, A, b->Dhi, b->Dlo, b->k, Q); return;
        case 10: launch_spmm_df64<10>(m->ctx, A, b->Dhi, b->Dlo, b->k, Q); return;
        case 16: launch_spmm_df64<16>(m->ctx, A, b->Dhi, b->Dlo, b->k, Q); return;
    }
    throw Error(MGLDG_ERR_UNSUPPORTED, "double-float SpMM: unsupported block size");
}

static void outer_spmm(mgldg_mg* m, const mgldg_bsr* A, double alpha, const double* X, double beta, const double* Yin,
                       double* Y) {
    SpmmArgs<double> a = args_of<double>(A, bsr_vals<double>(A), m->batch->k);
    a.alpha = alpha;
    a.beta = beta;
    a.X = X;
    a.Yin = Yin;
    a.Y = Y;
    spmm_launch<double>(m->ctx, A->br, A->bc, a, 0, m->batch->outer, MGLDG_K_SPMV);
}

static void ensure_bpcg(mgldg_mg* m, int64_t nk, int maxit) {
    Batch* b = m->batch;
    if (b->pcg_nk != nk) {
        dfree(b->R); dfree(b->D); dfree(b->Q); dfree(b->S); dfree(b->Dhi); dfree(b->Dlo);
        b->R = nullptr; b->D = nullptr; b->Q = nullptr; b->S = nullptr; b->Dhi = nullptr; b->Dlo = nullptr;
        b->R = dalloc<double>(nk); b->D = dalloc<double>(nk); b->Q = dalloc<double>(nk); b->S = dalloc<double>(nk);
        if (m->p.precision != MGLDG_PREC_FP64) {
            b->Dhi = dalloc<float>(nk);
            b->Dlo = dalloc<float>(nk);
        }
        b->pcg_nk = nk;
    }
    const int len = std::max(1, maxit) * b->k;
    if (b->hist_len < len) {
        dfree(b->hist);
        b->hist = nullptr;
        b->hist = dalloc<double>(len);
        b->hist_len = len;
    }
}

static void take_batch_errors(mgldg_mg* m) { take_device_error(m->ctx); }

// lock-step block PCG (krylov.h:22-68 per column)
static void bpcg(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, int k, const double* B, double* X, double tol,
                 int maxit, int* iters, double* res_hist) {
    const int64_t n = (int64_t)A->nbr * A->br;
    const int64_t nk = n * k;
    ensure_batch(m, k, A);
    ensure_bpcg(m, nk, maxit);
    Batch* b = m->batch;
    BatchScalars sc = b->sc;
    const int gk = (k + 127) / 128;
    const int gvec = (int)std::max<int64_t>(1, std::min<int64_t>((nk + 255) / 256, ctx->sm_count * 16));
    const double tol2 = tol * tol;
    int np = 0;
    // R = B - A X ; D = M(R) ; delta = colsum(R o D)
    const bool df = df64_batch_ok(m, A);
    outer_spmm(m, A, -1.0, X, 1.0, B, b->R);
    bprecon(m, b->R, b->D, true);
    coldot<double>(ctx, n, k, b->R, b->D, b->partials, &np);
    if (df) {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bsplit<<<gvec, 256, 0, ctx->stream>>>(nk, b->D, b->Dhi, b->Dlo);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_init<<<gk, 128, 0, ctx->stream>>>(k, sc, b->partials, np, tol2, maxit);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_count<<<1, 256, 0, ctx->stream>>>(k, sc);
    }
    check_launch();
    MG_CHECK_CUDA(cudaMemcpyAsync(b->h_counter, sc.counter, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    sync(ctx);
    take_batch_errors(m);
    int i = 0;
    while (b->h_counter[0] > 0) {
        // Q = A D ; alpha = delta / colsum(D o Q)
        if (df) outer_spmm_df64(m, A, b->Q);
        else outer_spmm(m, A, 1.0, b->D, 0.0, nullptr, b->Q);
        coldot<double>(ctx, n, k, b->D, b->Q, b->partials, &np);
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_bpcg_alpha<<<gk, 128, 0, ctx->stream>>>(k, sc, b->partials, np);
        }
        check_launch();
        const bool replace = i % 50 == 0;
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_bpcg_update<<<gvec, 256, 0, ctx->stream>>>(nk, k, sc, b->D, b->Q, X, b->R, replace ? 0 : 1);
        }
        check_launch();
        if (replace) outer_spmm(m, A, -1.0, X, 1.0, B, b->R);
        coldot<double>(ctx, n, k, b->R, b->R, b->partials, &np);
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_bpcg_rr<<<gk, 128, 0, ctx->stream>>>(k, sc, b->partials, np, b->hist, maxit, i);
        }
        check_launch();
        // S = M(R) ; delta_new = colsum(R o S) ; beta ; D = S + beta D
        bprecon(m, b->R, b->S, true);
        coldot<double>(ctx, n, k, b->R, b->S, b->partials, &np);
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_bpcg_beta<<<gk, 128, 0, ctx->stream>>>(k, sc, b->partials, np);
        }
        check_launch();
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            if (df) k_bpcg_dir_split<<<gvec, 256, 0, ctx->stream>>>(nk, k, sc, b->S, b->D, b->Dhi, b->Dlo);
            else k_bpcg_dir<<<gvec, 256, 0, ctx->stream>>>(nk, k, sc, b->S, b->D);
        }
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_bpcg_end<<<gk, 128, 0, ctx->stream>>>(k, sc, tol2, maxit, i);
        }
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_bpcg_count<<<1, 256, 0, ctx->stream>>>(k, sc);
        }
        check_launch();
        MG_CHECK_CUDA(cudaMemcpyAsync(b->h_counter, sc.counter, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        sync(ctx);
        ++i;
    }
    take_batch_errors(m);
    std::vector<int> it(k);
    download(ctx, it.data(), sc.iters, k);
    std::vector<int> broken(k);
    download(ctx, broken.data(), sc.broken, k);
    sync(ctx);
    if (iters) std::copy(it.begin(), it.end(), iters);
    if (res_hist && maxit > 0) {
        download(ctx, res_hist, b->hist, (int64_t)maxit * k);
        sync(ctx);
    }
    for (int c = 0; c < k; ++c)
        if (broken[c]) throw Error(MGLDG_ERR_BREAKDOWN, "pcg breakdown in column " + std::to_string(c));
}

static void require_batch(mgldg_mg* m, int k) {
    MG_REQUIRE(k >= 1 && k <= kMaxCols, MGLDG_ERR_ARG, "k must be in 1..1024");
    MG_REQUIRE(m && !m->L.empty(), MGLDG_ERR_ARG, "multi-RHS solves need a multigrid preconditioner");
    MG_REQUIRE(m->p.relaxation == MGLDG_RELAX_JACOBI, MGLDG_ERR_UNSUPPORTED,
               "the multi-RHS V-cycle smooths with block Jacobi only");
}

// --------------------------------------------------------- segmented PCG --
// Many independent systems stored as one block-diagonal operator (a union of
// meshes): segment s holds unknowns [off[s], off[s+1]).  The SpMV and the
// V-cycle run over the whole union; every segment keeps its own CG scalars
// and stopping test, so segment s follows the single-system pcg
// (krylov.h:22-68) of its own mesh.
struct SegWork {
    int nseg = 0;
    int64_t n = 0;
    int gx = 0;
    int64_t* off = nullptr;
    double *R = nullptr, *D = nullptr, *Q = nullptr, *S = nullptr, *hist = nullptr, *partials = nullptr;
    int hist_len = 0;
    BatchScalars sc{};
    double* sc_mem = nullptr;
    int* sc_int = nullptr;
    int* h_counter = nullptr;
    // blocks of up to 50 iterations as one CUDA graph (as in pcg_dev),
    // keyed by the operands
    cudaGraphExec_t exec = nullptr;
    const mgldg_bsr* gA = nullptr;
    const double* gb = nullptr;
    double* gx_ = nullptr;
    double gtol = 0;
    int gmaxit = 0;
    int64_t pro_launches[MGLDG_K_NCLASS] = {0}, body_launches[MGLDG_K_NCLASS] = {0};
    bool graph_off = false;
};

void seg_free(SegWork* w) {
    if (!w) return;
    if (w->exec) cudaGraphExecDestroy(w->exec);
    dfree(w->off);
    dfree(w->R); dfree(w->D); dfree(w->Q); dfree(w->S); dfree(w->hist); dfree(w->partials);
    dfree(w->sc_mem);
    dfree(w->sc_int);
    if (w->h_counter) cudaFreeHost(w->h_counter);
    delete w;
}

// partials[blockIdx.x * nseg + s] = this CTA's part of segment s of a.b
__global__ void __launch_bounds__(256) k_segdot(const int64_t* __restrict__ off, int nseg, const double* __restrict__ a,
                                               const double* __restrict__ b, double* __restrict__ partials) {
    __shared__ double red[8];
    const int s = blockIdx.y;
    const int64_t lo = off[s], hi = off[s + 1];
    double acc = 0;
    for (int64_t i = lo + (int64_t)blockIdx.x * 256 + threadIdx.x; i < hi; i += (int64_t)gridDim.x * 256)
        acc += a[i] * b[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < 8; ++w) t += red[w];
        partials[(size_t)blockIdx.x * nseg + s] = t;
    }
}

// x += alpha_s d ; (r -= alpha_s q) on active segments
__global__ void __launch_bounds__(256) k_segupdate(const int64_t* __restrict__ off, BatchScalars sc,
                                                  const double* __restrict__ d, const double* __restrict__ q,
                                                  double* __restrict__ x, double* __restrict__ r, int update_r) {
    const int s = blockIdx.y;
    if (!sc.active[s]) return;
    const double al = sc.alpha[s];
    const int64_t lo = off[s], hi = off[s + 1];
    for (int64_t i = lo + (int64_t)blockIdx.x * 256 + threadIdx.x; i < hi; i += (int64_t)gridDim.x * 256) {
        x[i] += al * d[i];
        if (update_r) r[i] -= al * q[i];
    }
}

// d = s + beta_s d on active segments
__global__ void __launch_bounds__(256) k_segdir(const int64_t* __restrict__ off, BatchScalars sc,
                                               const double* __restrict__ sv, double* __restrict__ d) {
    const int s = blockIdx.y;
    if (!sc.active[s]) return;
    const double be = sc.beta[s];
    const int64_t lo = off[s], hi = off[s + 1];
    for (int64_t i = lo + (int64_t)blockIdx.x * 256 + threadIdx.x; i < hi; i += (int64_t)gridDim.x * 256)
        d[i] = sv[i] + be * d[i];
}

static SegWork* ensure_seg(mgldg_mg* m, const std::vector<int64_t>& off, int maxit) {
    mgldg_ctx* ctx = m->ctx;
    const int nseg = (int)off.size() - 1;
    const int64_t n = off.back();
    SegWork* w = m->seg;
    if (w && (w->nseg != nseg || w->n != n)) {
        seg_free(w);
        w = m->seg = nullptr;
    }
    if (!w) {
        w = new SegWork();
        m->seg = w;
        w->nseg = nseg;
        w->n = n;
        int64_t maxlen = 1;
        for (int s = 0; s < nseg; ++s) maxlen = std::max<int64_t>(maxlen, off[s + 1] - off[s]);
        w->gx = (int)std::max<int64_t>(1, std::min<int64_t>((maxlen + 2047) / 2048, 4 * ctx->sm_count / std::max(1, nseg) + 1));
        w->off = dalloc<int64_t>(nseg + 1);
        w->R = dalloc<double>(n); w->D = dalloc<double>(n); w->Q = dalloc<double>(n); w->S = dalloc<double>(n);
        w->partials = dalloc<double>((size_t)w->gx * nseg);
        w->sc_mem = dalloc<double>(5 * (size_t)nseg);
        w->sc_int = dalloc<int>(3 * (size_t)nseg + 3);
        w->sc.delta_new = w->sc_mem;
        w->sc.delta_old = w->sc_mem + nseg;
        w->sc.delta0 = w->sc_mem + 2 * nseg;
        w->sc.alpha = w->sc_mem + 3 * nseg;
        w->sc.beta = w->sc_mem + 4 * nseg;
        w->sc.active = w->sc_int;
        w->sc.iters = w->sc_int + nseg;
        w->sc.broken = w->sc_int + 2 * nseg;
        w->sc.counter = w->sc_int + 3 * nseg;
        MG_CHECK_CUDA(cudaMallocHost(&w->h_counter, 3 * sizeof(int)));
    }
    upload(ctx, w->off, off.data(), off.size());
    const int len = std::max(1, maxit) * nseg;
    if (w->hist_len < len && w->exec) {
        cudaGraphExecDestroy(w->exec);   // bakes the old history buffer
        w->exec = nullptr;
    }
    if (w->hist_len < len) {
        dfree(w->hist);
        w->hist = nullptr;
        w->hist = dalloc<double>(len);
        w->hist_len = len;
    }
    return w;
}

__global__ void k_seg_advance(BatchScalars sc) { sc.counter[2] += 1; }

// while-loop condition of a block of segmented iterations: some segment is
// still active and the next iteration is not a residual-replacement one
__global__ void k_seg_cond(BatchScalars sc, cudaGraphConditionalHandle h) {
    cudaGraphSetConditional(h, (sc.counter[0] > 0 && (sc.counter[2] % 50) != 0) ? 1u : 0u);
}

// one iteration of every active segment's pcg (krylov.h:43-61); `it` < 0:
// the iteration index is the device-side counter (graph capture)
static void seg_iteration(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, SegWork* w, const double* b, double* x,
                          double tol2, int maxit, bool replace, int it, bool eager) {
    const int nseg = w->nseg;
    BatchScalars sc = w->sc;
    const dim3 grid(w->gx, nseg);
    const int gk = (nseg + 127) / 128;
    auto segdot = [&](const double* a, const double* c) {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_segdot<<<grid, 256, 0, ctx->stream>>>(w->off, nseg, a, c, w->partials);
    };
    spmv<double>(ctx, A, 1.0, w->D, 0.0, nullptr, w->Q);
    segdot(w->D, w->Q);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_alpha<<<gk, 128, 0, ctx->stream>>>(nseg, sc, w->partials, w->gx);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_segupdate<<<grid, 256, 0, ctx->stream>>>(w->off, sc, w->D, w->Q, x, w->R, replace ? 0 : 1);
    }
    check_launch();
    if (replace) spmv<double>(ctx, A, -1.0, x, 1.0, b, w->R);
    segdot(w->R, w->R);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_rr<<<gk, 128, 0, ctx->stream>>>(nseg, sc, w->partials, w->gx, w->hist, maxit, it);
    }
    check_launch();
    if (eager) mg_precon_eager(m, w->R, w->S);
    else mg_precon(m, w->R, w->S);
    segdot(w->R, w->S);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_beta<<<gk, 128, 0, ctx->stream>>>(nseg, sc, w->partials, w->gx);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_segdir<<<grid, 256, 0, ctx->stream>>>(w->off, sc, w->S, w->D);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_end<<<gk, 128, 0, ctx->stream>>>(nseg, sc, tol2, maxit, it);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_count<<<1, 256, 0, ctx->stream>>>(nseg, sc);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_seg_advance<<<1, 1, 0, ctx->stream>>>(sc);
    }
    check_launch();
}

// A block of segmented iterations as one CUDA graph: the residual-replacement
// iteration, then a conditional while node over ordinary iterations.
static bool build_seg_graph(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, SegWork* w, const double* b, double* x,
                            double tol, int maxit) {
    if (w->exec) {
        cudaGraphExecDestroy(w->exec);
        w->exec = nullptr;
    }
    const double tol2 = tol * tol;
    int64_t before[MGLDG_K_NCLASS];
    std::memcpy(before, ctx->launches, sizeof before);
    cudaGraph_t graph = nullptr;
    bool ok = true;
    if (cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    try {
        seg_iteration(ctx, m, A, w, b, x, tol2, maxit, true, -1, true);
        for (int k = 0; k < MGLDG_K_NCLASS; ++k) w->pro_launches[k] = ctx->launches[k] - before[k];
        cudaStreamCaptureStatus st;
        cudaGraph_t cg = nullptr;
        const cudaGraphNode_t* deps = nullptr;
        size_t ndeps = 0;
        MG_CHECK_CUDA(cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, nullptr, &ndeps));
        cudaGraphConditionalHandle h;
        MG_CHECK_CUDA(cudaGraphConditionalHandleCreate(&h, cg, 0, 0));
        k_seg_cond<<<1, 1, 0, ctx->stream>>>(w->sc, h);
        check_launch();
        MG_CHECK_CUDA(cudaStreamGetCaptureInfo(ctx->stream, &st, nullptr, &cg, &deps, nullptr, &ndeps));
        cudaGraphNodeParams cp = {};
        cp.type = cudaGraphNodeTypeConditional;
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeWhile;
        cp.conditional.size = 1;
        cudaGraphNode_t wnode;
        MG_CHECK_CUDA(cudaGraphAddNode(&wnode, cg, deps, nullptr, ndeps, &cp));
        cudaGraph_t body = cp.conditional.phGraph_out[0];
        MG_CHECK_CUDA(cudaStreamUpdateCaptureDependencies(ctx->stream, &wnode, nullptr, 1,
                                                          cudaStreamSetCaptureDependencies));
        if (cudaStreamEndCapture(ctx->stream, &graph) != cudaSuccess || !graph) ok = false;
        if (ok) {
            int64_t b2[MGLDG_K_NCLASS];
            std::memcpy(b2, ctx->launches, sizeof b2);
            MG_CHECK_CUDA(cudaStreamBeginCaptureToGraph(ctx->stream, body, nullptr, nullptr, 0,
                                                        cudaStreamCaptureModeThreadLocal));
            seg_iteration(ctx, m, A, w, b, x, tol2, maxit, false, -1, true);
            k_seg_cond<<<1, 1, 0, ctx->stream>>>(w->sc, h);
            check_launch();
            cudaGraph_t bg = nullptr;
            if (cudaStreamEndCapture(ctx->stream, &bg) != cudaSuccess) ok = false;
            for (int k = 0; k < MGLDG_K_NCLASS; ++k) w->body_launches[k] = ctx->launches[k] - b2[k];
        }
    } catch (...) {
        ok = false;
        cudaGraph_t junk = nullptr;
        cudaStreamEndCapture(ctx->stream, &junk);
        if (junk) cudaGraphDestroy(junk);
    }
    if (ok && cudaGraphInstantiate(&w->exec, graph, 0) != cudaSuccess) {
        w->exec = nullptr;
        ok = false;
    }
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    std::memcpy(ctx->launches, before, sizeof before);   // captured, not run
    if (!ok) return false;
    w->gA = A;
    w->gb = b;
    w->gx_ = x;
    w->gtol = tol;
    w->gmaxit = maxit;
    return true;
}

static void segpcg(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, const std::vector<int64_t>& off, const double* b,
                   double* x, double tol, int maxit, int* iters, double* res_hist) {
    SegWork* w = ensure_seg(m, off, maxit);
    const int nseg = w->nseg;
    BatchScalars sc = w->sc;
    const dim3 grid(w->gx, nseg);
    const int gk = (nseg + 127) / 128;
    const double tol2 = tol * tol;
    // R = b - A x ; D = M(R) ; delta = R.D per segment
    spmv<double>(ctx, A, -1.0, x, 1.0, b, w->R);
    mg_precon(m, w->R, w->D);
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_segdot<<<grid, 256, 0, ctx->stream>>>(w->off, nseg, w->R, w->D, w->partials);
    }
    check_launch();
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_init<<<gk, 128, 0, ctx->stream>>>(nseg, sc, w->partials, w->gx, tol2, maxit);
    }
    {
        Launch L(ctx, MGLDG_K_VECTOR);
        k_bpcg_count<<<1, 256, 0, ctx->stream>>>(nseg, sc);
    }
    check_launch();
    MG_CHECK_CUDA(cudaMemsetAsync(sc.counter + 2, 0, sizeof(int), ctx->stream));
    MG_CHECK_CUDA(cudaMemcpyAsync(w->h_counter, sc.counter, 3 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    sync(ctx);
    mg_take_errors(m);
    int i = 0;
    static const bool host_loop = std::getenv("MGLDG_PCG_HOST_LOOP") != nullptr;
    const bool use_graph = !ctx->prof && !w->graph_off && !host_loop;
    while (w->h_counter[0] > 0) {
        if (use_graph && !w->graph_off) {
            if (!(w->exec && w->gA == A && w->gb == b && w->gx_ == x && w->gtol == tol && w->gmaxit == maxit) &&
                !build_seg_graph(ctx, m, A, w, b, x, tol, maxit))
                w->graph_off = true;
            if (!w->graph_off && cudaGraphLaunch(w->exec, ctx->stream) != cudaSuccess) {
                cudaGetLastError();
                cudaGraphExecDestroy(w->exec);
                w->exec = nullptr;
                w->graph_off = true;
            }
            if (!w->graph_off) {
                MG_CHECK_CUDA(cudaMemcpyAsync(w->h_counter, sc.counter, 3 * sizeof(int), cudaMemcpyDeviceToHost,
                                              ctx->stream));
                sync(ctx);
                const int done = w->h_counter[2] - i;
                for (int k = 0; k < MGLDG_K_NCLASS; ++k)
                    ctx->launches[k] += w->pro_launches[k] + (int64_t)(done - 1) * w->body_launches[k];
                i = w->h_counter[2];
                continue;
            }
        }
        seg_iteration(ctx, m, A, w, b, x, tol2, maxit, i % 50 == 0, i, false);
        MG_CHECK_CUDA(cudaMemcpyAsync(w->h_counter, sc.counter, 3 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        sync(ctx);
        ++i;
    }
    mg_take_errors(m);
    std::vector<int> it(nseg), broken(nseg);
    download(ctx, it.data(), sc.iters, nseg);
    download(ctx, broken.data(), sc.broken, nseg);
    sync(ctx);
    if (iters) std::copy(it.begin(), it.end(), iters);
    if (res_hist && maxit > 0) {
        download(ctx, res_hist, w->hist, (int64_t)maxit * nseg);
        sync(ctx);
    }
    for (int s = 0; s < nseg; ++s)
        if (broken[s]) throw Error(MGLDG_ERR_BREAKDOWN, "pcg breakdown in segment " + std::to_string(s));
}

}  // namespace mg

// ================================================================== C ABI ==
extern "C" int mgldg_bsr_mm_dev(mgldg_ctx* ctx, double alpha, const mgldg_bsr* A, int k, const double* X, double beta,
                                double* Y) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && X && Y && k >= 1 && k <= kMaxCols, MGLDG_ERR_ARG, "bad spmm arguments");
    SpmmArgs<double> a = args_of<double>(A, bsr_vals<double>(A), k);
    a.alpha = alpha;
    a.beta = beta;
    a.X = X;
    a.Yin = Y;
    a.Y = Y;
    spmm_launch<double>(ctx, A->br, A->bc, a, 0, default_cfg(k, sizeof(double)), MGLDG_K_SPMV);
    MG_API_END
}

extern "C" int mgldg_mg_vcycle_batched_dev(mgldg_ctx* ctx, mgldg_mg* m, int k, const double* B, double* X) {
    MG_API_BEGIN(ctx)
    require_batch(m, k);
    MG_REQUIRE(B && X, MGLDG_ERR_ARG, "null multi-vector");
    ensure_batch(m, k, nullptr);
    bprecon(m, B, X, false);
    sync(ctx);
    take_batch_errors(m);
    MG_API_END
}

extern "C" int mgldg_pcg_batched_dev(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, int k, const double* B,
                                     double* X, double tol, int maxit, int* iters, double* res_hist) {
    MG_API_BEGIN(ctx)
    require_batch(m, k);
    MG_REQUIRE(A && B && X && maxit >= 0, MGLDG_ERR_ARG, "bad pcg arguments");
    MG_REQUIRE(A->br == A->bc && A->nbr == A->nbc, MGLDG_ERR_SHAPE, "pcg needs a square matrix");
    MG_REQUIRE(m->L[0].n == (int64_t)A->nbr * A->br, MGLDG_ERR_SHAPE, "preconditioner size mismatch");
    bpcg(ctx, m, A, k, B, X, tol, maxit, iters, res_hist);
    MG_API_END
}

extern "C" int mgldg_pcg_batched(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, int k, const double* B, double* X,
                                 double tol, int maxit, int* iters, double* res_hist) {
    MG_API_BEGIN(ctx)
    require_batch(m, k);
    MG_REQUIRE(A && B && X && maxit >= 0, MGLDG_ERR_ARG, "bad pcg arguments");
    MG_REQUIRE(A->br == A->bc && A->nbr == A->nbc, MGLDG_ERR_SHAPE, "pcg needs a square matrix");
    MG_REQUIRE(m->L[0].n == (int64_t)A->nbr * A->br, MGLDG_ERR_SHAPE, "preconditioner size mismatch");
    const int64_t nk = (int64_t)A->nbr * A->br * k;
    double *dB = nullptr, *dX = nullptr;
    try {
        dB = dalloc<double>(nk);
        dX = dalloc<double>(nk);
        upload(ctx, dB, B, nk);
        upload(ctx, dX, X, nk);
        bpcg(ctx, m, A, k, dB, dX, tol, maxit, iters, res_hist);
        download(ctx, X, dX, nk);
        sync(ctx);
    } catch (...) {
        dfree(dB);
        dfree(dX);
        throw;
    }
    dfree(dB);
    dfree(dX);
    MG_API_END
}

extern "C" int mgldg_mg_batch_tiles(const mgldg_mg* m, int level, int* spmm, int* jacobi, int* restrict_,
                                    int* prolong, int* outer) {
    if (!m || !m->batch || level < 0 || level >= (int)m->batch->L.size()) return MGLDG_ERR_ARG;
    const BatchLevel& B = m->batch->L[level];
    if (spmm) *spmm = 32 * B.spmm.V;
    if (jacobi) *jacobi = 32 * B.jac.V;
    if (restrict_) *restrict_ = 32 * B.restrict_.V;
    if (prolong) *prolong = 32 * B.prolong.V;
    if (outer) *outer = 32 * m->batch->outer.V;
    return MGLDG_OK;
}

extern "C" int mgldg_pcg_segmented_dev(mgldg_ctx* ctx, mgldg_mg* m, const mgldg_bsr* A, int nseg,
                                       const int64_t* seg_offsets, const double* b, double* x, double tol, int maxit,
                                       int* iters, double* res_hist) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(m && !m->L.empty(), MGLDG_ERR_ARG, "segmented pcg needs a multigrid preconditioner");
    MG_REQUIRE(A && b && x && seg_offsets && nseg >= 1 && nseg <= 65535 && maxit >= 0, MGLDG_ERR_ARG,
               "bad segmented pcg arguments");
    MG_REQUIRE(A->br == A->bc && A->nbr == A->nbc, MGLDG_ERR_SHAPE, "pcg needs a square matrix");
    const int64_t n = (int64_t)A->nbr * A->br;
    MG_REQUIRE(m->L[0].n == n, MGLDG_ERR_SHAPE, "preconditioner size mismatch");
    std::vector<int64_t> off(seg_offsets, seg_offsets + nseg + 1);
    MG_REQUIRE(off[0] == 0 && off[nseg] == n, MGLDG_ERR_SHAPE, "segments must cover the unknowns");
    for (int s = 0; s < nseg; ++s) MG_REQUIRE(off[s + 1] > off[s], MGLDG_ERR_ARG, "empty or unsorted segment");
    segpcg(ctx, m, A, off, b, x, tol, maxit, iters, res_hist);
    MG_API_END
}

// bulk.cu -- FP32 block-row kernels (SpMV and the damped block-Jacobi sweep)
// that stream the matrix through shared memory with the bulk-copy engine.
//
// A CTA of 8 warps owns groups of 8 consecutive block rows.  The values of a
// group's rows are one contiguous run in HBM (block CSR keeps a row's blocks
// together and rows in order), so one elected thread moves the whole run --
// and, for Jacobi, the group's 8 inverse diagonal blocks -- into a shared-
// memory stage with cp.async.bulk, completion tracked by an mbarrier.  Two
// stages per CTA, two CTAs per SM: while the warps work on one group the
// next group's bytes are already in flight, without holding them in
// registers.  Each warp then computes one row from shared memory, gathering
// x from L2.  Groups whose blocks do not fit a stage are read from HBM
// directly.  Every barrier wait is bounded (about one second); on expiry the
// kernel sets the context's error word, drains its own copies (again
// bounded) and returns, and the host reports MGLDG_ERR_TIMEOUT.
//
// Handles 16 x 16 blocks (Q3 in 2-D) stored in FP32 (the mixed form's
// V-cycle) or block-scaled FP16 (MGLDG_PREC_MIXED_F16: half the value bytes;
// the stage then also holds the group's block scales, and each block's
// partial product is multiplied by its scale), arithmetic in FP32.
#include "api.cuh"
#include "rowdot.cuh"

namespace mg {

namespace {
constexpr int kRows = 8;                          // rows per group (= warps per CTA)
constexpr int kB = 16;                            // block rows / columns
constexpr int kBlk = kB * kB;                     // values per block
constexpr int kCap = 40;                          // matrix blocks per stage
constexpr int kColInts = kCap + 4;                // column indices (copy starts 16-byte aligned)
// stage layout in bytes: values | Dinv (FP32) | column indices | scales (FP16 only)
template <class VT>
struct Stage {
    static constexpr int kVal = kCap * kBlk * (int)sizeof(VT);
    static constexpr int kDinv = kVal;
    static constexpr int kCol = kDinv + kRows * kBlk * 4;
    static constexpr int kScl = kCol + kColInts * 4;
    static constexpr int kBytes = kScl + (sizeof(VT) == 2 ? kColInts * 4 : 0);
    // stages per CTA (FP16: three CTAs per SM hold about as many bytes in
    // flight as two FP32 CTAs)
    static constexpr int kNS = 2;
    static constexpr size_t kSmem = (size_t)kNS * kBytes;   // ~96 KiB (FP32), ~57 KiB (FP16)
    static constexpr int kMinBlocks = sizeof(VT) == 2 ? 3 : 2;   // CTAs per SM
    static_assert(kBytes % 16 == 0 && kCol % 16 == 0 && kScl % 16 == 0, "stage regions must stay 16-byte aligned");
};
}  // namespace

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// bounded wait for the completion of `phase` of an mbarrier
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned phase, int64_t timeout_ns) {
    if (mbar_try_wait(bar, phase)) return true;
    const uint64_t t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, phase))
        if ((int64_t)(globaltimer_ns() - t0) > timeout_ns) return false;
    return true;
}

// One row's partial product from a block array `a` and its column indices
// `cols` (both in the shared-memory stage, or both in HBM) with x gathered
// from L2, five blocks in flight.
__device__ __forceinline__ float row_from(const float* a, const float* /*scl*/, const int* cols,
                                          const float* __restrict__ x, int nb, int r, int c0, int lane) {
    float acc = 0.f;
    for (int qb = 0; qb < nb; qb += 5) {
        const int m = min(5, nb - qb);
        const int jl = (lane < m) ? cols[qb + lane] : 0;
        float4 xv[5][2];
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            const int j = __shfl_sync(0xffffffffu, jl, q);
            if (q < m) {
                const float4* xp = reinterpret_cast<const float4*>(x + (size_t)j * kB + c0);
                xv[q][0] = __ldg(xp);
                xv[q][1] = __ldg(xp + 1);
            }
        }
#pragma unroll
        for (int q = 0; q < 5; ++q)
            if (q < m) {
                const float4* ap = reinterpret_cast<const float4*>(a + (size_t)(qb + q) * kBlk + r * kB + c0);
                vfma(acc, ap[0], xv[q][0]);
                vfma(acc, ap[1], xv[q][1]);
            }
    }
    return acc;
}

// The same on block-scaled FP16 values: eight halves (16 bytes) per lane and
// block, the block's partial product times its scale; three blocks in flight
// (fewer registers, three CTAs per SM instead of two).
constexpr int kDepth16 = 3;
__device__ __forceinline__ float row_from(const __half* a, const float* scl, const int* cols,
                                          const float* __restrict__ x, int nb, int r, int c0, int lane) {
    float acc = 0.f;
    for (int qb = 0; qb < nb; qb += kDepth16) {
        const int m = min(kDepth16, nb - qb);
        const int jl = (lane < m) ? cols[qb + lane] : 0;
        float4 xv[kDepth16][2];
#pragma unroll
        for (int q = 0; q < kDepth16; ++q) {
            const int j = __shfl_sync(0xffffffffu, jl, q);
            if (q < m) {
                const float4* xp = reinterpret_cast<const float4*>(x + (size_t)j * kB + c0);
                xv[q][0] = __ldg(xp);
                xv[q][1] = __ldg(xp + 1);
            }
        }
#pragma unroll
        for (int q = 0; q < kDepth16; ++q)
            if (q < m) {
                const uint4 raw = *reinterpret_cast<const uint4*>(a + (size_t)(qb + q) * kBlk + r * kB + c0);
                const __half2* h = reinterpret_cast<const __half2*>(&raw);
                const float2 f0 = __half22float2(h[0]), f1 = __half22float2(h[1]);
                const float2 f2 = __half22float2(h[2]), f3 = __half22float2(h[3]);
                float p = f0.x * xv[q][0].x;
                p = fmaf(f0.y, xv[q][0].y, p);
                p = fmaf(f1.x, xv[q][0].z, p);
                p = fmaf(f1.y, xv[q][0].w, p);
                p = fmaf(f2.x, xv[q][1].x, p);
                p = fmaf(f2.y, xv[q][1].y, p);
                p = fmaf(f3.x, xv[q][1].z, p);
                p = fmaf(f3.y, xv[q][1].w, p);
                acc = fmaf(scl[qb + q], p, acc);
            }
    }
    return acc;
}

// JACOBI: xout_i = xin_i + omega * Dinv_i (b_i - (A xin)_i); with xzero
//         (xin = 0) only the inverse diagonal blocks are staged and neither
//         A nor xin is read: (A 0)_i is +0, so the values are the full
//         sweep's bit for bit
// else:   y_i = alpha (A x)_i + beta yin_i
template <bool JACOBI, class VT>
__global__ void __launch_bounds__(kRows * 32, Stage<VT>::kMinBlocks)
    k_rows_bulk(int nbr, const int* __restrict__ row_ptr, const int* __restrict__ col_idx, const VT* __restrict__ val,
                const float* __restrict__ scale, const float* __restrict__ Dinv, const float* __restrict__ x,
                const float* bvec, float* y, float alpha, float beta, float omega, bool xzero, unsigned* err,
                int64_t timeout_ns) {
    using S = Stage<VT>;
    constexpr bool kF16 = sizeof(VT) == 2;
    extern __shared__ __align__(128) unsigned char smem[];
    constexpr int NS = S::kNS;
    __shared__ __align__(8) uint64_t bar[NS];     // "full": the stage's bytes have landed
    __shared__ __align__(8) uint64_t empty[NS];   // "empty": every warp is done with the stage
    __shared__ int s_fits[NS];
    __shared__ int s_rp[NS][kRows + 1];   // the group's row pointers
    __shared__ int s_col0[NS];            // first column index held by the stage
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r = lane >> 1, c0 = (lane & 1) * 8;   // 2 lanes per block row, 8 columns each
    // FP16: each CTA takes one contiguous run of groups, so that consecutive
    // rows (neighbours in the element order) share x entries through L1
    // (measured 4% faster there); FP32: groups strided over the CTAs
    // (3% faster there)
    const int ngroups_all = (nbr + kRows - 1) / kRows;
    const int gbeg = kF16 ? (int)((int64_t)blockIdx.x * ngroups_all / gridDim.x) : (int)blockIdx.x;
    const int ngroups = kF16 ? (int)((int64_t)(blockIdx.x + 1) * ngroups_all / gridDim.x) : ngroups_all;   // end
    const int G = kF16 ? 1 : (int)gridDim.x;
    if (threadIdx.x == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&bar[s], 1);
            mbar_init(&empty[s], kRows);
        }
        fence_mbar_init();
    }
    __syncthreads();

    // thread 0: start the copy of group g into stage st
    auto issue = [&](int st, int g) {
        const int r0 = g * kRows, r1 = min(r0 + kRows, nbr);
        for (int q = 0; q <= kRows; ++q) s_rp[st][q] = __ldg(row_ptr + min(r0 + q, r1));
        const int k0 = s_rp[st][0], k1 = s_rp[st][r1 - r0];
        const int nbk = k1 - k0;
        const int fits = nbk <= kCap;
        s_fits[st] = fits;
        unsigned char* sv = smem + (size_t)st * S::kBytes;
        // column indices (and scales): whole 16-byte words from k0 rounded
        // down (both arrays are padded by four entries, so the copy stays
        // inside them)
        const int cstart = k0 & ~3;
        const int ncol = ((k1 - cstart) + 3) & ~3;
        s_col0[st] = cstart;
        const bool copy_rows = fits && nbk > 0 && !xzero;
        unsigned bytes = 0;
        if (copy_rows) bytes += (unsigned)nbk * kBlk * sizeof(VT) + (unsigned)ncol * sizeof(int) * (kF16 ? 2 : 1);
        if (JACOBI) bytes += (unsigned)(r1 - r0) * kBlk * sizeof(float);
        fence_proxy_async();   // the warps' reads of this stage are complete (barrier before)
        mbar_arrive_expect_tx(&bar[st], bytes);
        if (copy_rows) {
            bulk_g2s(sv, val + (size_t)k0 * kBlk, (unsigned)nbk * kBlk * sizeof(VT), &bar[st]);
            bulk_g2s(sv + S::kCol, col_idx + cstart, (unsigned)ncol * sizeof(int), &bar[st]);
            if (kF16) bulk_g2s(sv + S::kScl, scale + cstart, (unsigned)ncol * sizeof(float), &bar[st]);
        }
        if (JACOBI) bulk_g2s(sv + S::kDinv, Dinv + (size_t)r0 * kBlk, (unsigned)(r1 - r0) * kBlk * sizeof(float), &bar[st]);
    };

    unsigned phase[NS];    // next completion of "full" to wait for
    unsigned ephase[NS];   // next completion of "empty" (thread 0)
    bool pending[NS];
    int g = gbeg;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        phase[s] = 0u;
        ephase[s] = 0u;
        pending[s] = g + s * G < ngroups;
        if (threadIdx.x == 0 && pending[s]) issue(s, g + s * G);
    }
    bool failed = false;
    for (int it = 0; g < ngroups; g += G, ++it) {
        const int st = it % NS;
        const bool ok = __all_sync(0xffffffffu, mbar_wait(&bar[st], phase[st], timeout_ns));
        if (!ok) {
            failed = true;
            break;
        }
        phase[st] ^= 1u;
        pending[st] = false;
        const int row = g * kRows + warp;
        if (row < nbr) {
            const int kg = s_rp[st][0];
            const int k0 = s_rp[st][warp], k1 = s_rp[st][warp + 1];
            const unsigned char* sv = smem + (size_t)st * S::kBytes;
            float bi = 0.f, xi = 0.f;
            if (JACOBI && (lane & 1) == 0) {
                bi = __ldg(bvec + (size_t)row * kB + r);
                if (!xzero) xi = __ldg(x + (size_t)row * kB + r);
            } else if (!JACOBI && beta != 0.f && (lane & 1) == 0) {
                // yin (it may be y itself: each entry is read and written
                // by the same lane), issued before the product
                bi = bvec[(size_t)row * kB + r];
            }
            const bool fits = s_fits[st] != 0;
            const VT* a = fits ? reinterpret_cast<const VT*>(sv) + (size_t)(k0 - kg) * kBlk : val + (size_t)k0 * kBlk;
            const int* cols = fits ? reinterpret_cast<const int*>(sv + S::kCol) + (k0 - s_col0[st]) : col_idx + k0;
            const float* scl = kF16 ? (fits ? reinterpret_cast<const float*>(sv + S::kScl) + (k0 - s_col0[st])
                                            : scale + k0)
                                    : nullptr;
            float acc = 0.f;
            if (!(JACOBI && xzero)) {
                acc = row_from(a, scl, cols, x, k1 - k0, r, c0, lane);
                acc += __shfl_xor_sync(0xffffffffu, acc, 1);
            }
            if (JACOBI) {
                const float t = bi - acc;   // valid in even lanes
                const float4* dp =
                    reinterpret_cast<const float4*>(reinterpret_cast<const float*>(sv + S::kDinv) + warp * kBlk + r * kB + c0);
                const float4 d0 = dp[0], d1 = dp[1];
                float tc[8];
#pragma unroll
                for (int c = 0; c < 8; ++c) tc[c] = __shfl_sync(0xffffffffu, t, ((c0 + c) * 2) & 31);
                float yv = d0.x * tc[0];
                yv = fmaf(d0.y, tc[1], yv);
                yv = fmaf(d0.z, tc[2], yv);
                yv = fmaf(d0.w, tc[3], yv);
                yv = fmaf(d1.x, tc[4], yv);
                yv = fmaf(d1.y, tc[5], yv);
                yv = fmaf(d1.z, tc[6], yv);
                yv = fmaf(d1.w, tc[7], yv);
                yv += __shfl_xor_sync(0xffffffffu, yv, 1);
                if ((lane & 1) == 0) y[(size_t)row * kB + r] = xi + omega * yv;
            } else if ((lane & 1) == 0) {
                float v = alpha * acc;
                if (beta != 0.f) v += beta * bi;
                y[(size_t)row * kB + r] = v;
            }
        }
        // this warp is done with stage st; only the producer (thread 0)
        // waits for the other warps before refilling it
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);
        if (g + NS * G < ngroups) {
            if (warp == 0) {
                bool refill = true;
                if (lane == 0) {
                    refill = mbar_wait(&empty[st], ephase[st], timeout_ns);
                    ephase[st] ^= 1u;
                    if (refill) issue(st, g + NS * G);
                }
                if (!__shfl_sync(0xffffffffu, refill, 0)) {
                    failed = true;
                    break;
                }
            }
            pending[st] = true;
        }
    }
    if (failed && threadIdx.x == 0) {
        // record the failure and wait (bounded) for this CTA's copies in flight
        atomicOr(err, 1u);
        for (int s = 0; s < NS; ++s)
            if (pending[s]) mbar_wait(&bar[s], phase[s], timeout_ns);
    }
}

// The first Jacobi sweep from x = 0 on 16 x 16 blocks: x_i = omega Dinv_i b_i
// with the bulk kernel's lane layout and arithmetic (lane pair 2r, 2r+1 holds
// row r, eight columns each; the same fma chain and pair sum), so the values
// are its xzero values bit for bit.  Only Dinv and b are read -- a plain
// coalesced stream (1 KiB of Dinv per row and warp), which needs no staging.
__global__ void __launch_bounds__(256) k_jacobi_zero16(int nbr, const float* __restrict__ Dinv,
                                                       const float* __restrict__ bvec, float* __restrict__ y,
                                                       float omega) {
    const int lane = threadIdx.x & 31;
    const int r = lane >> 1, c0 = (lane & 1) * 8;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < nbr; row += nw) {
        const float4* dp = reinterpret_cast<const float4*>(Dinv + (size_t)row * kBlk + r * kB + c0);
        const float4 d0 = __ldg(dp), d1 = __ldg(dp + 1);
        const float t = ((lane & 1) == 0) ? __ldg(bvec + (size_t)row * kB + r) : 0.f;   // b - (A 0) = b
        float tc[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) tc[c] = __shfl_sync(0xffffffffu, t, ((c0 + c) * 2) & 31);
        float yv = d0.x * tc[0];
        yv = fmaf(d0.y, tc[1], yv);
        yv = fmaf(d0.z, tc[2], yv);
        yv = fmaf(d0.w, tc[3], yv);
        yv = fmaf(d1.x, tc[4], yv);
        yv = fmaf(d1.y, tc[5], yv);
        yv = fmaf(d1.z, tc[6], yv);
        yv = fmaf(d1.w, tc[7], yv);
        yv += __shfl_xor_sync(0xffffffffu, yv, 1);
        const float xi = 0.f;
        if ((lane & 1) == 0) y[(size_t)row * kB + r] = xi + omega * yv;
    }
}

static void launch_jacobi_zero16(mgldg_ctx* ctx, const mgldg_bsr* A, const float* Dinv, const float* b, float* xout,
                                 float omega) {
    const int grid = std::max(1, std::min((A->nbr + 7) / 8, ctx->sm_count * 8));
    {
        Launch L(ctx, MGLDG_K_JACOBI);
        k_jacobi_zero16<<<grid, 256, 0, ctx->stream>>>(A->nbr, Dinv, b, xout, omega);
    }
    check_launch();
}

template <bool JACOBI, class VT>
static void launch_bulk(mgldg_ctx* ctx, const mgldg_bsr* A, const VT* vals, const float* scale, const float* Dinv,
                        const float* x, const float* bvec, float* y, float alpha, float beta, float omega, bool xzero,
                        int kclass) {
    static bool attr_set[64] = {false};
    if (ctx->device < 64 && !attr_set[ctx->device]) {
        MG_CHECK_CUDA(cudaFuncSetAttribute(k_rows_bulk<JACOBI, VT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)Stage<VT>::kSmem));
        attr_set[ctx->device] = true;
    }
    const int ngroups = (A->nbr + kRows - 1) / kRows;
    const int grid = std::max(1, std::min(ngroups, Stage<VT>::kMinBlocks * ctx->sm_count));
    {
        Launch L(ctx, kclass);
        k_rows_bulk<JACOBI, VT><<<grid, kRows * 32, Stage<VT>::kSmem, ctx->stream>>>(
            A->nbr, A->row_ptr, A->col_idx, vals, scale, Dinv, x, bvec, y, alpha, beta, omega, xzero, ctx->d_err,
            1000000000LL);
    }
    check_launch();
}

bool bulk_spmv_f32(mgldg_ctx* ctx, const mgldg_bsr* A, float alpha, const float* x, float beta, const float* yin,
                   float* y, int kclass) {
    if (A->br != kB || A->bc != kB || A->blk || !A->val32 || A->nbr == 0) return false;
    launch_bulk<false, float>(ctx, A, A->val32, nullptr, nullptr, x, yin, y, alpha, beta, 0.f, false, kclass);
    return true;
}

bool bulk_spmv_f16(mgldg_ctx* ctx, const mgldg_bsr* A, float alpha, const float* x, float beta, const float* yin,
                   float* y, int kclass) {
    if (A->br != kB || A->bc != kB || A->blk || !A->val16 || A->nbr == 0) return false;
    launch_bulk<false, __half>(ctx, A, A->val16, A->scale16, nullptr, x, yin, y, alpha, beta, 0.f, false, kclass);
    return true;
}

bool bulk_jacobi_f16(mgldg_ctx* ctx, const mgldg_bsr* A, const float* Dinv, const float* b, const float* xin,
                     float* xout, float omega, bool xzero) {
    if (A->br != kB || A->bc != kB || A->blk || !A->val16 || A->nbr == 0) return false;
    if (xzero) launch_jacobi_zero16(ctx, A, Dinv, b, xout, omega);
    else launch_bulk<true, __half>(ctx, A, A->val16, A->scale16, Dinv, xin, b, xout, 0.f, 0.f, omega, false,
                                   MGLDG_K_JACOBI);
    return true;
}

bool bulk_jacobi_f32(mgldg_ctx* ctx, const mgldg_bsr* A, const float* vals, const float* Dinv, const float* b,
                     const float* xin, float* xout, float omega, bool xzero) {
    if (A->br != kB || A->bc != kB || A->blk || A->nbr == 0) return false;
    if (xzero) launch_jacobi_zero16(ctx, A, Dinv, b, xout, omega);
    else launch_bulk<true, float>(ctx, A, vals, nullptr, Dinv, xin, b, xout, 0.f, 0.f, omega, false, MGLDG_K_JACOBI);
    return true;
}

void take_device_error(mgldg_ctx* ctx) {
    if (!ctx->d_err) return;
    unsigned h = 0;
    download(ctx, &h, ctx->d_err, 1);
    sync(ctx);
    if (h) {
        MG_CHECK_CUDA(cudaMemsetAsync(ctx->d_err, 0, sizeof(unsigned), ctx->stream));
        sync(ctx);
        throw Error(MGLDG_ERR_TIMEOUT, "a bulk-copy barrier wait ran out");
    }
}

}  // namespace mg

// tail.cu -- the coarse end of the mixed-precision Jacobi V-cycle as one
// cooperative launch.
//
// Below a few thousand block rows every level of the V-cycle
// (multigrid.h:361-383: pre-smoothing, residual, restriction, the coarsest
// solve, prolongation, post-smoothing) is a chain of launches that each move
// kilobytes: 3-6 us apiece, all latency.  Here one launch with every CTA
// co-resident runs all of those steps for the levels s .. last, separated by
// grid-wide barriers (an arrival counter in global memory, zeroed before the
// launch, every wait bounded by %globaltimer).  Each step repeats, lane for
// lane, the arithmetic of the kernel it replaces -- the FP32 16 x 16 block
// rows of bulk.cu (k_rows_bulk / k_jacobi_zero16: lane pair 2r, 2r+1 holds
// row r, eight columns each), the block-table transfers of bsr.cu
// (k_transfer) and the dense coarsest solve of mg.cu (k_coarse_solve) -- so
// the V-cycle's values do not change.  Values written during the launch are
// read through L2 (ld.global.cg), never through the SM-private L1 or the
// read-only path.
//
// Opt-in (MGLDG_VTAIL_ROWS = the largest level, in block rows, it starts
// at).  On the 512 x 512 Q3 solve from 64 x 64 down it cut the event-timed
// coarse-level work from 5.5 to 3.7 ms per solve, yet the graph-replayed
// solve took 54.5 ms against 53.2 ms: its ~28 grid barriers per V-cycle
// (about 5 us each with two CTAs per SM) cost as much as the replayed
// launches they replace.
#include "api.cuh"
#include "mg.cuh"
#include "rowdot.cuh"
#include "tail.cuh"

namespace mg {

namespace {
constexpr int kB = 16;
constexpr int kBlk = kB * kB;
constexpr int kChunk = 3;   // blocks of a row whose loads are in flight together

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// every CTA arrives; returns when `target` arrivals have been counted, or
// false (error word set) when the wait ran out or another CTA gave up
__device__ bool tail_barrier(unsigned* count, unsigned target, unsigned* err, int64_t timeout_ns) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        atomicAdd(count, 1u);
        if (ld_acquire(count) < target) {
            const uint64_t t0 = globaltimer_ns();
            while (ld_acquire(count) < target) {
                if (ld_acquire(err) != 0u || (int64_t)(globaltimer_ns() - t0) > timeout_ns) {
                    atomicOr(err, 1u);
                    ok = 0;
                    break;
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// r = alpha (A x) + beta b (RESID) or xo = x + omega Dinv (b - A x) (Jacobi;
// zero: x = 0, neither x nor A read).  One warp per block row.
template <bool RESID>
__device__ void tail_rows(const TailLevel& v, const float* x, float* out, float omega, bool zero, int gw, int nw,
                          int lane) {
    const int r = lane >> 1, c0 = (lane & 1) * 8;
    for (int row = gw; row < v.nbr; row += nw) {
        float bi = 0.f, xi = 0.f;
        if ((lane & 1) == 0) {
            bi = __ldcg(v.b + (size_t)row * kB + r);
            if (!RESID && !zero) xi = __ldcg(x + (size_t)row * kB + r);
        }
        float acc = 0.f;
        if (!zero) {
            const int k0 = __ldg(v.rp + row), k1 = __ldg(v.rp + row + 1);
            for (int qb = k0; qb < k1; qb += kChunk) {
                const int m = min(kChunk, k1 - qb);
                int jq[kChunk];
#pragma unroll
                for (int u = 0; u < kChunk; ++u) jq[u] = (u < m) ? __ldg(v.ci + qb + u) : 0;
                float4 av[kChunk][2], xv[kChunk][2];
#pragma unroll
                for (int u = 0; u < kChunk; ++u)
                    if (u < m) {
                        const float4* ap = reinterpret_cast<const float4*>(v.val + (size_t)(qb + u) * kBlk + r * kB + c0);
                        const float4* xp = reinterpret_cast<const float4*>(x + (size_t)jq[u] * kB + c0);
                        av[u][0] = __ldg(ap);
                        av[u][1] = __ldg(ap + 1);
                        xv[u][0] = __ldcg(xp);
                        xv[u][1] = __ldcg(xp + 1);
                    }
#pragma unroll
                for (int u = 0; u < kChunk; ++u)
                    if (u < m) {
                        vfma(acc, av[u][0], xv[u][0]);
                        vfma(acc, av[u][1], xv[u][1]);
                    }
            }
            acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        }
        if (RESID) {
            if ((lane & 1) == 0) {
                float o = -1.f * acc;
                o += 1.f * bi;
                __stcg(out + (size_t)row * kB + r, o);
            }
            continue;
        }
        const float t = bi - acc;   // valid in even lanes
        const float4* dp = reinterpret_cast<const float4*>(v.Dinv + (size_t)row * kBlk + r * kB + c0);
        const float4 d0 = __ldg(dp), d1 = __ldg(dp + 1);
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
        if ((lane & 1) == 0) __stcg(out + (size_t)row * kB + r, xi + omega * yv);
    }
}

// y = T x (+ yin when beta != 0) for a block-table interpolation operator,
// one thread per output entry
__device__ void tail_xfer(const TailXfer& T, const float* x, float beta, const float* yin, float* y, int gt, int nt) {
    const int64_t n = (int64_t)T.nbr * kB;
    for (int64_t t = gt; t < n; t += nt) {
        const int row = (int)(t / kB), r = (int)(t - (int64_t)row * kB);
        float acc = 0.f;
        const int k0 = __ldg(T.rp + row), k1 = __ldg(T.rp + row + 1);
        for (int k = k0; k < k1; ++k) {
            const float* a = T.tab + ((size_t)__ldg(T.blk + k) * kB + r) * kB;
            const float* xj = x + (size_t)__ldg(T.ci + k) * kB;
#pragma unroll
            for (int c = 0; c < kB; ++c) acc = fmaf(__ldg(a + c), __ldcg(xj + c), acc);
        }
        float v = 1.f * acc;
        if (beta != 0.f) v += beta * __ldcg(yin + t);
        __stcg(y + t, v);
    }
}

__global__ void __launch_bounds__(256, 2) k_vtail(const __grid_constant__ TailArgs a) {
    extern __shared__ double sb[];
    const int lane = threadIdx.x & 31;
    const int gw = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), nw = gridDim.x * (blockDim.x >> 5);
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    unsigned bars = 0;
#define MG_TAIL_SYNC                                                                              \
    if (!tail_barrier(a.count, ++bars * gridDim.x, a.err, a.timeout_ns)) return;
    const int L = a.nlev - 1;   // the coarsest level of the tail
    float* cur[kTailMaxLevels];
    float* oth[kTailMaxLevels];
    for (int l = 0; l < L; ++l) {
        const TailLevel& v = a.L[l];
        float* c = v.x;
        float* o = v.xt;
        for (int s = 0; s < a.npre; ++s) {
            tail_rows<false>(v, c, o, a.omega, s == 0, gw, nw, lane);
            float* tmp = c;
            c = o;
            o = tmp;
            MG_TAIL_SYNC
        }
        tail_rows<true>(v, c, v.r, 0.f, false, gw, nw, lane);
        MG_TAIL_SYNC
        tail_xfer(v.Tt, v.r, 0.f, nullptr, a.L[l + 1].b, gt, nt);
        MG_TAIL_SYNC
        cur[l] = c;
        oth[l] = o;
    }
    {
        // the coarsest solve x = Cinv b (b staged per CTA in FP64)
        const TailLevel& v = a.L[L];
        const int n = a.nc;
        for (int i = threadIdx.x; i < n; i += blockDim.x) sb[i] = (double)__ldcg(v.b + i);
        __syncthreads();
        for (int row = gw; row < n; row += nw) {
            const double* cr = a.Cinv + (size_t)row * n;
            double s = 0;
            for (int c = lane; c < n; c += 32) s += __ldg(cr + c) * sb[c];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) __stcg(v.x + row, (float)s);
        }
        MG_TAIL_SYNC
    }
    for (int l = L - 1; l >= 0; --l) {
        const TailLevel& v = a.L[l];
        const float* xc = (l + 1 == L) ? a.L[L].x : cur[l + 1];
        float* c = cur[l];
        float* o = oth[l];
        tail_xfer(v.T, xc, 1.f, c, c, gt, nt);
        MG_TAIL_SYNC
        for (int s = 0; s < a.npost; ++s) {
            tail_rows<false>(v, c, o, a.omega, false, gw, nw, lane);
            float* tmp = c;
            c = o;
            o = tmp;
            if (l > 0 || s + 1 < a.npost) MG_TAIL_SYNC
        }
        cur[l] = c;
    }
#undef MG_TAIL_SYNC
}
}  // namespace

bool tail_supported(const mgldg_mg* m, int s) {
    const int last = (int)m->L.size() - 1;
    if (s < 1 || s >= last || last - s + 1 > kTailMaxLevels) return false;
    const mgldg_mg_params& p = m->p;
    if (p.precision != MGLDG_PREC_MIXED && p.precision != MGLDG_PREC_MIXED_TF32) return false;
    if (p.relaxation != MGLDG_RELAX_JACOBI || p.npre < 1 || p.npost < 0 || p.mean_project) return false;
    if (p.solver != MGLDG_COARSE_DENSE && p.solver != MGLDG_COARSE_CHOLESKY) return false;
    if (!m->Cinv || m->nc != m->L[last].n || m->nc > 4096) return false;
    auto table_ok = [](const mgldg_bsr* T) {
        return T && T->blk && T->val32 && T->nuniq <= 16 && T->br == kB && T->bc == kB;
    };
    for (int l = s; l <= last; ++l) {
        const LevelData& L = m->L[l];
        if (L.b != kB || !L.x32 || !L.xt32 || !L.b32) return false;
        if (l < last) {
            if (L.A->br != kB || L.A->bc != kB || L.A->blk || !L.A->val32 || !L.Dinv32 || !L.r32) return false;
            if (!table_ok(L.Tt) || !table_ok(L.T)) return false;
        }
    }
    return true;
}

void tail_launch(mgldg_mg* m, int s, unsigned* count) {
    mgldg_ctx* ctx = m->ctx;
    const int last = (int)m->L.size() - 1;
    TailArgs a{};
    a.nlev = last - s + 1;
    for (int l = s; l <= last; ++l) {
        LevelData& L = m->L[l];
        TailLevel& v = a.L[l - s];
        v.nbr = L.ne;
        v.x = L.x32;
        v.xt = L.xt32;
        v.b = L.b32;
        v.r = L.r32;
        if (l < last) {
            v.rp = L.A->row_ptr;
            v.ci = L.A->col_idx;
            v.val = L.A->val32;
            v.Dinv = L.Dinv32;
            v.Tt = TailXfer{L.Tt->row_ptr, L.Tt->col_idx, L.Tt->blk, L.Tt->val32, L.Tt->nbr};
            v.T = TailXfer{L.T->row_ptr, L.T->col_idx, L.T->blk, L.T->val32, L.T->nbr};
        }
    }
    a.nc = m->nc;
    a.Cinv = m->Cinv;
    a.omega = (float)m->p.omega;
    a.npre = m->p.npre;
    a.npost = m->p.npost;
    a.count = count;
    a.err = ctx->d_err;
    a.timeout_ns = 1000000000LL;
    const size_t smem = (size_t)m->nc * sizeof(double);
    int per_sm = 0;
    MG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_vtail, 256, smem));
    MG_REQUIRE(per_sm > 0, MGLDG_ERR_CUDA, "coarse-tail kernel does not fit on an SM");
    const int grid = std::min(per_sm, 2) * ctx->sm_count;
    MG_CHECK_CUDA(cudaMemsetAsync(count, 0, sizeof(unsigned), ctx->stream));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;   // every CTA co-resident: the barriers need it
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    {
        Launch K(ctx, MGLDG_K_JACOBI);
        MG_CHECK_CUDA(cudaLaunchKernelEx(&cfg, k_vtail, a));
    }
}

}  // namespace mg

// smooth.cu -- block smoothers: fused damped block-Jacobi and block
// Gauss-Seidel run as a level-scheduled dataflow sweep that reproduces the
// reference's sequential order exactly.
//
// Reference: Level::jacobi and Level::gauss_seidel
// (src/cartesian/multigrid/multigrid.h:223-262).  The diagonal blocks are
// pre-inverted (Dinv) instead of LDL^T-solved.
//
// Gauss-Seidel.  A forward sweep updates block rows i = 0..n-1 in order,
// using new values of the neighbours j < i and old values of j > i.  Row i
// therefore depends only on its earlier neighbours; rows are grouped into
// level sets (level(i) = 1 + max level of its earlier neighbours) and the
// rows of one level are independent.  One persistent cooperative launch
// covers a sweep: warps take rows in level order (static round-robin), read
// the later neighbours (their old values are stable until row i publishes,
// because each of them waits for row i), then wait on a per-row completion
// flag of each earlier neighbour, finish the row and publish it with a
// release store.  Every wait is bounded (about one second of %globaltimer);
// on expiry the kernel records an error word, every other waiter gives up,
// and the host returns MGLDG_ERR_TIMEOUT with the context still usable.
// The sweep counter lives in device memory and is advanced by the last CTA
// to finish, so consecutive sweeps need no host involvement.
#include <algorithm>
#include <type_traits>

#include "api.cuh"
#include "rowdot.cuh"
#include "smooth.cuh"

using namespace mg;

namespace mg {

// ---------------------------------------------------------------- helpers --
template <class T, int BR, int BC>
__device__ __forceinline__ T chunk_dot_coherent(const T* __restrict__ a, const T* xj, int r, int c0) {
    // block values through the read-only path, x through L2 (it changes
    // during the sweep)
    using L = WL<BR, BC>;
    T acc = 0;
#pragma unroll
    for (int c = 0; c < L::CH; ++c)
        if (c0 + c < BC) acc += __ldg(a + r * BC + c0 + c) * __ldcg(xj + c0 + c);
    return acc;
}

// y_r = sum_c D(r,c) t_c where t_c is held by lane c*S (rows' first lanes)
template <class T, int B>
__device__ __forceinline__ T apply_block(const T* __restrict__ D, T t_mine, int r, int c0) {
    using L = WL<B, B>;
    T acc = 0;
#pragma unroll
    for (int c = 0; c < L::CH; ++c) {
        const int cc = c0 + c;
        T tc = __shfl_sync(0xffffffffu, t_mine, (cc * L::S) & 31);
        if (cc < B && r < B) acc += __ldg(D + r * B + cc) * tc;
    }
    return seg_sum<L::S>(acc);
}

__device__ __forceinline__ bool wait_flag(const unsigned* f, unsigned target, GsSync* sync, int64_t timeout_ns) {
    const uint64_t t0 = globaltimer_ns();
    unsigned it = 0;
    while (true) {
        const unsigned v = ld_acquire_u32(f);
        if ((int)(v - target) >= 0) return true;
        if ((++it & 63u) == 0) {
            if (*(volatile unsigned*)&sync->err) return false;
            if ((int64_t)(globaltimer_ns() - t0) > timeout_ns) {
                atomicOr(&sync->err, 1u);
                return false;
            }
            __nanosleep(32);
        }
    }
}

// -------------------------------------------------------------- GS sweep --
// Up to MAXE earlier-neighbour blocks per row are loaded into registers
// before the row waits, together with its Dinv row chunk, b_i and old x_i,
// so that after a dependency is released only the neighbour's new x_j (an
// L2 read) and the arithmetic remain on the critical path.
template <class T, int B, int WPB, int MAXE>
__global__ void __launch_bounds__(WPB * 32)
    k_gs_sweep(int n, const int* __restrict__ row_ptr, const int* __restrict__ col_idx, const T* __restrict__ val,
               const T* __restrict__ Dinv, const T* __restrict__ b, T* x, const int* __restrict__ order,
               const int* __restrict__ wptr, const int* __restrict__ widx, unsigned* flags, GsSync* sync, T omega,
               int reverse, int64_t timeout_ns) {
    using L = WL<B, B>;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = lane / L::S, s = lane - r * L::S;
    const bool active = r < B;
    const int c0 = s * L::CH;
    const unsigned target = __ldcg(&sync->epoch) + 1u;
    bool failed = false;
    for (int w = blockIdx.x * WPB + warp; w < n && !failed; w += gridDim.x * WPB) {
        const int i = __ldg(order + w);
        const int k0 = __ldg(row_ptr + i), k1 = __ldg(row_ptr + i + 1);
        // ---- work that does not depend on this sweep's progress ----
        T bi = 0, xi = 0;
        if (active && s == 0) {
            bi = __ldg(b + (size_t)i * B + r);
            xi = __ldcg(x + (size_t)i * B + r);
        }
        T dch[L::CH];
        const T* Di = Dinv + (size_t)i * B * B;
#pragma unroll
        for (int c = 0; c < L::CH; ++c) dch[c] = (active && c0 + c < B) ? __ldg(Di + r * B + c0 + c) : T(0);
        T ech[MAXE][L::CH];
        int ej[MAXE];
#pragma unroll
        for (int q = 0; q < MAXE; ++q) ej[q] = -1;
        int ne = 0;
        T acc = 0;
        for (int k = k0; k < k1; ++k) {
            const int j = __ldg(col_idx + k);
            if (j == i) continue;
            const bool earlier = reverse ? (j > i) : (j < i);
            const T* a = val + (size_t)k * B * B;
            if (!earlier) {
                // later neighbour: its old value is stable until row i publishes
                if (active) acc += chunk_dot_coherent<T, B, B>(a, x + (size_t)j * B, r, c0);
            } else {
#pragma unroll
                for (int q = 0; q < MAXE; ++q)
                    if (q == ne) {
                        ej[q] = j;
#pragma unroll
                        for (int c = 0; c < L::CH; ++c)
                            ech[q][c] = (active && c0 + c < B) ? __ldg(a + r * B + c0 + c) : T(0);
                    }
                ++ne;
            }
        }
        // ---- wait for the earlier neighbours (one lane per flag) ----
        const int q0 = __ldg(wptr + i), q1 = __ldg(wptr + i + 1);
        for (int q = q0 + lane; q < q1; q += 32)
            if (!wait_flag(flags + __ldg(widx + q), target, sync, timeout_ns)) failed = true;
        __syncwarp();
        failed = __any_sync(0xffffffffu, failed);
        if (failed) break;
        // ---- earlier neighbours' new values ----
#pragma unroll
        for (int q = 0; q < MAXE; ++q)
            if (ej[q] >= 0 && active) {
                const T* xj = x + (size_t)ej[q] * B;
#pragma unroll
                for (int c = 0; c < L::CH; ++c)
                    if (c0 + c < B) acc += ech[q][c] * __ldcg(xj + c0 + c);
            }
        if (ne > MAXE) {
            // rows with more earlier neighbours than registers: reload the rest
            int seen = 0;
            for (int k = k0; k < k1; ++k) {
                const int j = __ldg(col_idx + k);
                const bool earlier = reverse ? (j > i) : (j < i);
                if (j == i || !earlier) continue;
                if (seen++ < MAXE) continue;
                if (active) acc += chunk_dot_coherent<T, B, B>(val + (size_t)k * B * B, x + (size_t)j * B, r, c0);
            }
        }
        acc = seg_sum<L::S>(acc);
        // t = b_i - sum_{j != i} A_ij x_j ;  x_i += omega (Dinv_i t - x_i)
        const T t = (active && s == 0) ? bi - acc : T(0);
        T y = 0;
#pragma unroll
        for (int c = 0; c < L::CH; ++c) {
            const int cc = c0 + c;
            const T tc = __shfl_sync(0xffffffffu, t, (cc * L::S) & 31);
            if (cc < B && active) y += dch[c] * tc;
        }
        y = seg_sum<L::S>(y);
        if (active && s == 0) x[(size_t)i * B + r] = xi + omega * (y - xi);
        // publish: the warp barrier orders every lane's store before lane 0's
        // release, which makes them visible with the flag
        __syncwarp();
        if (lane == 0) st_release_u32(flags + i, target);
    }
    // the last CTA to finish advances the sweep counter
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&sync->done, 1u);
        if (prev == gridDim.x - 1) {
            sync->done = 0;
            __threadfence();
            atomicExch(&sync->epoch, target);
        }
    }
}

// ------------------------------------------------------------ Jacobi sweep --
// x_out_i = x_in_i + omega * Dinv_i (b_i - sum_j A_ij x_in_j)
template <class T, int B, int WPB>
__global__ void __launch_bounds__(WPB * 32, 2)
    k_jacobi(int n, const int* __restrict__ row_ptr, const int* __restrict__ col_idx, const T* __restrict__ val,
             const T* __restrict__ Dinv, const T* __restrict__ b, const T* __restrict__ xin, T* __restrict__ xout,
             T omega) {
    using L = WL<B, B>;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = lane / L::S, s = lane - r * L::S;
    const bool active = r < B;
    const int c0 = s * L::CH;
    for (int i = blockIdx.x * WPB + warp; i < n; i += gridDim.x * WPB) {
        // the row's own data is independent of the product: issue it first
        T bi = 0, xi = 0;
        if (active && s == 0) {
            bi = __ldg(b + (size_t)i * B + r);
            xi = __ldg(xin + (size_t)i * B + r);
        }
        T dch[L::CH];
        const T* Di = Dinv + (size_t)i * B * B;
#pragma unroll
        for (int c = 0; c < L::CH; ++c) dch[c] = (active && c0 + c < B) ? __ldg(Di + r * B + c0 + c) : T(0);
        const int k0 = __ldg(row_ptr + i), k1 = __ldg(row_ptr + i + 1);
        T acc = row_product<T, B, B>(col_idx, val, nullptr, xin, k0, k1, r, c0, active, lane);
        acc = seg_sum<L::S>(acc);
        const T t = (active && s == 0) ? bi - acc : T(0);
        T y = 0;
#pragma unroll
        for (int c = 0; c < L::CH; ++c) {
            const int cc = c0 + c;
            const T tc = __shfl_sync(0xffffffffu, t, (cc * L::S) & 31);
            if (cc < B && active) y += dch[c] * tc;
        }
        y = seg_sum<L::S>(y);
        if (active && s == 0) xout[(size_t)i * B + r] = xi + omega * y;
    }
}

// Small blocks (B <= 10): 32 / B block rows per warp, one lane per block
// column for the product (cols_accumulate, rows_reduce), then lane (g, r)
// holds t_r = b_r - (A x_in)_r and applies row r of Dinv with t's entries
// shuffled within the group.  The row loop is warp-uniform so every lane
// takes part in the shuffles and the shared-memory reduction.
template <class T, class VT, int B, int MAXB>
__global__ void __launch_bounds__(256)
    k_jacobi_rows(int n, const int* __restrict__ row_ptr, const int* __restrict__ col_idx, const VT* __restrict__ val,
                  const float* __restrict__ scl, const T* __restrict__ Dinv, const T* __restrict__ b,
                  const T* __restrict__ xin, T* __restrict__ xout, T omega) {
    using R = Rows<B>;
    __shared__ T sr[8 * R::SM];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane / R::S, c = lane - g * R::S;
    T* s = sr + warp * R::SM;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int base = (blockIdx.x * (blockDim.x >> 5) + warp) * R::G; base < n; base += nw * R::G) {
        const int row = base + g;
        const bool valid = g < R::G && row < n;
        const size_t o = (size_t)row * B + c;
        T acc[B];
#pragma unroll
        for (int r = 0; r < B; ++r) acc[r] = 0;
        T bi = 0, xi = 0;
        if (valid) {
            bi = __ldg(b + o);
            xi = __ldg(xin + o);
            cols_accumulate<T, VT, B, B, MAXB>(col_idx, val, scl, nullptr, xin, __ldg(row_ptr + row),
                                               __ldg(row_ptr + row + 1), c, acc);
        }
        const T t = bi - rows_reduce<T, B, B>(acc, s, g, c, g < R::G);
        // lane (g, c) now holds t_c; y_c = sum_k Dinv(c, k) t_k
        const T* Di = Dinv + ((size_t)row * B + c) * B;
        const int src = (g < R::G ? g : 0) * B;
        T y = 0;
#pragma unroll
        for (int k = 0; k < B; ++k) {
            const T tk = __shfl_sync(0xffffffffu, t, src + k);
            if (valid) y = fma(__ldg(Di + k), tk, y);
        }
        if (valid) xout[o] = xi + omega * y;
    }
}

template <class T, int B, class VT = T>
static void launch_jacobi_rows(mgldg_ctx* ctx, const mgldg_bsr* A, const VT* vals, const T* Dinv, const T* b,
                               const T* xin, T* xout, T omega, const float* scl = nullptr) {
    constexpr int MAXB = (sizeof(T) == 4 || B <= 4) ? 4 : 2;
    const int rows_per_cta = 8 * Rows<B>::G;
    const int grid = std::max(1, std::min((A->nbr + rows_per_cta - 1) / rows_per_cta, ctx->sm_count * 8));
    {
        Launch L(ctx, MGLDG_K_JACOBI);
        k_jacobi_rows<T, VT, B, MAXB><<<grid, 256, 0, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, vals, scl, Dinv,
                                                                     b, xin, xout, omega);
    }
    check_launch();
}

// -------------------------------------------------------------- scheduling --
// Level sets of one sweep direction (dir 0: rows ascending, 1: descending).
// A row depends on its earlier neighbours in the symmetrised pattern (an
// entry A_ij or A_ji); level(i) = 1 + max level of those, 0 if none.
// Outputs the level of every row, the wait lists and the rows in level order.
void gs_levels_host(int n, const int* row_ptr, const int* col_idx, int dir, std::vector<int>& lev,
                    std::vector<int>& wp, std::vector<int>& wi, std::vector<int>& order, int& nlev) {
    std::vector<std::vector<int>> nb(n);
    for (int i = 0; i < n; ++i)
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            int j = col_idx[k];
            if (j == i || j < 0 || j >= n) continue;
            nb[i].push_back(j);
            nb[j].push_back(i);
        }
    for (auto& v : nb) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    lev.assign(n, 0);
    wp.assign(n + 1, 0);
    wi.clear();
    int maxlev = 0;
    for (int t = 0; t < n; ++t) {
        const int i = dir == 0 ? t : n - 1 - t;
        int l = 0;
        for (int j : nb[i]) {
            const bool earlier = dir == 0 ? (j < i) : (j > i);
            if (earlier) l = std::max(l, lev[j] + 1);
        }
        lev[i] = l;
        maxlev = std::max(maxlev, l);
    }
    for (int i = 0; i < n; ++i) {
        for (int j : nb[i]) {
            const bool earlier = dir == 0 ? (j < i) : (j > i);
            if (earlier) wi.push_back(j);
        }
        wp[i + 1] = (int)wi.size();
    }
    // counting sort by level; ascending rows inside a level for the forward
    // sweep, descending for the reverse sweep
    std::vector<int> cnt(maxlev + 2, 0);
    order.assign(n, 0);
    for (int i = 0; i < n; ++i) cnt[lev[i] + 1]++;
    for (int l = 0; l <= maxlev; ++l) cnt[l + 1] += cnt[l];
    for (int t = 0; t < n; ++t) {
        const int i = dir == 0 ? t : n - 1 - t;
        order[cnt[lev[i]]++] = i;
    }
    nlev = n ? maxlev + 1 : 0;
}

void sched_build(mgldg_ctx* ctx, const mgldg_bsr* A, Sched& S) {
    const int n = A->nbr;
    for (int dir = 0; dir < 2; ++dir) {
        std::vector<int> lev, wp, wi, order;
        gs_levels_host(n, A->h_row_ptr.data(), A->h_col_idx.data(), dir, lev, wp, wi, order, S.nlev[dir]);
        S.h_level[dir] = lev;
        S.order[dir] = dalloc<int>(std::max(1, n));
        S.wptr[dir] = dalloc<int>(n + 1);
        S.widx[dir] = dalloc<int>(std::max<size_t>(1, wi.size()));
        upload(ctx, S.order[dir], order.data(), order.size());
        upload(ctx, S.wptr[dir], wp.data(), wp.size());
        upload(ctx, S.widx[dir], wi.data(), wi.size());
    }
    S.n = n;
    S.flags = dalloc<unsigned>(std::max(1, n));
    S.sync = dalloc<GsSync>(1);
    MG_CHECK_CUDA(cudaMemsetAsync(S.flags, 0, std::max(1, n) * sizeof(unsigned), ctx->stream));
    MG_CHECK_CUDA(cudaMemsetAsync(S.sync, 0, sizeof(GsSync), ctx->stream));
    sync(ctx);
}

void sched_free(Sched& S) {
    for (int d = 0; d < 2; ++d) {
        dfree(S.order[d]);
        dfree(S.wptr[d]);
        dfree(S.widx[d]);
    }
    dfree(S.flags);
    dfree(S.sync);
}

int gs_take_error(mgldg_ctx* ctx, Sched& S) {
    if (!S.sync) return 0;
    GsSync h;
    download(ctx, &h, S.sync, 1);
    sync(ctx);
    if (h.err) {
        // clear the error word; flags stay monotone, so the next sweep's
        // target exceeds every stale flag and the schedule stays valid
        unsigned zero = 0;
        upload(ctx, &S.sync->err, &zero, 1);
        sync(ctx);
        return 1;
    }
    return 0;
}

template <class T, int B>
static void launch_gs(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, T* x, Sched& S,
                      T omega, bool reverse) {
    constexpr int WPB = 4;
    auto kern = k_gs_sweep<T, B, WPB, 4>;
    int per_sm = 0;
    MG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WPB * 32, 0));
    MG_REQUIRE(per_sm > 0, MGLDG_ERR_CUDA, "Gauss-Seidel kernel does not fit on an SM");
    int grid = std::max(1, std::min((S.n + WPB - 1) / WPB, per_sm * ctx->sm_count));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(WPB * 32);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = ctx->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;   // all CTAs co-resident
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const int dir = reverse ? 1 : 0;
    {
        Launch L(ctx, MGLDG_K_GS);
        MG_CHECK_CUDA(cudaLaunchKernelEx(&cfg, kern, S.n, (const int*)A->row_ptr, (const int*)A->col_idx, vals, Dinv, b,
                                         x, (const int*)S.order[dir], (const int*)S.wptr[dir], (const int*)S.widx[dir],
                                         S.flags, S.sync, omega, (int)reverse, S.timeout_ns));
    }
}

template <class T>
void gs_sweep(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, T* x, Sched& S, T omega,
              bool reverse) {
    if (S.n == 0) return;
    MG_REQUIRE(A->br == A->bc, MGLDG_ERR_SHAPE, "smoother needs square blocks");
    switch (A->br) {
        case 1: launch_gs<T, 1>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 3: launch_gs<T, 3>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 4: launch_gs<T, 4>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 6: launch_gs<T, 6>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 8: launch_gs<T, 8>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 9: launch_gs<T, 9>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 10: launch_gs<T, 10>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 16: launch_gs<T, 16>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 25: launch_gs<T, 25>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
        case 27: launch_gs<T, 27>(ctx, A, vals, Dinv, b, x, S, omega, reverse); return;
    }
    throw Error(MGLDG_ERR_UNSUPPORTED, "Gauss-Seidel: unsupported block size");
}
template void gs_sweep<double>(mgldg_ctx*, const mgldg_bsr*, const double*, const double*, const double*, double*,
                               Sched&, double, bool);
template void gs_sweep<float>(mgldg_ctx*, const mgldg_bsr*, const float*, const float*, const float*, float*, Sched&,
                              float, bool);

template <class T, int B>
static void launch_jacobi(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b,
                          const T* xin, T* xout, T omega) {
    constexpr int WPB = 8;
    int grid = std::max(1, std::min((A->nbr + WPB - 1) / WPB, ctx->sm_count * 16));
    {
        Launch L(ctx, MGLDG_K_JACOBI);
        k_jacobi<T, B, WPB><<<grid, WPB * 32, 0, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, vals, Dinv, b, xin,
                                                                xout, omega);
    }
    check_launch();
}

template <class T>
void jacobi_sweep(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, const T* xin,
                  T* xout, T omega) {
    if (A->nbr == 0) return;
    if constexpr (std::is_same<T, float>::value) {
        if (bulk_jacobi_f32(ctx, A, vals, Dinv, b, xin, xout, omega)) return;
    }
    if (!A->blk) switch (A->br) {
            case 3: launch_jacobi_rows<T, 3>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
            case 4: launch_jacobi_rows<T, 4>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
            case 6: launch_jacobi_rows<T, 6>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
            case 8: launch_jacobi_rows<T, 8>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
            case 9: launch_jacobi_rows<T, 9>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
            case 10: launch_jacobi_rows<T, 10>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        }
    switch (A->br) {
        case 1: launch_jacobi<T, 1>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 3: launch_jacobi<T, 3>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 4: launch_jacobi<T, 4>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 6: launch_jacobi<T, 6>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 8: launch_jacobi<T, 8>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 9: launch_jacobi<T, 9>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 10: launch_jacobi<T, 10>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 16: launch_jacobi<T, 16>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 25: launch_jacobi<T, 25>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
        case 27: launch_jacobi<T, 27>(ctx, A, vals, Dinv, b, xin, xout, omega); return;
    }
    throw Error(MGLDG_ERR_UNSUPPORTED, "Jacobi: unsupported block size");
}
bool jacobi_f16(mgldg_ctx* ctx, const mgldg_bsr* A, const float* Dinv, const float* b, const float* xin, float* xout,
                float omega) {
    if (!A->val16 || A->blk || A->nbr == 0 || !f16_shape(A->br, A->bc)) return false;
    return bulk_jacobi_f16(ctx, A, Dinv, b, xin, xout, omega);
}

template void jacobi_sweep<double>(mgldg_ctx*, const mgldg_bsr*, const double*, const double*, const double*,
                                   const double*, double*, double);
template void jacobi_sweep<float>(mgldg_ctx*, const mgldg_bsr*, const float*, const float*, const float*, const float*,
                                  float*, float);

}  // namespace mg

// ================================================================== C ABI ==
extern "C" int mgldg_gs_levels(int nbr, const int* row_ptr, const int* col_idx, int reverse, int* level,
                               int* order, int* nlevels) {
    if (nbr < 0 || !row_ptr || (nbr > 0 && row_ptr[nbr] > 0 && !col_idx)) return MGLDG_ERR_ARG;
    try {
        std::vector<int> lev, wp, wi, ord;
        int nl = 0;
        mg::gs_levels_host(nbr, row_ptr, col_idx, reverse ? 1 : 0, lev, wp, wi, ord, nl);
        if (level) std::copy(lev.begin(), lev.end(), level);
        if (order) std::copy(ord.begin(), ord.end(), order);
        if (nlevels) *nlevels = nl;
    } catch (...) {
        return MGLDG_ERR_NOMEM;
    }
    return MGLDG_OK;
}

// Runs the Gauss-Seidel kernel on a two-row system in which row 1 waits for
// row 0 but row 0 is never scheduled, so the wait can only end by its time
// limit.  Reports the status the kernel left and checks that the stream is
// still usable afterwards.
extern "C" int mgldg_selftest_wait_timeout(mgldg_ctx* ctx, int64_t timeout_ns, int* status) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(status && timeout_ns > 0 && timeout_ns <= 2000000000LL, MGLDG_ERR_ARG, "bad self-test arguments");
    std::vector<int> rp{0, 2, 4}, ci{0, 1, 0, 1};
    mgldg_bsr* A = bsr_new(ctx, 2, 2, 1, 1, rp, ci);
    Sched S;
    double *dinv = nullptr, *b = nullptr, *x = nullptr;
    try {
        const double av[4] = {2.0, 1.0, 1.0, 2.0}, dv[2] = {0.5, 0.5}, zero[2] = {0.0, 0.0};
        upload(ctx, A->val, av, 4);
        dinv = dalloc<double>(2); b = dalloc<double>(2); x = dalloc<double>(2);
        upload(ctx, dinv, dv, 2); upload(ctx, b, dv, 2); upload(ctx, x, zero, 2);
        const int ord[1] = {1}, wp[3] = {0, 0, 1}, wi[1] = {0};
        S.n = 1;
        S.order[0] = dalloc<int>(1); S.wptr[0] = dalloc<int>(3); S.widx[0] = dalloc<int>(1);
        upload(ctx, S.order[0], ord, 1); upload(ctx, S.wptr[0], wp, 3); upload(ctx, S.widx[0], wi, 1);
        S.flags = dalloc<unsigned>(2);
        S.sync = dalloc<GsSync>(1);
        MG_CHECK_CUDA(cudaMemsetAsync(S.flags, 0, 2 * sizeof(unsigned), ctx->stream));
        MG_CHECK_CUDA(cudaMemsetAsync(S.sync, 0, sizeof(GsSync), ctx->stream));
        S.timeout_ns = timeout_ns;
        gs_sweep<double>(ctx, A, A->val, dinv, b, x, S, 1.0, false);
        sync(ctx);
        *status = gs_take_error(ctx, S) ? MGLDG_ERR_TIMEOUT : MGLDG_OK;
        // the context must still work: a plain SpMV
        spmv<double>(ctx, A, 1.0, b, 0.0, nullptr, x);
        sync(ctx);
    } catch (...) {
        sched_free(S);
        dfree(dinv); dfree(b); dfree(x);
        delete A;
        throw;
    }
    sched_free(S);
    dfree(dinv); dfree(b); dfree(x);
    delete A;
    MG_API_END
}

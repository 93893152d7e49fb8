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

// ------------------------------------------------------------ GS pass --
// One launch runs a smoothing pass: nsw consecutive sweeps in one direction
// (the npre forward or npost reverse sweeps of multigrid.h:202-216).  Its
// work items are (sweep s, row i), ordered by the level sets of the combined
// dependency graph: (s, i) needs sweep s's new values of its earlier
// neighbours and sweep s-1's values of its later neighbours and of itself, so
// sweep s+1 trails sweep s by a few levels instead of starting after it
// (2 n_side + 1 dependent steps for two sweeps of an n_side^2 grid, not
// 2 (2 n_side - 1)).  Every row reads exactly the values the sequential
// sweeps of the reference read.
//
// Rows publish their values as packed 64-bit words, (epoch << 32) | 32 value
// bits: one word per FP32 entry, two (high and low halves) per FP64 entry,
// written and read with relaxed gpu-scope 64-bit accesses (single-copy
// atomic), so a reader that finds every word of a row at the epoch it needs
// holds that version of the row -- no separate flag, fence or second read on
// the dependency's critical path.  Epoch base + s + 1 marks sweep s of the
// launch whose device-side counter reads base; the last CTA to finish adds
// nsw.  Values a row reads before its launch's first sweep touches them come
// from the plain vector x, which only the last sweep of the pass writes.
// Every wait is bounded (about one second of %globaltimer); on expiry the
// kernel records an error word, every other waiter gives up and the host
// returns MGLDG_ERR_TIMEOUT with the context still usable.
template <class T>
struct Packed {
    static constexpr int WPV = sizeof(T) / 4;   // 64-bit words per entry
};

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Reads the packed row j (W words, word w in lane w % 32, register w / 32)
// until every word carries an epoch at or after tgt.  Warp-uniform result:
// false if the wait ran out or another waiter gave up.
template <int W>
__device__ __forceinline__ bool read_row(const unsigned long long* xp, int j, unsigned tgt, unsigned (&v)[(W + 31) / 32],
                                         GsSync* sync, int64_t timeout_ns, int lane) {
    constexpr int NW = (W + 31) / 32;
    const unsigned long long* row = xp + (size_t)j * W;
    uint64_t t0 = 0;
    unsigned it = 0;
    while (true) {
        bool ok = true;
#pragma unroll
        for (int q = 0; q < NW; ++q) {
            const int w = lane + 32 * q;
            if (w < W) {
                const unsigned long long u = ld_relaxed_u64(row + w);
                v[q] = (unsigned)u;
                ok = ok && (int)((unsigned)(u >> 32) - tgt) >= 0;
            }
        }
        if (__all_sync(0xffffffffu, ok)) return true;
        ++it;
        if (it == 1) t0 = globaltimer_ns();
        if ((it & 15u) == 0) {
            bool stop = *(volatile unsigned*)&sync->err != 0;
            if (!stop && (int64_t)(globaltimer_ns() - t0) > timeout_ns) {
                atomicOr(&sync->err, 1u);
                stop = true;
            }
            if (__any_sync(0xffffffffu, stop)) return false;
        }
    }
}

// Polls several packed rows at once: the rows of the slots in `sel` (a
// warp-uniform bit mask) are loaded together, one L2 round trip per polling
// round, until every word of each carries an epoch at or after its target.
// Warp-uniform result: false if the wait ran out or another waiter gave up.
template <int W, int MAXE>
__device__ __forceinline__ bool poll_rows(const unsigned long long* xp, const int (&rows)[MAXE],
                                          const unsigned (&tgt)[MAXE], unsigned sel,
                                          unsigned (&v)[MAXE][(W + 31) / 32], GsSync* sync, int64_t timeout_ns,
                                          int lane) {
    constexpr int NW = (W + 31) / 32;
    uint64_t t0 = 0;
    unsigned it = 0;
    unsigned pending = sel;
    while (pending) {
        unsigned long long u[MAXE][NW];
        // issue every load of the round before checking any of them
#pragma unroll
        for (int q = 0; q < MAXE; ++q)
            if ((pending >> q) & 1u) {
                const unsigned long long* row = xp + (size_t)rows[q] * W;
#pragma unroll
                for (int k = 0; k < NW; ++k) {
                    const int w = lane + 32 * k;
                    u[q][k] = w < W ? ld_relaxed_u64(row + w) : ((unsigned long long)tgt[q] << 32);
                }
            }
        unsigned still = 0;
#pragma unroll
        for (int q = 0; q < MAXE; ++q)
            if ((pending >> q) & 1u) {
                bool ok = true;
#pragma unroll
                for (int k = 0; k < NW; ++k) {
                    v[q][k] = (unsigned)u[q][k];
                    ok = ok && (int)((unsigned)(u[q][k] >> 32) - tgt[q]) >= 0;
                }
                if (!__all_sync(0xffffffffu, ok)) still |= 1u << q;
            }
        pending = still;
        if (!pending) return true;
        ++it;
        if (it == 1) t0 = globaltimer_ns();
        if ((it & 15u) == 0) {
            bool stop = *(volatile unsigned*)&sync->err != 0;
            if (!stop && (int64_t)(globaltimer_ns() - t0) > timeout_ns) {
                atomicOr(&sync->err, 1u);
                stop = true;
            }
            if (__any_sync(0xffffffffu, stop)) return false;
        }
    }
    return true;
}

// entry cc of a row read by read_row (every lane of the warp takes part)
template <class T, int W>
__device__ __forceinline__ T row_entry(const unsigned (&v)[(W + 31) / 32], int cc) {
    constexpr int NW = (W + 31) / 32;
    if constexpr (sizeof(T) == 4) {
        unsigned u = __shfl_sync(0xffffffffu, v[0], cc & 31);
        if constexpr (NW > 1) {
            const unsigned u1 = __shfl_sync(0xffffffffu, v[1], cc & 31);
            if (cc >= 32) u = u1;
        }
        return __uint_as_float(u);
    } else {
        const int wh = 2 * cc, wl = 2 * cc + 1;
        unsigned h = __shfl_sync(0xffffffffu, v[0], wh & 31);
        unsigned l = __shfl_sync(0xffffffffu, v[0], wl & 31);
        if constexpr (NW > 1) {
            const unsigned h1 = __shfl_sync(0xffffffffu, v[1], wh & 31);
            const unsigned l1 = __shfl_sync(0xffffffffu, v[1], wl & 31);
            if (wh >= 32) h = h1;
            if (wl >= 32) l = l1;
        }
        return __hiloint2double((int)h, (int)l);
    }
}

template <class T>
__device__ __forceinline__ void publish(unsigned long long* xp, size_t e, T val, unsigned tag) {
    const unsigned long long hi = (unsigned long long)tag << 32;
    if constexpr (sizeof(T) == 4) {
        st_relaxed_u64(xp + e, hi | __float_as_uint(val));
    } else {
        st_relaxed_u64(xp + 2 * e, hi | (unsigned)__double2hiint(val));
        st_relaxed_u64(xp + 2 * e + 1, hi | (unsigned)__double2loint(val));
    }
}

// Up to MAXE neighbour blocks per row (every neighbour whose value the row
// waits for) are loaded into registers, with the row's Dinv chunk and b_i,
// before the row waits; the later neighbours of the pass's first sweep are
// multiplied at once (their values predate the launch).
template <class T, int B, int WPB, int MAXE>
__global__ void __launch_bounds__(WPB * 32)
    k_gs_pass(int nitems, const int* __restrict__ items, int nsw, const int* __restrict__ row_ptr,
              const int* __restrict__ col_idx, const T* __restrict__ val, const T* __restrict__ Dinv,
              const T* __restrict__ b, T* x, unsigned long long* xp, const int* __restrict__ xptr,
              const int* __restrict__ xidx, GsSync* sync, T omega, int reverse, int64_t timeout_ns) {
    using L = WL<B, B>;
    constexpr int W = B * Packed<T>::WPV;
    constexpr int NW = (W + 31) / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = lane / L::S, sl = lane - r * L::S;
    const bool active = r < B;
    const int c0 = sl * L::CH;
    const unsigned base = __ldcg(&sync->epoch);
    bool failed = false;
    for (int w = blockIdx.x * WPB + warp; w < nitems && !failed; w += gridDim.x * WPB) {
        const int item = __ldg(items + w);
        const int i = item >> 3, s = item & 7;
        const unsigned tgt_new = base + (unsigned)s + 1u;   // this sweep's values
        const unsigned tgt_old = base + (unsigned)s;        // the previous sweep's values
        const int k0 = __ldg(row_ptr + i), k1 = __ldg(row_ptr + i + 1);
        // ---- work that does not depend on the pass's progress ----
        T bi = 0, xi = 0;
        if (active && sl == 0) {
            bi = __ldg(b + (size_t)i * B + r);
            if (s == 0) xi = __ldcg(x + (size_t)i * B + r);
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
            if (!earlier && s == 0) {
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
        // ---- neighbours of the symmetrised pattern outside the row's own
        // pattern: wait for them without reading ----
        const int e0 = __ldg(xptr + i), e1 = __ldg(xptr + i + 1);
        for (int q = e0; q < e1 && !failed; ++q) {
            const int j = __ldg(xidx + q);
            const bool earlier = reverse ? (j > i) : (j < i);
            if (!earlier && s == 0) continue;
            unsigned v[NW];
            if (!read_row<W>(xp, j, earlier ? tgt_new : tgt_old, v, sync, timeout_ns, lane)) failed = true;
        }
        if (failed) break;
        // ---- neighbours' values at the versions this sweep reads: first the
        // later neighbours and the row itself (the previous sweep's values,
        // usually published long before), then the earlier neighbours (this
        // sweep's values, the dependency chain); each group is polled as a
        // batch and summed in column order ----
        unsigned tg[MAXE + 1];
        int rw[MAXE + 1];
        unsigned later_sel = 0, earlier_sel = 0;
#pragma unroll
        for (int q = 0; q < MAXE; ++q) {
            rw[q] = ej[q] < 0 ? i : ej[q];
            const bool earlier = reverse ? (ej[q] > i) : (ej[q] < i);
            tg[q] = earlier ? tgt_new : tgt_old;
            if (ej[q] >= 0) {
                if (earlier) earlier_sel |= 1u << q;
                else later_sel |= 1u << q;
            }
        }
        rw[MAXE] = i;
        tg[MAXE] = tgt_old;
        if (s > 0) later_sel |= 1u << MAXE;
        unsigned v[MAXE + 1][NW];
        if (later_sel && !poll_rows<W, MAXE + 1>(xp, rw, tg, later_sel, v, sync, timeout_ns, lane)) failed = true;
        if (failed) break;
#pragma unroll
        for (int q = 0; q < MAXE; ++q) {
            if (!((later_sel >> q) & 1u)) continue;
#pragma unroll
            for (int c = 0; c < L::CH; ++c) {
                const int cc = c0 + c;
                const T xv = row_entry<T, W>(v[q], cc < B ? cc : 0);
                if (cc < B && active) acc += ech[q][c] * xv;
            }
        }
        if (s > 0) {
            const T xv = row_entry<T, W>(v[MAXE], active ? r : 0);
            if (active && sl == 0) xi = xv;
        }
        if (earlier_sel && !poll_rows<W, MAXE + 1>(xp, rw, tg, earlier_sel, v, sync, timeout_ns, lane)) failed = true;
        if (failed) break;
#pragma unroll
        for (int q = 0; q < MAXE; ++q) {
            if (!((earlier_sel >> q) & 1u)) continue;
#pragma unroll
            for (int c = 0; c < L::CH; ++c) {
                const int cc = c0 + c;
                const T xv = row_entry<T, W>(v[q], cc < B ? cc : 0);
                if (cc < B && active) acc += ech[q][c] * xv;
            }
        }
        if (ne > MAXE) {
            // rows with more waited-for neighbours than registers: the rest,
            // one at a time
            int seen = 0;
            for (int k = k0; k < k1 && !failed; ++k) {
                const int j = __ldg(col_idx + k);
                const bool earlier = reverse ? (j > i) : (j < i);
                if (j == i || (!earlier && s == 0)) continue;
                if (seen++ < MAXE) continue;
                unsigned v1[NW];
                if (!read_row<W>(xp, j, earlier ? tgt_new : tgt_old, v1, sync, timeout_ns, lane)) {
                    failed = true;
                    break;
                }
                const T* a = val + (size_t)k * B * B;
#pragma unroll
                for (int c = 0; c < L::CH; ++c) {
                    const int cc = c0 + c;
                    const T xv = row_entry<T, W>(v1, cc < B ? cc : 0);
                    if (cc < B && active) acc += __ldg(a + r * B + cc) * xv;
                }
            }
        }
        if (failed) break;
        acc = seg_sum<L::S>(acc);
        // t = b_i - sum_{j != i} A_ij x_j ;  x_i += omega (Dinv_i t - x_i)
        const T t = (active && sl == 0) ? bi - acc : T(0);
        T y = 0;
#pragma unroll
        for (int c = 0; c < L::CH; ++c) {
            const int cc = c0 + c;
            const T tc = __shfl_sync(0xffffffffu, t, (cc * L::S) & 31);
            if (cc < B && active) y += dch[c] * tc;
        }
        y = seg_sum<L::S>(y);
        if (active && sl == 0) {
            const T xn = xi + omega * (y - xi);
            if (s == nsw - 1) x[(size_t)i * B + r] = xn;
            publish<T>(xp, (size_t)i * B + r, xn, tgt_new);
        }
    }
    // the last CTA to finish advances the epoch past this pass
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned prev = atomicAdd(&sync->done, 1u);
        if (prev == gridDim.x - 1) {
            sync->done = 0;
            __threadfence();
            atomicExch(&sync->epoch, base + (unsigned)nsw);
        }
    }
}

// ------------------------------------------------------------ Jacobi sweep --
// x_out_i = x_in_i + omega * Dinv_i (b_i - sum_j A_ij x_in_j)
//
// xzero: x_in is the zero vector (the first sweep of a V-cycle level), so
// the kernels neither read A nor x_in.  The product of A with zeros is +0 in
// every lane and b_i - (+0) = b_i, so the sweep still gives the full
// sweep's values bit for bit.
template <class T, int B, int WPB>
__global__ void __launch_bounds__(WPB * 32, 2)
    k_jacobi(int n, const int* __restrict__ row_ptr, const int* __restrict__ col_idx, const T* __restrict__ val,
             const T* __restrict__ Dinv, const T* __restrict__ b, const T* __restrict__ xin, T* __restrict__ xout,
             T omega, bool xzero) {
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
            if (!xzero) xi = __ldg(xin + (size_t)i * B + r);
        }
        T dch[L::CH];
        const T* Di = Dinv + (size_t)i * B * B;
#pragma unroll
        for (int c = 0; c < L::CH; ++c) dch[c] = (active && c0 + c < B) ? __ldg(Di + r * B + c0 + c) : T(0);
        T acc = 0;
        if (!xzero) {
            const int k0 = __ldg(row_ptr + i), k1 = __ldg(row_ptr + i + 1);
            acc = row_product<T, B, B>(col_idx, val, nullptr, xin, k0, k1, r, c0, active, lane);
            acc = seg_sum<L::S>(acc);
        }
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
                  const T* __restrict__ xin, T* __restrict__ xout, T omega, bool xzero) {
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
            if (!xzero) {
                xi = __ldg(xin + o);
                cols_accumulate<T, VT, B, B, MAXB>(col_idx, val, scl, nullptr, xin, __ldg(row_ptr + row),
                                                   __ldg(row_ptr + row + 1), c, acc);
            }
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
                               const T* xin, T* xout, T omega, bool xzero, const float* scl = nullptr) {
    constexpr int MAXB = (sizeof(T) == 4 || B <= 4) ? 4 : 2;
    const int rows_per_cta = 8 * Rows<B>::G;
    const int grid = std::max(1, std::min((A->nbr + rows_per_cta - 1) / rows_per_cta, ctx->sm_count * 8));
    {
        Launch L(ctx, MGLDG_K_JACOBI);
        k_jacobi_rows<T, VT, B, MAXB><<<grid, 256, 0, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, vals, scl, Dinv,
                                                                     b, xin, xout, omega, xzero);
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

static void symmetrised_neighbours(int n, const int* row_ptr, const int* col_idx, std::vector<std::vector<int>>& nb) {
    nb.assign(n, {});
    for (int i = 0; i < n; ++i)
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
            const int j = col_idx[k];
            if (j == i || j < 0 || j >= n) continue;
            nb[i].push_back(j);
            nb[j].push_back(i);
        }
    for (auto& v : nb) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
}

void sched_build(mgldg_ctx* ctx, const mgldg_bsr* A, Sched& S) {
    const int n = A->nbr;
    S.n = n;
    S.A = A;
    symmetrised_neighbours(n, A->h_row_ptr.data(), A->h_col_idx.data(), S.nb);
    // neighbours j of i with A_ji stored but not A_ij: waited for, not read
    std::vector<int> xp_(n + 1, 0), xi;
    for (int i = 0; i < n; ++i) {
        const int* c0 = A->h_col_idx.data() + A->h_row_ptr[i];
        const int* c1 = A->h_col_idx.data() + A->h_row_ptr[i + 1];
        for (int j : S.nb[i])
            if (std::find(c0, c1, j) == c1) xi.push_back(j);
        xp_[i + 1] = (int)xi.size();
    }
    S.xptr = dalloc<int>(n + 1);
    S.xidx = dalloc<int>(std::max<size_t>(1, xi.size()));
    upload(ctx, S.xptr, xp_.data(), xp_.size());
    if (!xi.empty()) upload(ctx, S.xidx, xi.data(), xi.size());
    S.sync = dalloc<GsSync>(1);
    MG_CHECK_CUDA(cudaMemsetAsync(S.sync, 0, sizeof(GsSync), ctx->stream));
    sync(ctx);
}

// Level sets of nsw consecutive sweeps: (s, i) follows (s, j) for earlier
// neighbours j, (s - 1, j) for later neighbours j and (s - 1, i).
// lev[s * n + i] is the level of (s, i); returns the number of levels.
static int gs_pass_levels_host(int n, const std::vector<std::vector<int>>& nb, int dir, int nsw, std::vector<int>& lev) {
    lev.assign((size_t)nsw * n, 0);
    int maxlev = -1;
    for (int s = 0; s < nsw; ++s)
        for (int t = 0; t < n; ++t) {
            const int i = dir == 0 ? t : n - 1 - t;
            int l = s > 0 ? lev[(size_t)(s - 1) * n + i] + 1 : 0;
            for (int j : nb[i]) {
                const bool earlier = dir == 0 ? (j < i) : (j > i);
                if (earlier) l = std::max(l, lev[(size_t)s * n + j] + 1);
                else if (s > 0) l = std::max(l, lev[(size_t)(s - 1) * n + j] + 1);
            }
            lev[(size_t)s * n + i] = l;
            maxlev = std::max(maxlev, l);
        }
    return maxlev + 1;
}

static void pass_build(mgldg_ctx* ctx, Sched& S, int dir, int nsw, GsPass& P) {
    const int n = S.n;
    MG_REQUIRE(n < (1 << 28) && nsw >= 1 && nsw <= 7, MGLDG_ERR_UNSUPPORTED, "Gauss-Seidel pass too large");
    std::vector<int> lev;
    const int maxlev = gs_pass_levels_host(n, S.nb, dir, nsw, lev) - 1;
    // counting sort by level; inside a level by sweep, then in sweep order
    std::vector<int> cnt(maxlev + 2, 0);
    for (int l : lev) cnt[l + 1]++;
    for (int l = 0; l <= maxlev; ++l) cnt[l + 1] += cnt[l];
    std::vector<int> items((size_t)nsw * n);
    for (int s = 0; s < nsw; ++s)
        for (int t = 0; t < n; ++t) {
            const int i = dir == 0 ? t : n - 1 - t;
            items[cnt[lev[(size_t)s * n + i]]++] = (i << 3) | s;
        }
    P.nsw = nsw;
    P.dir = dir;
    P.nitems = nsw * n;
    P.depth = n ? maxlev + 1 : 0;
    P.items = dalloc<int>(std::max<size_t>(1, items.size()));
    upload(ctx, P.items, items.data(), items.size());
    sync(ctx);
}

static GsPass& get_pass(mgldg_ctx* ctx, Sched& S, int dir, int nsw) {
    for (auto& P : S.passes)
        if (P.dir == dir && P.nsw == nsw) return P;
    GsPass P;
    try {
        pass_build(ctx, S, dir, nsw, P);
    } catch (...) {
        dfree(P.items);
        throw;
    }
    S.passes.push_back(P);
    return S.passes.back();
}

void sched_free(Sched& S) {
    for (auto& P : S.passes) dfree(P.items);
    S.passes.clear();
    dfree(S.xptr);
    dfree(S.xidx);
    dfree(S.xp);
    dfree(S.sync);
    S.xptr = S.xidx = nullptr;
    S.xp = nullptr;
    S.sync = nullptr;
}

int gs_take_error(mgldg_ctx* ctx, Sched& S) {
    if (!S.sync) return 0;
    GsSync h;
    download(ctx, &h, S.sync, 1);
    sync(ctx);
    if (h.err) {
        // clear the error word; epochs stay monotone, so the next pass's
        // targets exceed every stale word and the schedule stays valid
        unsigned zero = 0;
        upload(ctx, &S.sync->err, &zero, 1);
        sync(ctx);
        return 1;
    }
    return 0;
}

template <class T, int B>
static void launch_gs(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, T* x, Sched& S,
                      T omega, bool reverse, int nsw) {
    constexpr int WPB = 4;
    constexpr int MAXE = B <= 10 ? 8 : (B <= 16 ? 4 : 1);
    auto kern = k_gs_pass<T, B, WPB, MAXE>;
    const int words = B * Packed<T>::WPV;
    if (!S.xp || S.words_per_row != words) {
        dfree(S.xp);
        S.xp = nullptr;
        S.xp = dalloc<unsigned long long>((size_t)std::max(1, S.n) * words);
        S.words_per_row = words;
        MG_CHECK_CUDA(cudaMemsetAsync(S.xp, 0, (size_t)std::max(1, S.n) * words * sizeof(unsigned long long),
                                      ctx->stream));
        // epochs restart below every word
        MG_CHECK_CUDA(cudaMemsetAsync(S.sync, 0, sizeof(GsSync), ctx->stream));
    }
    GsPass& P = get_pass(ctx, S, reverse ? 1 : 0, nsw);
    int per_sm = 0;
    MG_CHECK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, WPB * 32, 0));
    MG_REQUIRE(per_sm > 0, MGLDG_ERR_CUDA, "Gauss-Seidel kernel does not fit on an SM");
    const int grid = std::max(1, std::min((P.nitems + WPB - 1) / WPB, per_sm * ctx->sm_count));
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
    {
        Launch L(ctx, MGLDG_K_GS);
        MG_CHECK_CUDA(cudaLaunchKernelEx(&cfg, kern, P.nitems, (const int*)P.items, nsw, (const int*)A->row_ptr,
                                         (const int*)A->col_idx, vals, Dinv, b, x, S.xp, (const int*)S.xptr,
                                         (const int*)S.xidx, S.sync, omega, (int)reverse, S.timeout_ns));
    }
}

template <class T>
void gs_sweeps(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, T* x, Sched& S, T omega,
               bool reverse, int nsw) {
    if (S.n == 0 || nsw <= 0) return;
    MG_REQUIRE(A->br == A->bc, MGLDG_ERR_SHAPE, "smoother needs square blocks");
    while (nsw > 0) {
        const int k = std::min(nsw, 4);
        switch (A->br) {
            case 1: launch_gs<T, 1>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 3: launch_gs<T, 3>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 4: launch_gs<T, 4>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 6: launch_gs<T, 6>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 8: launch_gs<T, 8>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 9: launch_gs<T, 9>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 10: launch_gs<T, 10>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 16: launch_gs<T, 16>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 25: launch_gs<T, 25>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            case 27: launch_gs<T, 27>(ctx, A, vals, Dinv, b, x, S, omega, reverse, k); break;
            default: throw Error(MGLDG_ERR_UNSUPPORTED, "Gauss-Seidel: unsupported block size");
        }
        nsw -= k;
    }
}
template void gs_sweeps<double>(mgldg_ctx*, const mgldg_bsr*, const double*, const double*, const double*, double*,
                                Sched&, double, bool, int);
template void gs_sweeps<float>(mgldg_ctx*, const mgldg_bsr*, const float*, const float*, const float*, float*, Sched&,
                               float, bool, int);

template <class T, int B>
static void launch_jacobi(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b,
                          const T* xin, T* xout, T omega, bool xzero) {
    constexpr int WPB = 8;
    int grid = std::max(1, std::min((A->nbr + WPB - 1) / WPB, ctx->sm_count * 16));
    {
        Launch L(ctx, MGLDG_K_JACOBI);
        k_jacobi<T, B, WPB><<<grid, WPB * 32, 0, ctx->stream>>>(A->nbr, A->row_ptr, A->col_idx, vals, Dinv, b, xin,
                                                                xout, omega, xzero);
    }
    check_launch();
}

template <class T>
void jacobi_sweep(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, const T* xin,
                  T* xout, T omega, bool xzero) {
    if (A->nbr == 0) return;
    if constexpr (std::is_same<T, float>::value) {
        if (bulk_jacobi_f32(ctx, A, vals, Dinv, b, xin, xout, omega, xzero)) return;
    }
    if (!A->blk) switch (A->br) {
            case 3: launch_jacobi_rows<T, 3>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
            case 4: launch_jacobi_rows<T, 4>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
            case 6: launch_jacobi_rows<T, 6>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
            case 8: launch_jacobi_rows<T, 8>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
            case 9: launch_jacobi_rows<T, 9>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
            case 10: launch_jacobi_rows<T, 10>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        }
    switch (A->br) {
        case 1: launch_jacobi<T, 1>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 3: launch_jacobi<T, 3>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 4: launch_jacobi<T, 4>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 6: launch_jacobi<T, 6>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 8: launch_jacobi<T, 8>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 9: launch_jacobi<T, 9>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 10: launch_jacobi<T, 10>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 16: launch_jacobi<T, 16>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 25: launch_jacobi<T, 25>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
        case 27: launch_jacobi<T, 27>(ctx, A, vals, Dinv, b, xin, xout, omega, xzero); return;
    }
    throw Error(MGLDG_ERR_UNSUPPORTED, "Jacobi: unsupported block size");
}
bool jacobi_f16(mgldg_ctx* ctx, const mgldg_bsr* A, const float* Dinv, const float* b, const float* xin, float* xout,
                float omega, bool xzero) {
    if (!A->val16 || A->blk || A->nbr == 0 || !f16_shape(A->br, A->bc)) return false;
    return bulk_jacobi_f16(ctx, A, Dinv, b, xin, xout, omega, xzero);
}

template void jacobi_sweep<double>(mgldg_ctx*, const mgldg_bsr*, const double*, const double*, const double*,
                                   const double*, double*, double, bool);
template void jacobi_sweep<float>(mgldg_ctx*, const mgldg_bsr*, const float*, const float*, const float*, const float*,
                                  float*, float, bool);

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

extern "C" int mgldg_gs_pass_levels(int nbr, const int* row_ptr, const int* col_idx, int reverse, int nsw,
                                    int* level, int* nlevels) {
    if (nbr < 0 || !row_ptr || nsw < 1 || nsw > 7 || (nbr > 0 && row_ptr[nbr] > 0 && !col_idx)) return MGLDG_ERR_ARG;
    try {
        std::vector<std::vector<int>> nb;
        mg::symmetrised_neighbours(nbr, row_ptr, col_idx, nb);
        std::vector<int> lev;
        const int nl = mg::gs_pass_levels_host(nbr, nb, reverse ? 1 : 0, nsw, lev);
        if (level) std::copy(lev.begin(), lev.end(), level);
        if (nlevels) *nlevels = nl;
    } catch (...) {
        return MGLDG_ERR_NOMEM;
    }
    return MGLDG_OK;
}

// Runs the Gauss-Seidel kernel on a two-row system in which row 1 waits for
// row 0 but row 0 is never scheduled (a pass whose only item is row 1), so
// the wait can only end by its time limit.  Reports the status the kernel
// left and checks that the stream is still usable afterwards.
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
        sched_build(ctx, A, S);
        GsPass P;
        const int item = (1 << 3) | 0;
        P.nsw = 1;
        P.dir = 0;
        P.nitems = 1;
        P.depth = 1;
        P.items = dalloc<int>(1);
        upload(ctx, P.items, &item, 1);
        S.passes.push_back(P);
        S.timeout_ns = timeout_ns;
        gs_sweeps<double>(ctx, A, A->val, dinv, b, x, S, 1.0, false, 1);
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

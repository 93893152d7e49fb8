// rowdot.cuh -- one warp computes (A x)_i for a block row i of a BSR matrix.
//
// Lane layout: S = 32 / br lanes per block row, each owning a contiguous
// chunk of CH columns.  For up to MAXB blocks at a time the warp first issues
// every load of the row -- the block values (128-bit loads where the row is
// 16-byte aligned; their addresses need no index), then the column indices
// (one lane each, broadcast by shuffle) and the x chunks -- and only then
// does the arithmetic, one fused multiply-add per product, so a warp keeps
// MAXB blocks in flight instead of one.
#pragma once

#include "internal.cuh"

namespace mg {

template <class T>
struct V16;
template <>
struct V16<double> { typedef double2 type; static constexpr int n = 2; };
template <>
struct V16<float> { typedef float4 type; static constexpr int n = 4; };

// acc += a . b as a chain of fused multiply-adds (one FMA per product)
__device__ __forceinline__ void vfma(double& acc, const double2& a, const double2& b) {
    acc = fma(a.x, b.x, acc);
    acc = fma(a.y, b.y, acc);
}
__device__ __forceinline__ void vfma(float& acc, const float4& a, const float4& b) {
    acc = fmaf(a.x, b.x, acc);
    acc = fmaf(a.y, b.y, acc);
    acc = fmaf(a.z, b.z, acc);
    acc = fmaf(a.w, b.w, acc);
}

// can this block shape use 128-bit loads for every lane chunk?
template <class T, int BR, int BC>
struct RowVec {
    using L = WL<BR, BC>;
    static constexpr bool ok = ((BC * sizeof(T)) % 16 == 0) && ((L::CH * sizeof(T)) % 16 == 0) &&
                               (L::CH * L::S == BC) && ((BR * BC * sizeof(T)) % 16 == 0);
    static constexpr int NV = ok ? (int)(L::CH * sizeof(T) / 16) : 1;
};

// Partial (A x)_i over this lane's chunk; reduce with seg_sum<S> afterwards.
// XL: load x through the read-only path (true) or through L2 (false, when x
// changes during the kernel).
template <class T, int BR, int BC, int MAXB, bool XL = true>
__device__ __forceinline__ T row_dot(const int* __restrict__ col_idx, const T* __restrict__ val,
                                     const int* __restrict__ blk, const T* x, int k0, int k1, int r, int c0,
                                     bool active, int lane) {
    using L = WL<BR, BC>;
    using RV = RowVec<T, BR, BC>;
    T acc = 0;
    for (int kb = k0; kb < k1; kb += MAXB) {
        const int nb = min(MAXB, k1 - kb);
        // block values first: their addresses need no loaded index (unless
        // the matrix stores a block table), so they go out immediately
        if constexpr (RV::ok) {
            typedef typename V16<T>::type V;
            V av[MAXB][RV::NV], xv[MAXB][RV::NV];
#pragma unroll
            for (int q = 0; q < MAXB; ++q)
                if (q < nb && active) {
                    const int bq = blk ? __ldg(blk + kb + q) : kb + q;
                    const V* ap = reinterpret_cast<const V*>(val + (size_t)bq * (BR * BC) + r * BC + c0);
#pragma unroll
                    for (int v = 0; v < RV::NV; ++v) av[q][v] = __ldg(ap + v);
                }
            const int jl = (lane < nb) ? __ldg(col_idx + kb + lane) : 0;
#pragma unroll
            for (int q = 0; q < MAXB; ++q) {
                const int j = __shfl_sync(0xffffffffu, jl, q);
                if (q < nb && active) {
                    const V* xp = reinterpret_cast<const V*>(x + (size_t)j * BC + c0);
#pragma unroll
                    for (int v = 0; v < RV::NV; ++v) xv[q][v] = XL ? __ldg(xp + v) : __ldcg(xp + v);
                }
            }
#pragma unroll
            for (int q = 0; q < MAXB; ++q)
                if (q < nb && active) {
#pragma unroll
                    for (int v = 0; v < RV::NV; ++v) vfma(acc, av[q][v], xv[q][v]);
                }
        } else {
            T av[MAXB][L::CH], xv[MAXB][L::CH];
#pragma unroll
            for (int q = 0; q < MAXB; ++q)
                if (q < nb && active) {
                    const int bq = blk ? __ldg(blk + kb + q) : kb + q;
                    const T* ap = val + (size_t)bq * (BR * BC) + r * BC + c0;
#pragma unroll
                    for (int c = 0; c < L::CH; ++c) av[q][c] = (c0 + c < BC) ? __ldg(ap + c) : T(0);
                }
            const int jl = (lane < nb) ? __ldg(col_idx + kb + lane) : 0;
#pragma unroll
            for (int q = 0; q < MAXB; ++q) {
                const int j = __shfl_sync(0xffffffffu, jl, q);
                if (q < nb && active) {
                    const T* xp = x + (size_t)j * BC + c0;
#pragma unroll
                    for (int c = 0; c < L::CH; ++c)
                        xv[q][c] = (c0 + c < BC) ? (XL ? __ldg(xp + c) : __ldcg(xp + c)) : T(0);
                }
            }
#pragma unroll
            for (int q = 0; q < MAXB; ++q)
                if (q < nb && active) {
#pragma unroll
                    for (int c = 0; c < L::CH; ++c) acc = fma(av[q][c], xv[q][c], acc);
                }
        }
    }
    return acc;
}

// One block at a time with 128-bit loads: the lean form for FP64, whose
// block products are bound by GB300's FP64 pipes rather than by HBM, so
// registers are better spent on occupancy than on loads in flight.
template <class T, int BR, int BC>
__device__ __forceinline__ T row_dot_lean(const int* __restrict__ col_idx, const T* __restrict__ val,
                                          const int* __restrict__ blk, const T* x, int k0, int k1, int r, int c0,
                                          bool active) {
    using L = WL<BR, BC>;
    using RV = RowVec<T, BR, BC>;
    T acc = 0;
#pragma unroll 2
    for (int k = k0; k < k1; ++k) {
        const int j = __ldg(col_idx + k);
        const T* a = val + (size_t)(blk ? __ldg(blk + k) : k) * (BR * BC) + r * BC + c0;
        const T* xj = x + (size_t)j * BC + c0;
        if (!active) continue;
        if constexpr (RV::ok) {
            typedef typename V16<T>::type V;
#pragma unroll
            for (int v = 0; v < RV::NV; ++v) vfma(acc, __ldg(reinterpret_cast<const V*>(a) + v), __ldg(reinterpret_cast<const V*>(xj) + v));
        } else {
#pragma unroll
            for (int c = 0; c < L::CH; ++c)
                if (c0 + c < BC) acc = fma(__ldg(a + c), __ldg(xj + c), acc);
        }
    }
    return acc;
}

// (A x)_i partial for this lane: prefetching form for FP32 (HBM-bound, five
// blocks -- a full 5-point block row -- in flight), lean form for FP64
template <class T, int BR, int BC>
__device__ __forceinline__ T row_product(const int* __restrict__ col_idx, const T* __restrict__ val,
                                         const int* __restrict__ blk, const T* x, int k0, int k1, int r, int c0,
                                         bool active, int lane) {
    if constexpr (sizeof(T) == 4) return row_dot<T, BR, BC, 5>(col_idx, val, blk, x, k0, k1, r, c0, active, lane);
    else return row_dot_lean<T, BR, BC>(col_idx, val, blk, x, k0, k1, r, c0, active);
}

// ---------------------------------------------------------- small blocks --
// Blocks of BR x BC with max(BR, BC) <= 32 (used for square 3..10): lane
// groups of S = max(BR, BC) lanes, 32 / S block rows per warp, lane (g, c) owning
// column c (< BC) of the warp's g-th block row.  For every block the lane
// reads column c of each block row r -- a[r][c], the group's lanes together
// one contiguous BC-value row per load -- and its single entry x_j[c], and
// keeps BR partial sums acc[r].  The warp's block rows are consecutive, so
// their blocks are one contiguous run of the value array.  rows_reduce then
// sums acc[r] over the group's lanes through shared memory, in column
// order, and leaves row r's total on lane (g, r) (r < BR).
template <int BR, int BC = BR>
struct Rows {
    static constexpr int S = BR > BC ? BR : BC;   // lanes per block row
    static constexpr int G = 32 / S;              // block rows per warp
    static constexpr int LD = BC + 1;             // padded shared-memory row
    static constexpr int SM = G * BR * LD;        // values per warp
};

// value readers: T from the stored type (FP64, FP32 or block-scaled FP16)
__device__ __forceinline__ double ld_val(const double* p) { return __ldg(p); }
__device__ __forceinline__ float ld_val(const float* p) { return __ldg(p); }
__device__ __forceinline__ float ld_val(const __half* p) { return __half2float(__ldg(p)); }

// scl: per-block scales of a block-scaled FP16 matrix (null otherwise); a
// block's scale is folded into the lane's x entry
template <class T, class VT, int BR, int BC, int MAXB>
__device__ __forceinline__ void cols_accumulate(const int* __restrict__ col_idx, const VT* __restrict__ val,
                                                const float* __restrict__ scl, const int* __restrict__ blk,
                                                const T* __restrict__ x, int k0, int k1, int c, T (&acc)[BR]) {
    for (int kb = k0; kb < k1; kb += MAXB) {
        const int nb = min(MAXB, k1 - kb);
        T a[MAXB][BR], xv[MAXB], sc[MAXB];
        int j[MAXB];
#pragma unroll
        for (int q = 0; q < MAXB; ++q) j[q] = (q < nb) ? __ldg(col_idx + kb + q) : 0;
#pragma unroll
        for (int q = 0; q < MAXB; ++q)
            if (q < nb) {
                const int bq = blk ? __ldg(blk + kb + q) : kb + q;
                const VT* ap = val + (size_t)bq * (BR * BC) + c;
#pragma unroll
                for (int r = 0; r < BR; ++r) a[q][r] = ld_val(ap + r * BC);
                sc[q] = scl ? (T)__ldg(scl + bq) : T(1);
            }
#pragma unroll
        for (int q = 0; q < MAXB; ++q) xv[q] = (q < nb) ? __ldg(x + (size_t)j[q] * BC + c) * sc[q] : T(0);
#pragma unroll
        for (int q = 0; q < MAXB; ++q)
            if (q < nb) {
#pragma unroll
                for (int r = 0; r < BR; ++r) acc[r] = fma(a[q][r], xv[q], acc[r]);
            }
    }
}

// Sum of acc[r] over the group's lanes c < BC, returned on lane (g, r) for
// r < BR (0 elsewhere); `s` is the warp's Rows<BR, BC>::SM values of shared
// memory.  All lanes must call it.
template <class T, int BR, int BC>
__device__ __forceinline__ T rows_reduce(const T (&acc)[BR], T* s, int g, int c, bool in_group) {
    using R = Rows<BR, BC>;
    if (in_group && c < BC) {
#pragma unroll
        for (int r = 0; r < BR; ++r) s[(g * BR + r) * R::LD + c] = acc[r];
    }
    __syncwarp();
    T y = 0;
    if (in_group && c < BR) {
#pragma unroll
        for (int cc = 0; cc < BC; ++cc) y += s[(g * BR + c) * R::LD + cc];
    }
    __syncwarp();
    return y;
}

}  // namespace mg

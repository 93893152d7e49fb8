// rowdot.cuh -- one warp computes (A x)_i for a block row i of a BSR matrix.
//
// Lane layout: S = 32 / br lanes per block row, each owning a contiguous
// chunk of CH columns.  For up to MAXB blocks at a time the warp first issues
// every load of the row -- the column indices (one lane each, broadcast by
// shuffle), the block values (128-bit loads where the row is 16-byte
// aligned) and the x chunks -- and only then does the arithmetic, so a warp
// keeps MAXB blocks in flight instead of one.
#pragma once

#include "internal.cuh"

namespace mg {

template <class T>
struct V16;
template <>
struct V16<double> { typedef double2 type; static constexpr int n = 2; };
template <>
struct V16<float> { typedef float4 type; static constexpr int n = 4; };

template <class T>
__device__ __forceinline__ T vdot(const typename V16<T>::type& a, const typename V16<T>::type& b);
template <>
__device__ __forceinline__ double vdot<double>(const double2& a, const double2& b) {
    return a.x * b.x + a.y * b.y;
}
template <>
__device__ __forceinline__ float vdot<float>(const float4& a, const float4& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w;
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
        const int jl = (lane < nb) ? __ldg(col_idx + kb + lane) : 0;
        const int bl = (lane < nb) ? (blk ? __ldg(blk + kb + lane) : kb + lane) : 0;
        if constexpr (RV::ok) {
            typedef typename V16<T>::type V;
            V av[MAXB][RV::NV], xv[MAXB][RV::NV];
#pragma unroll
            for (int q = 0; q < MAXB; ++q) {
                const int j = __shfl_sync(0xffffffffu, jl, q);
                const int bq = __shfl_sync(0xffffffffu, bl, q);
                if (q < nb && active) {
                    const V* ap = reinterpret_cast<const V*>(val + (size_t)bq * (BR * BC) + r * BC + c0);
                    const V* xp = reinterpret_cast<const V*>(x + (size_t)j * BC + c0);
#pragma unroll
                    for (int v = 0; v < RV::NV; ++v) {
                        av[q][v] = __ldg(ap + v);
                        xv[q][v] = XL ? __ldg(xp + v) : __ldcg(xp + v);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < MAXB; ++q)
                if (q < nb && active) {
#pragma unroll
                    for (int v = 0; v < RV::NV; ++v) acc += vdot<T>(av[q][v], xv[q][v]);
                }
        } else {
            T av[MAXB][L::CH], xv[MAXB][L::CH];
#pragma unroll
            for (int q = 0; q < MAXB; ++q) {
                const int j = __shfl_sync(0xffffffffu, jl, q);
                const int bq = __shfl_sync(0xffffffffu, bl, q);
                if (q < nb && active) {
                    const T* ap = val + (size_t)bq * (BR * BC) + r * BC + c0;
                    const T* xp = x + (size_t)j * BC + c0;
#pragma unroll
                    for (int c = 0; c < L::CH; ++c) {
                        const bool in = c0 + c < BC;
                        av[q][c] = in ? __ldg(ap + c) : T(0);
                        xv[q][c] = in ? (XL ? __ldg(xp + c) : __ldcg(xp + c)) : T(0);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < MAXB; ++q)
                if (q < nb && active) {
#pragma unroll
                    for (int c = 0; c < L::CH; ++c) acc += av[q][c] * xv[q][c];
                }
        }
    }
    return acc;
}

// blocks kept in flight per warp: more for FP32 (bandwidth-bound), fewer for
// FP64 (bound by the FP64 pipes, registers are better spent on occupancy)
template <class T>
struct RowDepth { static constexpr int value = sizeof(T) == 4 ? 6 : 3; };

}  // namespace mg

// internal.cuh -- shared host structures and device helpers of libmgldg.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <exception>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/mgldg.h"

namespace mg {

// ------------------------------------------------------------------ errors --
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define MG_CHECK_CUDA(call)                                                           \
    do {                                                                              \
        cudaError_t e_ = (call);                                                      \
        if (e_ != cudaSuccess)                                                        \
            throw ::mg::Error(e_ == cudaErrorMemoryAllocation ? MGLDG_ERR_NOMEM       \
                                                              : MGLDG_ERR_CUDA,       \
                              std::string(#call) + ": " + cudaGetErrorString(e_));    \
    } while (0)

#define MG_REQUIRE(cond, code, msg)                 \
    do {                                            \
        if (!(cond)) throw ::mg::Error(code, msg);  \
    } while (0)

// ------------------------------------------------------------ host threads --
// parallel_ranges(n, grain, f): f(begin, end) over [0, n) in chunks of
// `grain` on up to hardware_concurrency threads (the caller is one of them).
// Every index is visited exactly once, so loops whose iterations write
// disjoint outputs give the serial loop's result bit for bit.  The first
// exception thrown by f is rethrown on the caller after all threads joined.
template <class F>
void parallel_ranges(int64_t n, int64_t grain, F&& f) {
    if (n <= 0) return;
    grain = std::max<int64_t>(1, grain);
    const int64_t chunks = (n + grain - 1) / grain;
    const int nth = (int)std::min<int64_t>(chunks, std::max(1u, std::min(std::thread::hardware_concurrency(), 64u)));
    if (nth <= 1) {
        f((int64_t)0, n);
        return;
    }
    std::atomic<int64_t> next{0};
    std::exception_ptr err;
    std::mutex m;
    auto work = [&]() {
        try {
            for (;;) {
                const int64_t s = next.fetch_add(grain);
                if (s >= n) break;
                f(s, std::min(n, s + grain));
            }
        } catch (...) {
            std::lock_guard<std::mutex> g(m);
            if (!err) err = std::current_exception();
            next.store(n);
        }
    };
    std::vector<std::thread> th;
    th.reserve(nth - 1);
    for (int t = 1; t < nth; ++t) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
    if (err) std::rethrow_exception(err);
}
template <class F>
void parallel_for(int64_t n, int64_t grain, F&& f) {
    parallel_ranges(n, grain, [&](int64_t s, int64_t e) {
        for (int64_t i = s; i < e; ++i) f(i);
    });
}

// --------------------------------------------------------------- profiling --
struct ProfEvent {
    cudaEvent_t a, b;
    int kclass;
    int level;
};
constexpr int kProfLevels = 33;   // multigrid level + 1 (slot 0: work outside a level)

}  // namespace mg

struct mgldg_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    bool prof = false;
    int64_t launches[MGLDG_K_NCLASS] = {0};
    double ms[MGLDG_K_NCLASS] = {0};
    int cur_level = -1;   // multigrid level the next launches work on (-1: none)
    int64_t lv_launches[MGLDG_K_NCLASS][mg::kProfLevels] = {};
    double lv_ms[MGLDG_K_NCLASS][mg::kProfLevels] = {};
    std::vector<mg::ProfEvent> pending;
    std::vector<cudaEvent_t> event_pool;
    // scratch for deterministic two-stage reductions
    double* d_partials = nullptr;
    int n_partials = 0;
    // device error word of the bulk-copy kernels (bounded barrier waits)
    unsigned* d_err = nullptr;
};

namespace mg {

// RAII timer around one kernel launch: counts it and, when profiling is on,
// brackets it with CUDA events on the context's stream.
struct Launch {
    mgldg_ctx* ctx;
    int kc;
    int lv;
    cudaEvent_t a = nullptr, b = nullptr;
    Launch(mgldg_ctx* c, int kclass);
    ~Launch();
};
void prof_flush(mgldg_ctx* ctx);

// ------------------------------------------------------------ device memory --
template <class T>
T* dalloc(size_t n) {
    if (n == 0) return nullptr;
    void* p = nullptr;
    MG_CHECK_CUDA(cudaMalloc(&p, n * sizeof(T)));
    return (T*)p;
}
template <class T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}
template <class T>
void upload(mgldg_ctx* ctx, T* d, const T* h, size_t n) {
    if (n) MG_CHECK_CUDA(cudaMemcpyAsync(d, h, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
}
template <class T>
void download(mgldg_ctx* ctx, T* h, const T* d, size_t n) {
    if (n) MG_CHECK_CUDA(cudaMemcpyAsync(h, d, n * sizeof(T), cudaMemcpyDeviceToHost, ctx->stream));
}
inline void sync(mgldg_ctx* ctx) { MG_CHECK_CUDA(cudaStreamSynchronize(ctx->stream)); }
inline void check_launch() { MG_CHECK_CUDA(cudaGetLastError()); }

}  // namespace mg

// ------------------------------------------------------------- BSR matrix --
// Block-CSR with sorted columns.  Values are either one block per stored
// entry (blk == null) or a table of distinct blocks indexed through blk
// (used for interpolation operators, whose blocks repeat on quadtrees).
struct mgldg_bsr {
    mgldg_ctx* ctx = nullptr;
    int nbr = 0, nbc = 0, br = 0, bc = 0;
    int64_t nnzb = 0;
    std::vector<int> h_row_ptr, h_col_idx;   // host copy of the pattern
    int* row_ptr = nullptr;
    int* col_idx = nullptr;
    double* val = nullptr;       // FP64 values (nnzb or nuniq blocks)
    float* val32 = nullptr;      // FP32 copy, built on demand (mixed precision)
    // block-scaled FP16 copy (MGLDG_PREC_MIXED_F16): block k's entries are
    // scale16[k] * val16[k * bsz() + e], scale16[k] the block's largest
    // magnitude, so every stored half lies in [-1, 1]; scale16 has four
    // spare entries (bulk copies move whole 16-byte words)
    __half* val16 = nullptr;
    float* scale16 = nullptr;
    // low half of a two-float split of the FP64 values: val = val32 + lo32
    // to about 2^-48 (mixed forms' double-float outer products)
    float* lo32 = nullptr;
    int* blk = nullptr;          // optional block indirection
    std::vector<int> h_blk;
    int64_t nuniq = 0;
    int* diag = nullptr;         // per row: position of the diagonal block or -1
    std::vector<int> h_diag;
    ~mgldg_bsr();
    int64_t nvals_blocks() const { return blk ? nuniq : nnzb; }
    size_t bsz() const { return (size_t)br * bc; }
};

struct mgldg_ops {
    mgldg_ctx* ctx = nullptr;
    int ndim = 0;
    mgldg_bsr* M = nullptr;
    mgldg_bsr* G[3] = {nullptr, nullptr, nullptr};
    mgldg_bsr* T = nullptr;
    mgldg_bsr* A = nullptr;
    ~mgldg_ops();
    bool has_MGT() const { return M && T && G[0]; }
};

namespace mg {

// bsr.cu
mgldg_bsr* bsr_new(mgldg_ctx* ctx, int nbr, int nbc, int br, int bc,
                   const std::vector<int>& row_ptr, const std::vector<int>& col_idx);
void bsr_build_diag(mgldg_bsr* A);
void bsr_ensure_fp32(mgldg_bsr* A);
void bsr_ensure_f16(mgldg_bsr* A);
void bsr_ensure_lo32(mgldg_bsr* A);
// V-cycle products on the block-scaled FP16 copy (FP32 vectors and
// arithmetic); false when the matrix has no such copy or the shape has no kernel
bool spmv_f16(mgldg_ctx* ctx, const mgldg_bsr* A, float alpha, const float* x, float beta, const float* yin, float* y,
              int kclass);
bool jacobi_f16(mgldg_ctx* ctx, const mgldg_bsr* A, const float* Dinv, const float* b, const float* xin, float* xout,
                float omega, bool xzero = false);
// block sizes read from the FP16 copy: 16x16 only.  The small-block kernels
// (3..10) are bound by load latency rather than bytes, and an FP16 copy made
// them slower (392k-triangle disk solve 53 -> 72 ms), so those levels keep
// FP32 in the F16 form.
inline bool f16_shape(int br, int bc) { return br == 16 && bc == 16; }
template <class T>
const T* bsr_vals(const mgldg_bsr* A);
// y = alpha*A*x + beta*yin (yin may alias y or be null when beta == 0);
// if dotv != null the partial sums of y.dotv are written to partials[].
template <class T>
void spmv(mgldg_ctx* ctx, const mgldg_bsr* A, T alpha, const T* x, T beta, const T* yin, T* y,
          const T* dotv = nullptr, double* partials = nullptr, int* npart = nullptr,
          int kclass = MGLDG_K_SPMV);
// transpose of pattern and values (host pattern, device values)
mgldg_bsr* bsr_transpose(mgldg_ctx* ctx, const mgldg_bsr* A);
// collapse repeated blocks into a table (bitwise equal blocks)
void bsr_dedupe(mgldg_ctx* ctx, mgldg_bsr* A);
mgldg_bsr* bsr_clone(mgldg_ctx* ctx, const mgldg_bsr* A);

// deterministic dot products: partial sums then a fixed-order finish
int reduce_grid(int n);
template <class T>
void dot_partials(mgldg_ctx* ctx, int n, const T* a, const T* b, double* partials, int* npart);
void finish_sum(mgldg_ctx* ctx, const double* partials, int npart, double* out);

// setup.cu
void construct_laplacian(mgldg_ctx* ctx, mgldg_ops* ops);
// T + sum_d G_d^T M G_d for a block-diagonal M (new matrix)
mgldg_bsr* laplacian_of(mgldg_ctx* ctx, mgldg_bsr* M, mgldg_bsr* const* G, int ndim, mgldg_bsr* T);
void block_inverse(mgldg_ctx* ctx, const mgldg_bsr* A, double* out, int* status);
mgldg_ops* galerkin_ratrat(mgldg_ctx* ctx, const mgldg_ops* f, const mgldg_bsr* T);
// symbolic-plan and numeric-product milliseconds of the Galerkin products since the
// last call (setup tracing)
void setup_clock_take(double* plan_ms, double* prod_ms);
mgldg_ops* galerkin_rat(mgldg_ctx* ctx, const mgldg_ops* f, const mgldg_bsr* T);
// dense inverse of an SPD matrix assembled from A (Cholesky), device result
void dense_spd_inverse(mgldg_ctx* ctx, const mgldg_bsr* A, double* out_inv);

// bulk.cu: FP32 block-row kernels that stream values through shared memory
// with bulk copies; return false when the shape is not handled
bool bulk_spmv_f32(mgldg_ctx* ctx, const mgldg_bsr* A, float alpha, const float* x, float beta, const float* yin,
                   float* y, int kclass);
bool bulk_jacobi_f32(mgldg_ctx* ctx, const mgldg_bsr* A, const float* vals, const float* Dinv, const float* b,
                     const float* xin, float* xout, float omega, bool xzero = false);
bool bulk_spmv_f16(mgldg_ctx* ctx, const mgldg_bsr* A, float alpha, const float* x, float beta, const float* yin,
                   float* y, int kclass);
bool bulk_jacobi_f16(mgldg_ctx* ctx, const mgldg_bsr* A, const float* Dinv, const float* b, const float* xin,
                     float* xout, float omega, bool xzero = false);
// reads and clears the device error word; throws MGLDG_ERR_TIMEOUT if set
void take_device_error(mgldg_ctx* ctx);

}  // namespace mg

// ---------------------------------------------------------- device helpers --
namespace mg {

// Warp layout for one br x bc block: S lanes per block row, each lane owns a
// contiguous chunk of CH columns.
template <int BR, int BC>
struct WL {
    static_assert(BR >= 1 && BR <= 32, "block rows must fit a warp");
    static constexpr int S = 32 / BR;
    static constexpr int CH = (BC + S - 1) / S;
};

template <int S, class T>
__device__ __forceinline__ T seg_sum(T v) {
    // sum over the S consecutive lanes of a row segment; valid in the
    // segment's first lane (and in all lanes when S is a power of two)
    if constexpr ((S & (S - 1)) == 0) {
#pragma unroll
        for (int o = S / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        return v;
    } else {
        T t = v;
#pragma unroll
        for (int k = 1; k < S; ++k) t += __shfl_down_sync(0xffffffffu, v, k);
        return t;
    }
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

}  // namespace mg

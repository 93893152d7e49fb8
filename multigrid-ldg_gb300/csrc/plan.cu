// plan.cu -- symbolic pass of the Galerkin block SpGEMM on the GPU.
//
// The products of the reference's coarse-level constructor
// (src/cartesian/multigrid/multigrid.h:115-157) and of construct_laplacian
// (src/cartesian/dg/ldgpoisson.h:34-52) sum, into every output block, the
// terms the loops of multiply_mm / multiply_mm_t
// (src/cartesian/util/sparseblockmatrix.tpp:234-280) meet in this order:
//   X * Y     : row i of X, its blocks a in column order, Y's row col(a)
//   X^T * Y   : row k of X, its blocks a, Y's row k       (output row col(a))
//   X^T D X   : row k of X, blocks a, b of that row         (output col(a), col(b))
// In each case an output block receives at most one term per step of the
// outer loop, so its terms are ordered by that step.  The symbolic pass
// writes every candidate term as (output key, term) in exactly this loop
// order -- one thread per operand row, rows at offsets from a scan of their
// counts -- and a stable radix sort by key then groups the terms of each
// output block without reordering them.  The numeric kernel therefore adds
// the terms of each block in the reference's order.
//
// Scratch arrays come from the stream-ordered allocator, so a plan costs no
// device synchronisation beyond the one read of its output size.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include "plan.cuh"

namespace mg {

namespace {

template <class T>
T* salloc(mgldg_ctx* ctx, size_t n) {
    void* p = nullptr;
    MG_CHECK_CUDA(cudaMallocAsync(&p, std::max<size_t>(1, n) * sizeof(T), ctx->stream));
    return (T*)p;
}
template <class T>
void sfree(mgldg_ctx* ctx, T*& p) {
    if (p) cudaFreeAsync((void*)p, ctx->stream);
    p = nullptr;
}

// scratch pointers released together on scope exit
struct Scratch {
    mgldg_ctx* ctx;
    std::vector<void*> ps;
    explicit Scratch(mgldg_ctx* c) : ctx(c) {}
    template <class T>
    T* get(size_t n) {
        T* p = salloc<T>(ctx, n);
        ps.push_back((void*)p);
        return p;
    }
    ~Scratch() {
        for (void* p : ps) cudaFreeAsync(p, ctx->stream);
    }
};

int grid_for(mgldg_ctx* ctx, int64_t n, int per_block = 256) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + per_block - 1) / per_block, (int64_t)ctx->sm_count * 16));
}

int key_bits(uint64_t maxkey) {
    int b = 1;
    while (b < 64 && (maxkey >> b) != 0) ++b;
    return b;
}

template <class T>
void exclusive_scan(mgldg_ctx* ctx, Scratch& S, const T* in, T* out, int64_t n) {
    size_t tb = 0;
    MG_CHECK_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, in, out, n, ctx->stream));
    void* tmp = S.get<char>(tb);
    MG_CHECK_CUDA(cub::DeviceScan::ExclusiveSum(tmp, tb, in, out, n, ctx->stream));
}

struct Pat {
    const int* rp;
    const int* ci;
    int nbr;
};
Pat pat(const mgldg_bsr* A) { return Pat{A->row_ptr, A->col_idx, A->nbr}; }

enum { GEN_MM = 0, GEN_MMT = 1, GEN_TRIPLE = 2 };

// candidate terms of every row of X (the outer loop of the product)
__global__ void k_gen_count(int mode, Pat X, Pat Y, int64_t* cnt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < X.nbr; i += gridDim.x * blockDim.x) {
        int64_t c = 0;
        for (int a = X.rp[i]; a < X.rp[i + 1]; ++a) {
            const int k = (mode == GEN_MM) ? X.ci[a] : i;
            c += Y.rp[k + 1] - Y.rp[k];
        }
        cnt[i] = c;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cnt[X.nbr] = 0;
}

// every candidate as (output key, generation index, term) in loop order;
// bad |= 1 where the triple product's middle factor lacks a diagonal block
__global__ void k_gen_fill(int mode, Pat X, Pat Y, const int* __restrict__ diag, uint64_t nbc_out,
                           const int64_t* __restrict__ off, uint64_t* __restrict__ keys, int* __restrict__ idx,
                           int3* __restrict__ terms, int* bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < X.nbr; i += gridDim.x * blockDim.x) {
        int64_t t = off[i];
        int m = -1;
        if (mode == GEN_TRIPLE) {
            m = diag[i];
            if (m < 0) {
                atomicOr(bad, 1);
                m = 0;
            }
        }
        for (int a = X.rp[i]; a < X.rp[i + 1]; ++a) {
            const int k = (mode == GEN_MM) ? X.ci[a] : i;
            const uint64_t orow = (mode == GEN_MM) ? (uint64_t)i : (uint64_t)X.ci[a];
            for (int b = Y.rp[k]; b < Y.rp[k + 1]; ++b, ++t) {
                keys[t] = orow * nbc_out + (uint64_t)Y.ci[b];
                idx[t] = (int)t;
                terms[t] = make_int3(a, m, b);
            }
        }
    }
}

// sorted candidates: terms in sorted order, and a 1 at the first candidate
// of every output block (head[n] = 0 so the scan also yields the count)
__global__ void k_plan_heads(int64_t n, const uint64_t* __restrict__ keys, const int* __restrict__ idx,
                             const int3* __restrict__ tin, int3* __restrict__ tout, int* __restrict__ head) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= n; t += (int64_t)gridDim.x * blockDim.x) {
        if (t == n) {
            head[t] = 0;
            continue;
        }
        if (tout) tout[t] = tin[idx[t]];
        head[t] = (t == 0 || keys[t] != keys[t - 1]) ? 1 : 0;
    }
}

// output block q = pos[t] at every head t: its key, column and first term
__global__ void k_plan_keys(int64_t n, const uint64_t* __restrict__ keys, const int* __restrict__ head,
                            const int* __restrict__ pos, uint64_t nbc, uint64_t* __restrict__ ukeys,
                            int* __restrict__ col_idx, int* __restrict__ tptr) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t <= n; t += (int64_t)gridDim.x * blockDim.x) {
        if (t == n) {
            if (tptr) tptr[pos[n]] = (int)n;
            continue;
        }
        if (!head[t]) continue;
        const int q = pos[t];
        ukeys[q] = keys[t];
        col_idx[q] = (int)(keys[t] % nbc);
        if (tptr) tptr[q] = (int)t;
    }
}

// row_ptr from the sorted output keys: rows (row(q-1), row(q)] start at q
__global__ void k_plan_rows(int nkeys, const uint64_t* __restrict__ ukeys, uint64_t nbc, int nbr, int* row_ptr) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q <= nkeys; q += gridDim.x * blockDim.x) {
        const int64_t r = (q < nkeys) ? (int64_t)(ukeys[q] / nbc) : nbr;
        const int64_t rp = (q > 0) ? (int64_t)(ukeys[q - 1] / nbc) : -1;
        for (int64_t rr = rp + 1; rr <= r; ++rr) row_ptr[rr] = q;
    }
}

__device__ __forceinline__ int lower_bound_key(const uint64_t* a, int n, uint64_t v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// keys of a BSR pattern
__global__ void k_pattern_keys(Pat X, uint64_t nbc_out, uint64_t* __restrict__ keys) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < X.nbr; i += gridDim.x * blockDim.x)
        for (int a = X.rp[i]; a < X.rp[i + 1]; ++a) keys[a] = (uint64_t)i * nbc_out + (uint64_t)X.ci[a];
}

// term counts of one product's output blocks at their positions in the union
__global__ void k_plan_expand(int nk, const uint64_t* __restrict__ ukeys, const int* __restrict__ tptr, int nU,
                              const uint64_t* __restrict__ ukeysU, int* __restrict__ cntU) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nk; q += gridDim.x * blockDim.x)
        cntU[lower_bound_key(ukeysU, nU, ukeys[q])] = tptr[q + 1] - tptr[q];
}

__global__ void k_rowscale_plan(Pat g, int* __restrict__ tptr, int3* __restrict__ terms) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < g.nbr; i += gridDim.x * blockDim.x) {
        for (int a = g.rp[i]; a < g.rp[i + 1]; ++a) {
            tptr[a] = a;
            terms[a] = make_int3(i, -1, a);
        }
        if (i == g.nbr - 1) tptr[g.rp[g.nbr]] = g.rp[g.nbr];
    }
}

__global__ void k_scatter_index(Pat U, Pat T, int* __restrict__ src, int* bad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < T.nbr; i += gridDim.x * blockDim.x) {
        int q = U.rp[i];
        const int qe = U.rp[i + 1];
        for (int a = T.rp[i]; a < T.rp[i + 1]; ++a) {
            while (q < qe && U.ci[q] != T.ci[a]) ++q;
            if (q == qe) {
                atomicOr(bad, 1);
                break;
            }
            src[q] = a;
        }
    }
}

// Sorts the candidates by key (stably: equal keys keep their generation
// order) and fills P's pattern, keys and -- when `terms` is given -- its term
// ranges and sorted terms.  Reads the output size back (one stream
// synchronisation).
void finish(mgldg_ctx* ctx, Scratch& S, const uint64_t* keys, const int* idx, const int3* terms, int64_t n,
            DPlan* P) {
    MG_REQUIRE(n < (int64_t)INT32_MAX, MGLDG_ERR_UNSUPPORTED, "product plan exceeds 2^31 terms");
    const uint64_t nbc = (uint64_t)std::max(1, P->nbc);
    const int bits = key_bits((uint64_t)std::max(1, P->nbr) * nbc);
    uint64_t* skeys = S.get<uint64_t>(n);
    int* sidx = terms ? S.get<int>(n) : nullptr;
    if (n > 0) {
        size_t tb = 0;
        if (terms) {
            MG_CHECK_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, keys, skeys, idx, sidx, n, 0, bits, ctx->stream));
            void* tmp = S.get<char>(tb);
            MG_CHECK_CUDA(cub::DeviceRadixSort::SortPairs(tmp, tb, keys, skeys, idx, sidx, n, 0, bits, ctx->stream));
        } else {
            MG_CHECK_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tb, keys, skeys, n, 0, bits, ctx->stream));
            void* tmp = S.get<char>(tb);
            MG_CHECK_CUDA(cub::DeviceRadixSort::SortKeys(tmp, tb, keys, skeys, n, 0, bits, ctx->stream));
        }
    }
    P->nterms = terms ? n : 0;
    if (terms) P->terms = salloc<int3>(ctx, n);
    int* head = S.get<int>(n + 1);
    int* pos = S.get<int>(n + 1);
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_plan_heads<<<grid_for(ctx, n + 1), 256, 0, ctx->stream>>>(n, skeys, sidx, terms, P->terms, head);
    }
    check_launch();
    exclusive_scan(ctx, S, head, pos, n + 1);
    int nk = 0;
    download(ctx, &nk, pos + n, 1);
    sync(ctx);
    P->nkeys = nk;
    P->keys = salloc<uint64_t>(ctx, nk);
    P->col_idx = salloc<int>(ctx, nk);
    P->row_ptr = salloc<int>(ctx, (size_t)P->nbr + 1);
    if (terms) P->tptr = salloc<int>(ctx, (size_t)nk + 1);
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_plan_keys<<<grid_for(ctx, n + 1), 256, 0, ctx->stream>>>(n, skeys, head, pos, nbc, P->keys, P->col_idx,
                                                                   P->tptr);
    }
    check_launch();
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_plan_rows<<<grid_for(ctx, (int64_t)nk + 1), 256, 0, ctx->stream>>>(nk, P->keys, nbc, P->nbr, P->row_ptr);
    }
    check_launch();
}

// candidates of one product (mode GEN_*), sorted into P
void generate(mgldg_ctx* ctx, int mode, const mgldg_bsr* X, const mgldg_bsr* Y, const int* diag, DPlan* P) {
    Scratch S(ctx);
    int64_t* cnt = S.get<int64_t>((size_t)X->nbr + 1);
    int64_t* off = S.get<int64_t>((size_t)X->nbr + 1);
    const int g = grid_for(ctx, X->nbr, 128);
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_gen_count<<<g, 128, 0, ctx->stream>>>(mode, pat(X), pat(Y), cnt);
    }
    check_launch();
    exclusive_scan(ctx, S, cnt, off, (int64_t)X->nbr + 1);
    int64_t n = 0;
    download(ctx, &n, off + X->nbr, 1);
    sync(ctx);
    MG_REQUIRE(n < (int64_t)INT32_MAX, MGLDG_ERR_UNSUPPORTED, "product plan exceeds 2^31 terms");
    uint64_t* keys = S.get<uint64_t>(n);
    int* idx = S.get<int>(n);
    int3* terms = S.get<int3>(n);
    int* bad = S.get<int>(1);
    MG_CHECK_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_gen_fill<<<g, 128, 0, ctx->stream>>>(mode, pat(X), pat(Y), diag, (uint64_t)std::max(1, P->nbc), off, keys,
                                               idx, terms, bad);
    }
    check_launch();
    finish(ctx, S, keys, idx, terms, n, P);
    if (mode == GEN_TRIPLE) {
        int hb = 0;
        download(ctx, &hb, bad, 1);
        sync(ctx);
        MG_REQUIRE(hb == 0, MGLDG_ERR_SHAPE, "mass matrix lacks a diagonal block");
    }
}

}  // namespace

DPlan& DPlan::operator=(DPlan&& o) noexcept {
    if (this != &o) {
        release();
        ctx = o.ctx; nbr = o.nbr; nbc = o.nbc; nkeys = o.nkeys; nterms = o.nterms;
        row_ptr = o.row_ptr; col_idx = o.col_idx; tptr = o.tptr; terms = o.terms; keys = o.keys;
        o.row_ptr = o.col_idx = o.tptr = nullptr;
        o.terms = nullptr;
        o.keys = nullptr;
    }
    return *this;
}

void DPlan::release() {
    if (!ctx) return;
    sfree(ctx, row_ptr);
    sfree(ctx, col_idx);
    sfree(ctx, tptr);
    sfree(ctx, terms);
    sfree(ctx, keys);
}

void dplan_mm(mgldg_ctx* ctx, const mgldg_bsr* X, bool tX, const mgldg_bsr* Y, DPlan* P) {
    P->release();
    P->ctx = ctx;
    if (!tX) {
        MG_REQUIRE(X->nbc == Y->nbr && X->bc == Y->br, MGLDG_ERR_SHAPE, "multiply_mm: shapes do not conform");
        P->nbr = X->nbr;
    } else {
        MG_REQUIRE(X->nbr == Y->nbr && X->br == Y->br, MGLDG_ERR_SHAPE, "multiply_mm_t: shapes do not conform");
        P->nbr = X->nbc;
    }
    P->nbc = Y->nbc;
    generate(ctx, tX ? GEN_MMT : GEN_MM, X, Y, nullptr, P);
}

void dplan_triple(mgldg_ctx* ctx, const std::vector<const mgldg_bsr*>& Xs, const mgldg_bsr* D,
                  const mgldg_bsr* extra, std::vector<DPlan>* per, DPlan* U) {
    const int nout = Xs[0]->nbc;
    per->clear();
    for (const mgldg_bsr* X : Xs) {
        MG_REQUIRE(X->nbr == D->nbr && X->br == D->bc && X->nbc == nout, MGLDG_ERR_SHAPE,
                   "triple product: shapes do not conform");
        MG_REQUIRE(D->diag != nullptr, MGLDG_ERR_SHAPE, "mass matrix lacks a diagonal block");
        per->emplace_back();
        DPlan& P = per->back();
        P.ctx = ctx;
        P.nbr = P.nbc = nout;
        generate(ctx, GEN_TRIPLE, X, X, D->diag, &P);
    }
    if (extra)
        MG_REQUIRE(extra->nbr == nout && extra->nbc == nout, MGLDG_ERR_SHAPE, "triple product: extra pattern shape");
    // the union pattern: every product's blocks and `extra`'s
    U->release();
    U->ctx = ctx;
    U->nbr = U->nbc = nout;
    Scratch S(ctx);
    int64_t n = extra ? extra->nnzb : 0;
    for (const DPlan& P : *per) n += P.nkeys;
    uint64_t* keys = S.get<uint64_t>(n);
    int64_t o = 0;
    for (const DPlan& P : *per) {
        if (P.nkeys)
            MG_CHECK_CUDA(cudaMemcpyAsync(keys + o, P.keys, (size_t)P.nkeys * sizeof(uint64_t),
                                          cudaMemcpyDeviceToDevice, ctx->stream));
        o += P.nkeys;
    }
    if (extra && extra->nbr > 0) {
        Launch L(ctx, MGLDG_K_SETUP);
        k_pattern_keys<<<grid_for(ctx, extra->nbr), 256, 0, ctx->stream>>>(pat(extra), (uint64_t)std::max(1, nout),
                                                                           keys + o);
    }
    check_launch();
    finish(ctx, S, keys, nullptr, nullptr, n, U);
    // each product's term ranges re-indexed onto the union
    for (DPlan& P : *per) {
        int* cnt = S.get<int>((size_t)U->nkeys + 1);
        int* tptr = salloc<int>(ctx, (size_t)U->nkeys + 1);
        MG_CHECK_CUDA(cudaMemsetAsync(cnt, 0, ((size_t)U->nkeys + 1) * sizeof(int), ctx->stream));
        if (P.nkeys > 0) {
            Launch L(ctx, MGLDG_K_SETUP);
            k_plan_expand<<<grid_for(ctx, P.nkeys), 256, 0, ctx->stream>>>(P.nkeys, P.keys, P.tptr, U->nkeys, U->keys,
                                                                         cnt);
        }
        check_launch();
        exclusive_scan(ctx, S, cnt, tptr, (int64_t)U->nkeys + 1);
        sfree(ctx, P.tptr);
        sfree(ctx, P.row_ptr);
        sfree(ctx, P.col_idx);
        sfree(ctx, P.keys);
        P.tptr = tptr;
        P.nkeys = U->nkeys;
    }
}

void dplan_rowscale(mgldg_ctx* ctx, const mgldg_bsr* g, DPlan* P) {
    P->release();
    P->ctx = ctx;
    P->nbr = g->nbr;
    P->nbc = g->nbc;
    P->nkeys = (int)g->nnzb;
    P->nterms = g->nnzb;
    P->tptr = salloc<int>(ctx, (size_t)g->nnzb + 1);
    P->terms = salloc<int3>(ctx, (size_t)g->nnzb);
    if (g->nbr > 0) {
        Launch L(ctx, MGLDG_K_SETUP);
        k_rowscale_plan<<<grid_for(ctx, g->nbr), 256, 0, ctx->stream>>>(pat(g), P->tptr, P->terms);
    } else {
        MG_CHECK_CUDA(cudaMemsetAsync(P->tptr, 0, sizeof(int), ctx->stream));
    }
    check_launch();
}

void dplan_scatter_index(mgldg_ctx* ctx, const DPlan& U, const mgldg_bsr* T, int* src) {
    MG_REQUIRE(T->nbr <= U.nbr, MGLDG_ERR_SHAPE, "scatter: pattern rows do not conform");
    Scratch S(ctx);
    int* bad = S.get<int>(1);
    MG_CHECK_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
    MG_CHECK_CUDA(cudaMemsetAsync(src, 0xff, (size_t)std::max(1, U.nkeys) * sizeof(int), ctx->stream));
    if (T->nbr > 0) {
        Launch L(ctx, MGLDG_K_SETUP);
        k_scatter_index<<<grid_for(ctx, T->nbr), 256, 0, ctx->stream>>>(Pat{U.row_ptr, U.col_idx, U.nbr}, pat(T), src,
                                                                      bad);
    }
    check_launch();
    int hb = 0;
    download(ctx, &hb, bad, 1);
    sync(ctx);
    MG_REQUIRE(hb == 0, MGLDG_ERR_SHAPE, "product pattern is not contained in the union");
}

mgldg_bsr* bsr_from_dplan(mgldg_ctx* ctx, const DPlan& P, int br, int bc) {
    std::vector<int> rp((size_t)P.nbr + 1), ci((size_t)P.nkeys);
    download(ctx, rp.data(), P.row_ptr, rp.size());
    download(ctx, ci.data(), P.col_idx, ci.size());
    sync(ctx);
    return bsr_new(ctx, P.nbr, P.nbc, br, bc, rp, ci);
}

}  // namespace mg

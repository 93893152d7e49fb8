// builder.cu -- host-side block-by-block assembly with the reference's
// SparseBlockMatrix calls (reset / setBlock / addToBlock / blockExists,
// src/cartesian/util/sparseblockmatrix.tpp:79-127), then one sorted
// block-CSR upload.  Blocks live in insertion order in one array with a hash
// index by (i, j); addToBlock sums into the stored block in call order, as
// the reference's `blockMap_[Index(i,j)] += block` does, so every block holds
// the reference's sum bit for bit.
#include <unordered_map>

#include "api.cuh"

struct mgldg_bsr_builder {
    int nbr = 0, nbc = 0, br = 0, bc = 0;
    std::unordered_map<int64_t, int64_t> where;   // i * nbc + j -> block index
    std::vector<int> bi, bj;
    std::vector<double> vals;                     // blocks in insertion order
    size_t bs() const { return (size_t)br * bc; }
    int64_t key(int i, int j) const { return (int64_t)i * nbc + j; }
};

namespace {
int put(mgldg_bsr_builder* b, int i, int j, const double* block, bool add) {
    if (!b || !block || i < 0 || i >= b->nbr || j < 0 || j >= b->nbc) return MGLDG_ERR_ARG;
    try {
        const size_t bs = b->bs();
        auto it = b->where.find(b->key(i, j));
        if (it == b->where.end()) {
            // grow every array before indexing the new block, so a failed
            // allocation leaves the builder as it was
            const size_t nb = b->bi.size();
            b->vals.reserve(b->vals.size() + bs);
            b->bi.reserve(nb + 1);
            b->bj.reserve(nb + 1);
            b->where.emplace(b->key(i, j), (int64_t)nb);
            b->vals.insert(b->vals.end(), block, block + bs);
            b->bi.push_back(i);
            b->bj.push_back(j);
            return MGLDG_OK;
        }
        double* dst = b->vals.data() + (size_t)it->second * bs;
        if (add)
            for (size_t e = 0; e < bs; ++e) dst[e] += block[e];
        else
            std::copy(block, block + bs, dst);
    } catch (const std::bad_alloc&) {
        return MGLDG_ERR_NOMEM;
    }
    return MGLDG_OK;
}

// block indices sorted by (row, column)
std::vector<int64_t> sorted_order(const mgldg_bsr_builder* b) {
    std::vector<int64_t> order(b->bi.size());
    for (size_t q = 0; q < order.size(); ++q) order[q] = (int64_t)q;
    std::sort(order.begin(), order.end(), [b](int64_t x, int64_t y) {
        return b->bi[x] != b->bi[y] ? b->bi[x] < b->bi[y] : b->bj[x] < b->bj[y];
    });
    return order;
}

void export_csr(const mgldg_bsr_builder* b, int* row_ptr, int* col_idx, double* vals) {
    const std::vector<int64_t> order = sorted_order(b);
    const size_t bs = b->bs();
    if (row_ptr) {
        std::fill(row_ptr, row_ptr + b->nbr + 1, 0);
        for (int i : b->bi) row_ptr[i + 1]++;
        for (int i = 0; i < b->nbr; ++i) row_ptr[i + 1] += row_ptr[i];
    }
    for (size_t q = 0; q < order.size(); ++q) {
        if (col_idx) col_idx[q] = b->bj[order[q]];
        if (vals) std::copy(b->vals.begin() + order[q] * bs, b->vals.begin() + (order[q] + 1) * bs, vals + q * bs);
    }
}
}  // namespace

extern "C" int mgldg_bsr_builder_create(int nbr, int nbc, int br, int bc, mgldg_bsr_builder** out) {
    if (!out || nbr < 0 || nbc < 0 || br < 1 || bc < 1) return MGLDG_ERR_ARG;
    *out = nullptr;
    try {
        mgldg_bsr_builder* b = new mgldg_bsr_builder();
        b->nbr = nbr;
        b->nbc = nbc;
        b->br = br;
        b->bc = bc;
        *out = b;
    } catch (const std::bad_alloc&) {
        return MGLDG_ERR_NOMEM;
    }
    return MGLDG_OK;
}

extern "C" int mgldg_bsr_builder_set(mgldg_bsr_builder* b, int i, int j, const double* block) {
    return put(b, i, j, block, false);
}

extern "C" int mgldg_bsr_builder_add(mgldg_bsr_builder* b, int i, int j, const double* block) {
    return put(b, i, j, block, true);
}

extern "C" int mgldg_bsr_builder_exists(const mgldg_bsr_builder* b, int i, int j, int* exists) {
    if (!b || !exists || i < 0 || i >= b->nbr || j < 0 || j >= b->nbc) return MGLDG_ERR_ARG;
    *exists = b->where.count(b->key(i, j)) ? 1 : 0;
    return MGLDG_OK;
}

extern "C" int mgldg_bsr_builder_nnzb(const mgldg_bsr_builder* b, int64_t* nnzb) {
    if (!b || !nnzb) return MGLDG_ERR_ARG;
    *nnzb = (int64_t)b->bi.size();
    return MGLDG_OK;
}

extern "C" int mgldg_bsr_builder_export(const mgldg_bsr_builder* b, int* row_ptr, int* col_idx, double* vals) {
    if (!b) return MGLDG_ERR_ARG;
    try {
        export_csr(b, row_ptr, col_idx, vals);
    } catch (const std::bad_alloc&) {
        return MGLDG_ERR_NOMEM;
    }
    return MGLDG_OK;
}

extern "C" int mgldg_bsr_builder_finalize(mgldg_ctx* ctx, const mgldg_bsr_builder* b, mgldg_bsr** A) {
    if (!ctx || !b || !A) return MGLDG_ERR_ARG;
    std::vector<int> rp, ci;
    std::vector<double> v;
    try {
        rp.resize((size_t)b->nbr + 1);
        ci.resize(b->bi.size());
        v.resize(b->vals.size());
        export_csr(b, rp.data(), ci.data(), v.data());
    } catch (const std::bad_alloc&) {
        return MGLDG_ERR_NOMEM;
    }
    return mgldg_bsr_create(ctx, b->nbr, b->nbc, b->br, b->bc, rp.data(), ci.data(), v.data(), A);
}

extern "C" int mgldg_bsr_builder_destroy(mgldg_bsr_builder* b) {
    delete b;
    return MGLDG_OK;
}

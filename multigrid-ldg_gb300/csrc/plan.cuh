// plan.cuh -- device-side symbolic pass of the block SpGEMM (plan.cu).
//
// A product plan lists, for every output block, the ordered terms that sum
// into it; the numeric pass (setup.cu k_prod) walks those lists.  The plan
// is built on the GPU in two passes over the operands' patterns: one counts
// the candidate terms of every operand row, the other writes each candidate
// as (output key, term) in the loop order of the reference's products; a
// stable radix sort by output key then groups the terms of each output block
// while keeping that loop order inside the group.
#pragma once

#include "internal.cuh"

namespace mg {

// Device plan: output pattern (row_ptr, col_idx), term ranges per output
// block (tptr) and the terms {x, m, y}: operand block indices of op(X), of
// the middle factor (-1 when there is none) and of Y.
struct DPlan {
    mgldg_ctx* ctx = nullptr;
    int nbr = 0, nbc = 0;
    int nkeys = 0;          // output blocks
    int64_t nterms = 0;
    int* row_ptr = nullptr;   // nbr + 1
    int* col_idx = nullptr;   // nkeys
    int* tptr = nullptr;      // nkeys + 1
    int3* terms = nullptr;    // nterms
    uint64_t* keys = nullptr; // nkeys: row * nbc + col of every output block
    DPlan() = default;
    DPlan(const DPlan&) = delete;
    DPlan& operator=(const DPlan&) = delete;
    DPlan(DPlan&& o) noexcept { *this = std::move(o); }
    DPlan& operator=(DPlan&& o) noexcept;
    ~DPlan() { release(); }
    void release();
};

// C = op(X) * Y: multiply_mm (tX false) or multiply_mm_t (tX true)
void dplan_mm(mgldg_ctx* ctx, const mgldg_bsr* X, bool tX, const mgldg_bsr* Y, DPlan* P);

// sum over rows k of X_d(k,i)^T D(k,k) X_d(k,j) for every X_d in Xs: one
// plan per d, all over the union pattern U of the d products and of
// `extra`'s pattern (null for none).  U carries the pattern only.
void dplan_triple(mgldg_ctx* ctx, const std::vector<const mgldg_bsr*>& Xs, const mgldg_bsr* D,
                  const mgldg_bsr* extra, std::vector<DPlan>* per, DPlan* U);

// one term per block of g: output block a = (row(a) inverse) * g(a)
void dplan_rowscale(mgldg_ctx* ctx, const mgldg_bsr* g, DPlan* P);

// src[q] = index of T's block at U's output position q, -1 where T has none
// (T's pattern must be contained in U's)
void dplan_scatter_index(mgldg_ctx* ctx, const DPlan& U, const mgldg_bsr* T, int* src);

// new BSR matrix with the plan's output pattern (values uninitialised)
mgldg_bsr* bsr_from_dplan(mgldg_ctx* ctx, const DPlan& P, int br, int bc);

}  // namespace mg

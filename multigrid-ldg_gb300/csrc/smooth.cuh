// smooth.cuh -- smoother schedules and launch entry points.
#pragma once

#include "internal.cuh"

namespace mg {

// device-resident sweep state of one level
struct GsSync {
    unsigned epoch;   // number of completed sweeps
    unsigned done;    // CTAs finished in the current sweep
    unsigned err;     // nonzero: a bounded wait ran out
    unsigned pad;
};

// level schedule of one matrix: [0] forward sweep, [1] reverse sweep
struct Sched {
    int n = 0;
    int nlev[2] = {0, 0};
    int* order[2] = {nullptr, nullptr};   // rows sorted by level
    int* wptr[2] = {nullptr, nullptr};    // per row: earlier neighbours to wait for
    int* widx[2] = {nullptr, nullptr};
    std::vector<int> h_level[2];
    unsigned* flags = nullptr;            // per row: sweep number of its last update
    GsSync* sync = nullptr;
    int64_t timeout_ns = 1000000000LL;    // bound on any single wait
};

void sched_build(mgldg_ctx* ctx, const mgldg_bsr* A, Sched& S);
void sched_free(Sched& S);
// returns 1 (and clears it) if a sweep recorded a wait timeout
int gs_take_error(mgldg_ctx* ctx, Sched& S);

template <class T>
void gs_sweep(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, T* x, Sched& S, T omega,
              bool reverse);
template <class T>
void jacobi_sweep(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, const T* xin,
                  T* xout, T omega);

}  // namespace mg

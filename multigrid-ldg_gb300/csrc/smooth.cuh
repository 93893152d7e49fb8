// smooth.cuh -- smoother schedules and launch entry points.
#pragma once

#include "internal.cuh"

namespace mg {

// device-resident sweep state of one level
struct GsSync {
    unsigned epoch;   // number of completed sweeps
    unsigned done;    // CTAs finished in the current pass
    unsigned err;     // nonzero: a bounded wait ran out
    unsigned pad;
};

// work list of one smoothing pass: nsw sweeps in direction dir (0 forward,
// 1 reverse), items (row << 3 | sweep) in the level order of the combined
// dependency graph
struct GsPass {
    int nsw = 0, dir = 0, nitems = 0, depth = 0;
    int* items = nullptr;
};

// Gauss-Seidel schedule of one matrix
struct Sched {
    int n = 0;
    const mgldg_bsr* A = nullptr;            // the pattern the passes are built from
    std::vector<std::vector<int>> nb;        // symmetrised neighbours of every row (host)
    int* xptr = nullptr;                     // per row: symmetrised neighbours outside its own pattern
    int* xidx = nullptr;
    std::vector<GsPass> passes;              // built on first use per (direction, sweeps)
    unsigned long long* xp = nullptr;        // packed published values, words_per_row per row
    int words_per_row = 0;
    GsSync* sync = nullptr;
    int64_t timeout_ns = 1000000000LL;       // bound on any single wait
};

void sched_build(mgldg_ctx* ctx, const mgldg_bsr* A, Sched& S);
void sched_free(Sched& S);
// returns 1 (and clears it) if a sweep recorded a wait timeout
int gs_take_error(mgldg_ctx* ctx, Sched& S);

// nsw >= 1 sweeps of block Gauss-Seidel (forward, or reverse), in place on x
template <class T>
void gs_sweeps(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, T* x, Sched& S, T omega,
               bool reverse, int nsw);
// one damped block-Jacobi sweep xin -> xout; xzero: xin is the zero vector
// (neither it nor A is read; same values as the full sweep)
template <class T>
void jacobi_sweep(mgldg_ctx* ctx, const mgldg_bsr* A, const T* vals, const T* Dinv, const T* b, const T* xin,
                  T* xout, T omega, bool xzero = false);

}  // namespace mg

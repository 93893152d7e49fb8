// tail.cuh -- the coarse end of the mixed-precision Jacobi V-cycle in one
// cooperative launch (tail.cu).
#pragma once

#include "internal.cuh"

struct mgldg_mg;

namespace mg {

constexpr int kTailMaxLevels = 12;

// a block-table interpolation operator (restriction T^T or prolongation T)
struct TailXfer {
    const int* rp;
    const int* ci;
    const int* blk;
    const float* tab;   // FP32 block table
    int nbr;            // block rows of the output
};

// one level of the tail (16 x 16 blocks, FP32); x / xt are the level's two
// iterate buffers as the host holds them when the V-cycle reaches the level
struct TailLevel {
    int nbr;
    const int* rp;
    const int* ci;
    const float* val;
    const float* Dinv;
    float* x;
    float* xt;
    float* b;
    float* r;
    TailXfer Tt;   // to the next coarser level
    TailXfer T;    // from the next coarser level
};

struct TailArgs {
    int nlev;   // levels s .. last; the last one is solved directly
    TailLevel L[kTailMaxLevels];
    int nc;
    const double* Cinv;
    float omega;
    int npre, npost;
    unsigned* count;   // barrier arrivals (zeroed before each launch)
    unsigned* err;     // the context's device error word
    int64_t timeout_ns;
};

// Can levels s .. last of m run as one tail launch?  Mixed (FP32) Jacobi
// V-cycle with npre >= 1, a direct coarsest solve without mean projection,
// 16 x 16 FP32 level operators and block-table transfers.
bool tail_supported(const mgldg_mg* m, int s);
// Runs the V-cycle from level s (its b set, its x zero) down to the coarsest
// and back up to level s's post-smoothed x, on the context's stream.
void tail_launch(mgldg_mg* m, int s, unsigned* count);

}  // namespace mg

// mg.cuh -- multigrid hierarchy data shared by the single- and multi-RHS
// V-cycles (mg.cu, batched.cu).
#pragma once

#include "internal.cuh"
#include "smooth.cuh"

namespace mg {

struct LevelData {
    mgldg_ops* ops = nullptr;    // owned for coarse levels
    bool owns_ops = false;
    const mgldg_bsr* A = nullptr;
    int ne = 0, b = 0;
    int64_t n = 0;
    double* Dinv = nullptr;
    float* Dinv32 = nullptr;
    Sched sched;
    bool has_sched = false;
    double *x = nullptr, *bb = nullptr, *r = nullptr, *xt = nullptr;
    float *x32 = nullptr, *b32 = nullptr, *r32 = nullptr, *xt32 = nullptr;
    mgldg_bsr* T = nullptr;    // interpolation to this level from the next coarser one
    mgldg_bsr* Tt = nullptr;   // its transpose (restriction)
};

template <class T>
struct LV;
template <>
struct LV<double> {
    static double*& x(LevelData& L) { return L.x; }
    static double*& b(LevelData& L) { return L.bb; }
    static double*& r(LevelData& L) { return L.r; }
    static double*& xt(LevelData& L) { return L.xt; }
    static const double* D(LevelData& L) { return L.Dinv; }
};
template <>
struct LV<float> {
    static float*& x(LevelData& L) { return L.x32; }
    static float*& b(LevelData& L) { return L.b32; }
    static float*& r(LevelData& L) { return L.r32; }
    static float*& xt(LevelData& L) { return L.xt32; }
    static const float* D(LevelData& L) { return L.Dinv32; }
};

struct Batch;
void batch_free(Batch* b);
struct SegWork;
void seg_free(SegWork* w);
// one preconditioner application s = V-cycle(r) from x = 0 (graph replay
// when possible) and the collection of device-side error reports (mg.cu)
void mg_precon(mgldg_mg* m, const double* r, double* s);
// the same with every launch issued directly (for capture into a graph)
void mg_precon_eager(mgldg_mg* m, const double* r, double* s);
void mg_take_errors(mgldg_mg* m);
// true when level i's V-cycle starts from x = 0 with a Jacobi sweep that
// reads neither x nor the operator, so x need not be zeroed (mg.cu)
bool zero_start(const mgldg_mg* m, int i);

struct PcgScalars {
    double delta_new, delta_old, delta0, alpha, beta, dq, rr, pad;
    int breakdown;
    int it;   // completed iterations (advanced on the device)
    int pad2[2];
};

}  // namespace mg

struct mgldg_mg {
    mgldg_ctx* ctx = nullptr;
    mgldg_mg_params p;
    std::vector<mg::LevelData> L;
    double* Cinv = nullptr;   // dense inverse of the coarsest matrix
    int nc = 0;
    // pcg work space
    double *r = nullptr, *d = nullptr, *q = nullptr, *s = nullptr, *hist = nullptr;
    float *dhi = nullptr, *dlo = nullptr;   // d as a float pair (mixed forms, double-float q = A d)
    int64_t pcg_n = 0;
    int pcg_maxit = 0;
    mg::PcgScalars* sc = nullptr;
    mg::PcgScalars* h_sc = nullptr;   // pinned
    // preconditioner V-cycles captured as CUDA graphs, keyed by (in, out)
    struct Graph {
        const double* in = nullptr;
        double* out = nullptr;
        double* part = nullptr;   // r.s partial sums written by the graph (or none)
        cudaGraphExec_t exec = nullptr;
        int64_t launches[MGLDG_K_NCLASS] = {0};
    };
    Graph graphs[2];
    int next_graph = 0;
    bool graphs_off = false;
    // one block of up to 50 PCG iterations (a residual-replacement iteration,
    // then the others in a device-side while loop) captured as a CUDA graph,
    // keyed by its operands
    struct PcgGraph {
        const mgldg_bsr* A = nullptr;
        const double* b = nullptr;
        double* x = nullptr;
        double tol = 0;
        int maxit = 0;
        cudaGraphExec_t exec = nullptr;
        int64_t pro_launches[MGLDG_K_NCLASS] = {0};    // the replacement iteration
        int64_t body_launches[MGLDG_K_NCLASS] = {0};   // one loop iteration
    };
    PcgGraph pg;
    bool pcg_graph_off = false;
    // device copies of the host vectors of mgldg_pcg, kept between calls
    // (stable addresses let the iteration graph be reused)
    double *host_b = nullptr, *host_x = nullptr;
    int64_t host_n = 0;
    // the coarse end of the mixed Jacobi V-cycle as one launch (tail.cu):
    // first level it covers (-1: none) and its barrier counter
    int tail_start = -1;
    unsigned* tail_count = nullptr;
    mg::Batch* batch = nullptr;   // multi-RHS work space (batched.cu)
    mg::SegWork* seg = nullptr;   // segmented-PCG work space (batched.cu)
    ~mgldg_mg();
};

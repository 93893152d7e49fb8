// ldg_build.cuh -- pieces shared by the problem builders (uniform
// Cartesian grids in cartesian.cu, adaptive quadtrees in quadtree.cu): the
// master-element tables, block helpers, per-block contribution lists and the
// problem handle.
#pragma once

#include <cstdint>
#include <initializer_list>
#include <vector>

#include "internal.cuh"
#include "master_tables.inc"

namespace mg {

typedef std::vector<double> Blk;   // row-major b x b

struct Gauss8 {
    double cx[8], cy[8], w[8], a[8];
};

struct Ref2 {
    int P, b;
    const double* nodes;
    const double* denom;
    const double* mass1;
    const double* invmass1;
    const double* diff1;
    explicit Ref2(int P_) : P(P_), b(P_ * P_) {
        nodes = kNodes[P - 1]; denom = kDenom[P - 1];
        mass1 = kMass1[P - 1]; invmass1 = kInvMass1[P - 1]; diff1 = kDiff1[P - 1];
    }
    // tensorProduct<2,P> (master.h:121-135)
    Blk tensor(const double* A) const {
        Blk M((size_t)b * b);
        for (int i0 = 0; i0 < P; ++i0)
            for (int i1 = 0; i1 < P; ++i1)
                for (int j0 = 0; j0 < P; ++j0)
                    for (int j1 = 0; j1 < P; ++j1) {
                        double v = 1.0;
                        v *= A[i0 * P + j0];
                        v *= A[i1 * P + j1];
                        M[(size_t)(i0 * P + i1) * b + j0 * P + j1] = v;
                    }
        return M;
    }
    // Master<2,P>::diff(dim) (master.h:45-68)
    Blk diff(int dim) const {
        Blk D((size_t)b * b, 0.0);
        for (int i0 = 0; i0 < P; ++i0)
            for (int i1 = 0; i1 < P; ++i1)
                for (int j0 = 0; j0 < P; ++j0)
                    for (int j1 = 0; j1 < P; ++j1) {
                        int it[2] = {i0, i1}, jt[2] = {j0, j1};
                        if (it[1 - dim] != jt[1 - dim]) continue;
                        D[(size_t)(i0 * P + i1) * b + j0 * P + j1] = diff1[it[dim] * P + jt[dim]];
                    }
        return D;
    }
    // LagrangePoly<P>::eval (master.h:79-94)
    void lagrange1(double x, double* l) const {
        double alpha = 1;
        l[0] = denom[0];
        for (int i = 0; i < P - 1; ++i) {
            alpha *= x - nodes[i];
            l[i + 1] = alpha * denom[i + 1];
        }
        double beta = 1;
        for (int i = P - 1; i > 0; --i) {
            beta *= x - nodes[i];
            l[i - 1] *= beta;
        }
    }
    void lagrange2(const double* x, double* out) const {
        double g0[8], g1[8];
        lagrange1(x[0], g0);
        lagrange1(x[1], g1);
        for (int i0 = 0; i0 < P; ++i0)
            for (int i1 = 0; i1 < P; ++i1) {
                double v = 1;
                v *= g0[i0];
                v *= g1[i1];
                out[i0 * P + i1] = v;
            }
    }
};

inline Blk bscale(double s, const Blk& A) {
    Blk C(A.size());
    for (size_t k = 0; k < A.size(); ++k) C[k] = s * A[k];
    return C;
}
inline Blk bmul(const Blk& A, const Blk& B, int b) {
    Blk C((size_t)b * b);
    for (int i = 0; i < b; ++i)
        for (int j = 0; j < b; ++j) {
            double s = 0;
            for (int k = 0; k < b; ++k) s += A[(size_t)i * b + k] * B[(size_t)k * b + j];
            C[(size_t)i * b + j] = s;
        }
    return C;
}
inline Blk btrans(const Blk& A, int b) {
    Blk C(A.size());
    for (int i = 0; i < b; ++i)
        for (int j = 0; j < b; ++j) C[(size_t)j * b + i] = A[(size_t)i * b + j];
    return C;
}

// builds one operator from per-block contribution lists
struct Assembly {
    std::vector<int> row_ptr, col_idx;
    std::vector<int64_t> tptr{0};
    std::vector<int> tidx;
    void begin_row() {}
    void add_block(int col, std::initializer_list<int> contrib) {
        col_idx.push_back(col);
        for (int c : contrib) tidx.push_back(c);
        tptr.push_back((int64_t)tidx.size());
    }
    void add_block_v(int col, const std::vector<int>& contrib) {
        col_idx.push_back(col);
        for (int c : contrib) tidx.push_back(c);
        tptr.push_back((int64_t)tidx.size());
    }
};


// GPU: one operator from per-block contribution lists over a table of
// distinct blocks (k_sum_blocks), and a one-block-per-row operator over a
// table of distinct blocks (transfers)
mgldg_bsr* realize(mgldg_ctx* ctx, const Assembly& As, int ne, int b, const double* d_table);
mgldg_bsr* table_operator(mgldg_ctx* ctx, int nbr, int nbc, int br, int bc, const std::vector<int>& col,
                          const std::vector<int>& blk, const std::vector<double>& table);
Gauss8 gaussian_params(uint64_t seed);

}  // namespace mg

// A discretised problem: LDG operators, its h-interpolation hierarchy and
// the element geometry (lower corner and width of every square element, in
// element order) for right-hand sides and nodal dumps.
struct mgldg_problem {
    mgldg_ctx* ctx = nullptr;
    int P = 0, b = 0, ne = 0;
    int n = 0;                    // elements per side of a uniform grid, 0 if adaptive
    double h = 0;                 // uniform width (uniform grids)
    mgldg_ops* ops = nullptr;
    std::vector<mgldg_bsr*> T;
    std::vector<double> ex, ey, ew;   // host geometry
    double* d_geom = nullptr;         // device: ex | ey | ew
    double* d_nodes = nullptr;
    double* d_Mref = nullptr;         // tensor mass of the master element
    int nfaces = 0, nbfaces = 0, nlevels = 0;
    // simplex meshes: dimension, per element geometry, the master nodes
    // (b x N), the master volume and the aggregates per level
    bool simplex = false;
    int sdim = 2;
    std::vector<double> sgeom, snodes;   // 22 doubles per element: p0, J, Jinv, volume
    double svref = 0;
    std::vector<std::vector<int>> partitions;
    ~mgldg_problem() {
        delete ops;
        for (auto* t : T) delete t;
        mg::dfree(d_geom);
        mg::dfree(d_nodes);
        mg::dfree(d_Mref);
    }
};

namespace mg {
// uploads geometry, nodes and the master mass matrix of a built problem
void problem_upload_geometry(mgldg_ctx* ctx, mgldg_problem* pr);
// right-hand side b = M f (disk Gaussian sum of seed; seed 0: f = 1) on a
// triangle mesh (simplex.cu)
void simplex_rhs_dev(mgldg_ctx* ctx, const mgldg_problem* pr, uint64_t seed, double* b);
// coordinates of every DOF's node, dim values per DOF in DOF order
int problem_node_coords(const mgldg_problem* pr, std::vector<double>& xy);
}  // namespace mg

// dg_binding.cpp -- the C++ binding of INTEGRATION.md, compiled as written
// against include/mgldg.h and libmgldg.so (TEST INFRASTRUCTURE ONLY).
//
// to_device() and solve_on_gpu() are the code a maintainer adds next to the
// reference's driver (tests/cartesian/dg_tests.cpp:294-307); main() feeds
// them a small block problem built with the reference types of
// reference_stub.h and checks the residual of the returned solution.
// Exit status: 0 solved, 1 wrong answer or library error, 3 no CUDA device.
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "mgldg.h"
#include "reference_stub.h"

struct NoDevice : std::runtime_error {
    using std::runtime_error::runtime_error;
};

static void check(mgldg_ctx* ctx, int rc) {
    if (rc != MGLDG_OK) throw std::runtime_error(ctx ? mgldg_last_error(ctx) : "mgldg call failed");
}

// ---- the binding ----
// SparseBlockMatrix<P,Q> -> device BSR (sparseblockmatrix.h:62-165)
template <int P, int Q>
mgldg_bsr* to_device(mgldg_ctx* ctx, const DG::SparseBlockMatrix<P, Q>& S) {
    std::vector<int> rp(S.blockRows() + 1, 0), ci;
    std::vector<double> v;
    for (int i = 0; i < S.blockRows(); ++i) {
        for (int j : S.colsInRow(i)) {                 // any order: the library sorts
            ci.push_back(j);
            const auto& B = S.getBlock(i, j);          // RowMajor Mat<P,Q>
            v.insert(v.end(), B.data(), B.data() + P * Q);
        }
        rp[i + 1] = (int)ci.size();
    }
    mgldg_bsr* A = nullptr;
    check(ctx, mgldg_bsr_create(ctx, S.blockRows(), S.blockCols(), P, Q, rp.data(), ci.data(), v.data(), &A));
    return A;
}

// replaces dg_tests.cpp:294-307 (hierarchy, Multigrid, precon lambda, pcg);
// returns the iteration count
template <int P>
int solve_on_gpu(DG::LDGPoisson<2, P>& poisson, const DG::InterpolationHierarchy<2, P>& hier,
                 const DG::MG::Parameters& p, const DG::Vector& rhs, DG::Vector& u, double tol, int maxit) {
    mgldg_ctx* ctx = nullptr;
    if (mgldg_ctx_create(0, &ctx) != MGLDG_OK) throw NoDevice("no CUDA device");
    int iters = 0;
    try {
        auto ops_h = poisson.ops();
        mgldg_bsr* G[2] = {to_device(ctx, ops_h->G[0]), to_device(ctx, ops_h->G[1])};
        mgldg_ops* ops = nullptr;
        check(ctx, mgldg_ops_create(ctx, 2, to_device(ctx, ops_h->M), G, to_device(ctx, ops_h->T), &ops));
        check(ctx, mgldg_ops_construct_laplacian(ctx, ops));   // A = T + sum G^T M G on the GPU
        std::vector<mgldg_bsr*> T;
        for (const auto& t : hier.T) T.push_back(to_device(ctx, t));
        mgldg_mg_params mp;
        mgldg_mg_params_default(&mp);
        mp.relaxation = p.relaxation; mp.omega = p.omega; mp.solver = p.solver;
        mp.npre = p.npre; mp.npost = p.npost; mp.restriction = p.restriction;
        mgldg_mg* mg = nullptr;
        check(ctx, mgldg_mg_create(ctx, ops, (const mgldg_bsr* const*)T.data(), (int)T.size(), &mp, &mg));
        const mgldg_bsr* A = nullptr;
        check(ctx, mgldg_ops_get(ops, 4, &A));
        std::vector<double> hist(maxit);
        check(ctx, mgldg_pcg(ctx, mg, A, rhs.data(), u.data(), tol, maxit, &iters, hist.data()));
        // hist[k] is the ||r|| the reference prints for cycle k (krylov.h:62)
        for (auto* t : T) mgldg_bsr_destroy(t);               // mg keeps its own copies
        mgldg_mg_destroy(mg);
        mgldg_ops_destroy(ops);
    } catch (...) {
        mgldg_ctx_destroy(ctx);
        throw;
    }
    mgldg_ctx_destroy(ctx);
    return iters;
}
// ---- end of the binding ----

// A chain of 4 elements with 4 x 4 blocks (the block size of Q1 elements in
// two dimensions): M = I, G_0 = forward differences,
// G_1 = 0, penalty T = I, so A = I + G_0^T G_0 is SPD; hierarchy 4 -> 2 -> 1.
int main() {
    constexpr int P = 4, ne = 4;
    using B = DG::Mat<P, P>;
    B I, mI;
    for (int k = 0; k < P; ++k) {
        I(k, k) = 1.0;
        mI(k, k) = -1.0;
    }
    DG::LDGPoisson<2, P> poisson;
    auto& o = *poisson.ops();
    o.M = DG::SparseBlockMatrix<P, P>(ne, ne);
    o.T = DG::SparseBlockMatrix<P, P>(ne, ne);
    o.G[0] = DG::SparseBlockMatrix<P, P>(ne, ne);
    o.G[1] = DG::SparseBlockMatrix<P, P>(ne, ne);
    for (int e = 0; e < ne; ++e) {
        o.M.addToBlock(e, e, I);
        o.T.addToBlock(e, e, I);
        o.G[0].addToBlock(e, e, I);
        if (e > 0) o.G[0].addToBlock(e, e - 1, mI);
        o.G[1].addToBlock(e, e, B{});
    }
    DG::InterpolationHierarchy<2, P> hier;
    for (int nc = ne / 2; nc >= 1; nc /= 2) {
        DG::SparseBlockMatrix<P, P> t(2 * nc, nc);
        for (int f = 0; f < 2 * nc; ++f) t.addToBlock(f, f / 2, I);
        hier.T.push_back(t);
    }
    DG::MG::Parameters prm;   // the reference defaults: V(3,3) Gauss-Seidel, RATRAT, one-element Cholesky
    DG::Vector rhs(ne * P), u(ne * P, 0.0);
    for (int k = 0; k < ne * P; ++k) rhs[k] = 1.0 + 0.25 * k;
    int iters = 0;
    try {
        iters = solve_on_gpu<P>(poisson, hier, prm, rhs, u, 1e-12, 100);
    } catch (const NoDevice& e) {
        std::printf("binding compiled and linked; %s\n", e.what());
        return 3;
    } catch (const std::exception& e) {
        std::printf("library error: %s\n", e.what());
        return 1;
    }
    // residual with A = I + G_0^T G_0 applied on the host
    std::vector<double> g(ne * P, 0.0), r(ne * P);
    for (int e = 0; e < ne; ++e)
        for (int c = 0; c < P; ++c) g[e * P + c] = u[e * P + c] - (e > 0 ? u[(e - 1) * P + c] : 0.0);
    double rn = 0, bn = 0;
    for (int e = 0; e < ne; ++e)
        for (int c = 0; c < P; ++c) {
            const double gtg = g[e * P + c] - (e + 1 < ne ? g[(e + 1) * P + c] : 0.0);
            r[e * P + c] = rhs[e * P + c] - (u[e * P + c] + gtg);
            rn += r[e * P + c] * r[e * P + c];
            bn += rhs[e * P + c] * rhs[e * P + c];
        }
    std::printf("solved in %d iterations, relative residual %.3e\n", iters, std::sqrt(rn / bn));
    return std::sqrt(rn / bn) <= 1e-10 ? 0 : 1;
}

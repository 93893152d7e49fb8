// oracle.cpp -- CPU oracle for the GB300 MG-PCG build.  TEST INFRASTRUCTURE
// ONLY: loaded by tests/, __graft_entry__.smoke() and bench.py's cpu_baseline
// leg as the checker; never linked into, or called by, the product.
//
// A plain C++17 restatement (no Eigen, no MKL) of the reference's Cartesian
// LDG Poisson solver path of danfortunato/multigrid-ldg.  Every routine names
// the reference file:line it follows.  The reference's data structures are
// kept where they decide summation order: SparseBlockMatrix is a hash map of
// dense blocks keyed by the Szudzik pairing of (i,j), with per-row and
// per-column std::unordered_set<int> index sets, filled in the same insertion
// sequence, so row sums are accumulated in the reference's iteration order.
// Dense block arithmetic (Eigen in the reference) is written out here: plain
// loops for products and an LDL^T factorisation with symmetric diagonal
// pivoting (Golub & Van Loan, Matrix Computations, sec. 4.2) for the
// Eigen::LDLT solves.
//
// Parity: unpinned against the reference binary (Eigen 3 and MKL are absent,
// so it cannot be built); pinned against the reference's constant tables,
// its 2x2 known answer and the manufactured-solution convergence rate.

#include "oracle.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <functional>
#include <limits>
#include <map>
#include <memory>
#include <random>
#include <stdexcept>
#include <unordered_map>
#include <unordered_set>
#include <vector>

namespace orc {

static const int NDIM = 2;   // dg_tests.cpp:361 runs the 2-D solver
static const int QF = 10;    // common.h:15 face quadrature points

// ---------------------------------------------------------------- dense --
struct Mat {
    int r = 0, c = 0;
    std::vector<double> a;
    Mat() {}
    Mat(int r_, int c_) : r(r_), c(c_), a((size_t)r_ * c_, 0.0) {}
    double& operator()(int i, int j) { return a[(size_t)i * c + j]; }
    double operator()(int i, int j) const { return a[(size_t)i * c + j]; }
    Mat& operator+=(const Mat& o) {
        for (size_t k = 0; k < a.size(); ++k) a[k] += o.a[k];
        return *this;
    }
};

static Mat scaled(double s, const Mat& A) {
    Mat C = A;
    for (auto& v : C.a) v = s * v;
    return C;
}
static Mat transpose(const Mat& A) {
    Mat C(A.c, A.r);
    for (int i = 0; i < A.r; ++i)
        for (int j = 0; j < A.c; ++j) C(j, i) = A(i, j);
    return C;
}
// C = A * B, each C(i,j) summed over k in ascending order
static Mat matmul(const Mat& A, const Mat& B) {
    Mat C(A.r, B.c);
    for (int i = 0; i < A.r; ++i)
        for (int j = 0; j < B.c; ++j) {
            double s = 0.0;
            for (int k = 0; k < A.c; ++k) s += A(i, k) * B(k, j);
            C(i, j) = s;
        }
    return C;
}
// C = A^T * B
static Mat matmul_tn(const Mat& A, const Mat& B) {
    Mat C(A.c, B.c);
    for (int i = 0; i < A.c; ++i)
        for (int j = 0; j < B.c; ++j) {
            double s = 0.0;
            for (int k = 0; k < A.r; ++k) s += A(k, i) * B(k, j);
            C(i, j) = s;
        }
    return C;
}
static Mat identity(int n) {
    Mat I(n, n);
    for (int i = 0; i < n; ++i) I(i, i) = 1.0;
    return I;
}

// LDL^T with symmetric diagonal pivoting: P A P^T = L D L^T.  At step k the
// largest remaining Schur-complement diagonal entry (in magnitude) is swapped
// into position k.  Stands in for Eigen::LDLT (multigrid.h:93-95,133-135,
// 168-170; ldgpoisson.h:25).  Extension: an unknown whose row and column are
// exactly zero (a dropped coarse basis function) is absent -- it is factored
// as a unit diagonal and its solution entry is zero (the pseudo-inverse).
struct LDLT {
    int n = 0;
    std::vector<double> L;   // unit lower triangle, row-major n x n
    std::vector<double> D;
    std::vector<int> tr;     // transposition applied at step k
    std::vector<char> absent;
    LDLT() {}
    explicit LDLT(const Mat& A) { factor(A); }
    void factor(const Mat& A) {
        n = A.r;
        std::vector<double> W(A.a);
        absent.assign(n, 0);
        for (int i = 0; i < n; ++i) {
            bool z = true;
            for (int j = 0; j < n && z; ++j) z = W[(size_t)i * n + j] == 0.0 && W[(size_t)j * n + i] == 0.0;
            if (z) {
                absent[i] = 1;
                W[(size_t)i * n + i] = 1.0;
            }
        }
        tr.assign(n, 0);
        D.assign(n, 0.0);
        for (int k = 0; k < n; ++k) {
            int p = k;
            double best = std::fabs(W[(size_t)k * n + k]);
            for (int i = k + 1; i < n; ++i) {
                double v = std::fabs(W[(size_t)i * n + i]);
                if (v > best) { best = v; p = i; }
            }
            tr[k] = p;
            if (p != k) {
                for (int j = 0; j < n; ++j) std::swap(W[(size_t)k * n + j], W[(size_t)p * n + j]);
                for (int i = 0; i < n; ++i) std::swap(W[(size_t)i * n + k], W[(size_t)i * n + p]);
            }
            double dk = W[(size_t)k * n + k];
            D[k] = dk;
            // column k of L (stored in the strict lower part of W)
            for (int i = k + 1; i < n; ++i) W[(size_t)i * n + k] /= dk;
            // Schur complement update of the trailing block
            for (int i = k + 1; i < n; ++i) {
                double lik = W[(size_t)i * n + k];
                for (int j = k + 1; j <= i; ++j) {
                    double v = W[(size_t)i * n + j] - lik * dk * W[(size_t)j * n + k];
                    W[(size_t)i * n + j] = v;
                    W[(size_t)j * n + i] = v;
                }
            }
        }
        L.assign((size_t)n * n, 0.0);
        for (int i = 0; i < n; ++i) {
            L[(size_t)i * n + i] = 1.0;
            for (int j = 0; j < i; ++j) L[(size_t)i * n + j] = W[(size_t)i * n + j];
        }
    }
    void solve_inplace(double* x) const {
        for (int k = 0; k < n; ++k)
            if (tr[k] != k) std::swap(x[k], x[tr[k]]);
        for (int i = 0; i < n; ++i) {
            double s = x[i];
            for (int j = 0; j < i; ++j) s -= L[(size_t)i * n + j] * x[j];
            x[i] = s;
        }
        for (int i = 0; i < n; ++i) x[i] /= D[i];
        for (int i = n - 1; i >= 0; --i) {
            double s = x[i];
            for (int j = i + 1; j < n; ++j) s -= L[(size_t)j * n + i] * x[j];
            x[i] = s;
        }
        for (int k = n - 1; k >= 0; --k)
            if (tr[k] != k) std::swap(x[k], x[tr[k]]);
        for (int i = 0; i < n; ++i)
            if (absent[i]) x[i] = 0.0;
    }
    std::vector<double> solve(const double* b) const {
        std::vector<double> x(b, b + n);
        solve_inplace(x.data());
        return x;
    }
    Mat solve(const Mat& B) const {   // column by column
        Mat X(B.r, B.c);
        std::vector<double> col(n);
        for (int j = 0; j < B.c; ++j) {
            for (int i = 0; i < n; ++i) col[i] = B(i, j);
            solve_inplace(col.data());
            for (int i = 0; i < n; ++i) X(i, j) = col[i];
        }
        return X;
    }
};

// ------------------------------------------------------- reference tables --
// GaussLobatto<P>, LagrangePoly<P>, Master<1,P> and Quadrature<Q> of
// master.h:147-214, recomputed from their definitions in long double and
// rounded to double.
typedef long double ld;

static ld legendre(int n, ld t, ld* dp) {
    ld p0 = 1, p1 = t;
    if (n == 0) { if (dp) *dp = 0; return 1; }
    for (int k = 2; k <= n; ++k) {
        ld p2 = ((2 * k - 1) * t * p1 - (k - 1) * p0) / k;
        p0 = p1; p1 = p2;
    }
    if (dp) *dp = n * (t * p1 - p0) / (t * t - 1);
    return p1;
}

struct Tables {
    int P = 0;
    std::vector<double> nodes, denom, mass, invmass, diff;
};

static std::vector<ld> gll_nodes_ld(int P) {
    std::vector<ld> x(P);
    if (P == 1) { x[0] = 0.5L; return x; }
    const ld pi = 3.141592653589793238462643383279502884L;
    int n = P - 1;   // interior nodes are the roots of P_n'(t)
    x[0] = 0; x[P - 1] = 1;
    for (int i = 1; i < P - 1; ++i) {
        ld t = -std::cos(pi * i / n);
        for (int it = 0; it < 100; ++it) {
            // f = P_n'(t);  f' = P_n''(t) = (2t P_n' - n(n+1) P_n) / (1 - t^2)
            ld dp;
            ld p = legendre(n, t, &dp);
            ld d2 = (2 * t * dp - n * (n + 1) * p) / (1 - t * t);
            ld dt = dp / d2;
            t -= dt;
            if (std::fabs(dt) < 1e-30L) break;
        }
        x[i] = (t + 1) / 2;
    }
    return x;
}

static void gauss_legendre_ld(int Q, std::vector<ld>& x, std::vector<ld>& w) {
    const ld pi = 3.141592653589793238462643383279502884L;
    x.assign(Q, 0); w.assign(Q, 0);
    for (int i = 0; i < Q; ++i) {
        ld t = -std::cos(pi * (i + 0.75L) / (Q + 0.5L));
        ld dp = 0;
        for (int it = 0; it < 100; ++it) {
            ld p = legendre(Q, t, &dp);
            ld dt = p / dp;
            t -= dt;
            if (std::fabs(dt) < 1e-30L) break;
        }
        legendre(Q, t, &dp);
        x[i] = (t + 1) / 2;
        w[i] = 1 / ((1 - t * t) * dp * dp);   // 2/((1-t^2)P'^2) scaled to [0,1]
    }
}

static const Tables& tables(int P) {
    static std::unordered_map<int, Tables> cache;
    auto it = cache.find(P);
    if (it != cache.end()) return it->second;
    if (P < 1 || P > 6) throw std::invalid_argument("P out of range");
    Tables T;
    T.P = P;
    std::vector<ld> x = gll_nodes_ld(P);
    std::vector<ld> den(P);
    for (int i = 0; i < P; ++i) {
        ld d = 1;
        for (int k = 0; k < P; ++k) if (k != i) d *= (x[i] - x[k]);
        den[i] = 1 / d;
    }
    // mass: exact integral of l_i l_j on [0,1] (Gauss rule with P+1 points)
    std::vector<ld> qx, qw;
    gauss_legendre_ld(P + 1, qx, qw);
    std::vector<ld> M((size_t)P * P, 0);
    for (int q = 0; q < P + 1; ++q) {
        std::vector<ld> l(P);
        for (int i = 0; i < P; ++i) {
            ld v = den[i];
            for (int k = 0; k < P; ++k) if (k != i) v *= (qx[q] - x[k]);
            l[i] = v;
        }
        for (int i = 0; i < P; ++i)
            for (int j = 0; j < P; ++j) M[(size_t)i * P + j] += qw[q] * l[i] * l[j];
    }
    // inverse by Gauss-Jordan in long double
    std::vector<ld> Aug((size_t)P * 2 * P, 0);
    for (int i = 0; i < P; ++i) {
        for (int j = 0; j < P; ++j) Aug[(size_t)i * 2 * P + j] = M[(size_t)i * P + j];
        Aug[(size_t)i * 2 * P + P + i] = 1;
    }
    for (int k = 0; k < P; ++k) {
        int p = k;
        for (int i = k + 1; i < P; ++i)
            if (std::fabs(Aug[(size_t)i * 2 * P + k]) > std::fabs(Aug[(size_t)p * 2 * P + k])) p = i;
        for (int j = 0; j < 2 * P; ++j) std::swap(Aug[(size_t)k * 2 * P + j], Aug[(size_t)p * 2 * P + j]);
        ld piv = Aug[(size_t)k * 2 * P + k];
        for (int j = 0; j < 2 * P; ++j) Aug[(size_t)k * 2 * P + j] /= piv;
        for (int i = 0; i < P; ++i) {
            if (i == k) continue;
            ld f = Aug[(size_t)i * 2 * P + k];
            for (int j = 0; j < 2 * P; ++j) Aug[(size_t)i * 2 * P + j] -= f * Aug[(size_t)k * 2 * P + j];
        }
    }
    // differentiation: D(i,j) = l_j'(x_i)
    std::vector<ld> Dm((size_t)P * P, 0);
    for (int i = 0; i < P; ++i) {
        for (int j = 0; j < P; ++j) {
            if (i != j) {
                Dm[(size_t)i * P + j] = (den[j] / den[i]) / (x[i] - x[j]);
            } else {
                ld s = 0;
                for (int k = 0; k < P; ++k) if (k != i) s += 1 / (x[i] - x[k]);
                // interior Gauss-Lobatto nodes are symmetric about 1/2, so the
                // exact diagonal is zero there; drop the long-double residue
                if (std::fabs(s) < 1e-12L) s = 0;
                Dm[(size_t)i * P + j] = s;
            }
        }
    }
    T.nodes.resize(P); T.denom.resize(P);
    T.mass.resize((size_t)P * P); T.invmass.resize((size_t)P * P); T.diff.resize((size_t)P * P);
    for (int i = 0; i < P; ++i) { T.nodes[i] = (double)x[i]; T.denom[i] = (double)den[i]; }
    for (int i = 0; i < P; ++i)
        for (int j = 0; j < P; ++j) {
            T.mass[(size_t)i * P + j] = (double)M[(size_t)i * P + j];
            T.invmass[(size_t)i * P + j] = (double)Aug[(size_t)i * 2 * P + P + j];
            T.diff[(size_t)i * P + j] = (double)Dm[(size_t)i * P + j];
        }
    return cache.emplace(P, std::move(T)).first->second;
}

static void quadrature(int Q, std::vector<double>& x, std::vector<double>& w) {
    std::vector<ld> xl, wl;
    gauss_legendre_ld(Q, xl, wl);
    x.resize(Q); w.resize(Q);
    for (int i = 0; i < Q; ++i) { x[i] = (double)xl[i]; w[i] = (double)wl[i]; }
}

// tensorProduct<N,P> (master.h:121-135): M(i,j) = prod_k A(i_k, j_k), k ascending
static Mat tensor2(const std::vector<double>& A, int P) {
    int b = P * P;
    Mat M(b, b);
    for (int i0 = 0; i0 < P; ++i0)
        for (int i1 = 0; i1 < P; ++i1)
            for (int j0 = 0; j0 < P; ++j0)
                for (int j1 = 0; j1 < P; ++j1) {
                    double v = 1.0;
                    v *= A[(size_t)i0 * P + j0];
                    v *= A[(size_t)i1 * P + j1];
                    M(i0 * P + i1, j0 * P + j1) = v;
                }
    return M;
}

// Master<2,P>::diff(i) (master.h:45-68)
static Mat master_diff(int P, int dim) {
    const Tables& T = tables(P);
    int b = P * P;
    Mat D(b, b);
    for (int i0 = 0; i0 < P; ++i0)
        for (int i1 = 0; i1 < P; ++i1)
            for (int j0 = 0; j0 < P; ++j0)
                for (int j1 = 0; j1 < P; ++j1) {
                    int it[2] = {i0, i1}, jt[2] = {j0, j1};
                    bool nz = true;
                    for (int k = 0; k < NDIM; ++k)
                        if (k != dim && it[k] != jt[k]) { nz = false; break; }
                    if (nz) D(i0 * P + i1, j0 * P + j1) = T.diff[(size_t)it[dim] * P + jt[dim]];
                }
    return D;
}

// LagrangePoly<P>::eval(double) (master.h:79-94)
static void lagrange1(int P, double x, double* l) {
    const Tables& T = tables(P);
    double alpha = 1;
    l[0] = T.denom[0];
    for (int i = 0; i < P - 1; ++i) {
        alpha *= x - T.nodes[i];
        l[i + 1] = alpha * T.denom[i + 1];
    }
    double beta = 1;
    for (int i = P - 1; i > 0; --i) {
        beta *= x - T.nodes[i];
        l[i - 1] *= beta;
    }
}
// LagrangePoly<P>::eval(Tuple<double,N>) (master.h:96-115)
static void lagrange2(int P, const double* x, double* out) {
    double g[2][8];
    for (int j = 0; j < NDIM; ++j) lagrange1(P, x[j], g[j]);
    for (int i0 = 0; i0 < P; ++i0)
        for (int i1 = 0; i1 < P; ++i1) {
            double v = 1;
            v *= g[0][i0];
            v *= g[1][i1];
            out[i0 * P + i1] = v;
        }
}

// ----------------------------------------------------- sparse block matrix --
// SparseBlockMatrix<P,Q> (sparseblockmatrix.h:14-165, sparseblockmatrix.tpp)
struct Index {
    int i, j;
    bool operator==(const Index& o) const { return i == o.i && j == o.j; }
};
struct IndexHasher {
    // Szudzik pairing evaluated in wrapping 32-bit int arithmetic, then
    // widened like an int -> size_t conversion (sparseblockmatrix.h:43-48)
    size_t operator()(const Index& x) const {
        uint32_t i = (uint32_t)x.i, j = (uint32_t)x.j;
        uint32_t h = (x.i >= x.j) ? i * i + i + j : i + j * j;
        return (size_t)(int64_t)(int32_t)h;
    }
};

struct SBM {
    int m = 0, n = 0, P = 0, Q = 0;
    std::unordered_map<Index, Mat, IndexHasher> map;
    std::unordered_map<int, std::unordered_set<int>> cir, ric;
    std::unordered_set<int> empty;
    SBM() {}
    SBM(int m_, int n_, int P_, int Q_) : m(m_), n(n_), P(P_), Q(Q_) {}
    void reset(int m_, int n_) { m = m_; n = n_; map.clear(); cir.clear(); ric.clear(); }
    int blockRows() const { return m; }
    int blockCols() const { return n; }
    int rows() const { return m * P; }
    int cols() const { return n * Q; }
    bool exists(int i, int j) const { return map.count(Index{i, j}) > 0; }
    const Mat& get(int i, int j) const { return map.at(Index{i, j}); }
    void set(int i, int j, const Mat& b) {
        map[Index{i, j}] = b;
        cir[i].insert(j);
        ric[j].insert(i);
    }
    void add(int i, int j, const Mat& b) {
        if (exists(i, j)) map[Index{i, j}] += b;
        else set(i, j, b);
    }
    const std::unordered_set<int>& colsInRow(int i) const {
        auto it = cir.find(i);
        return it == cir.end() ? empty : it->second;
    }
    const std::unordered_set<int>& rowsInCol(int j) const {
        auto it = ric.find(j);
        return it == ric.end() ? empty : it->second;
    }
    long nnzb() const { return (long)map.size(); }
};

// multiply_mm (sparseblockmatrix.tpp:234-250): C := A * B
static void multiply_mm(const SBM& A, const SBM& B, SBM& C) {
    if (A.blockCols() != B.blockRows()) throw std::invalid_argument("shape");
    C.P = A.P; C.Q = B.Q;
    C.reset(A.blockRows(), B.blockCols());
    for (int i = 0; i < A.blockRows(); ++i)
        for (int k : A.colsInRow(i))
            for (int j : B.colsInRow(k)) C.add(i, j, matmul(A.get(i, k), B.get(k, j)));
}
// multiply_mm_t (sparseblockmatrix.tpp:261-277): C := A^T * B
static void multiply_mm_t(const SBM& A, const SBM& B, SBM& C) {
    if (A.blockRows() != B.blockRows()) throw std::invalid_argument("shape");
    C.P = A.Q; C.Q = B.Q;
    C.reset(A.blockCols(), B.blockCols());
    for (int i = 0; i < A.blockCols(); ++i)
        for (int k : A.rowsInCol(i))
            for (int j : B.colsInRow(k)) C.add(i, j, matmul_tn(A.get(k, i), B.get(k, j)));
}
// multiply_add_mv (sparseblockmatrix.tpp:358-371): y := alpha*A*x + beta*y
static void multiply_add_mv(double alpha, const SBM& A, const double* x, double beta, double* y) {
    const int P = A.P, Q = A.Q;
    std::vector<double> t(P);
    for (int i = 0; i < A.blockRows(); ++i) {
        double* yi = y + (size_t)P * i;
        for (int r = 0; r < P; ++r) yi[r] *= beta;
        for (int j : A.colsInRow(i)) {
            const Mat& B = A.get(i, j);
            const double* xj = x + (size_t)Q * j;
            for (int r = 0; r < P; ++r) {
                double s = 0.0;
                for (int c = 0; c < Q; ++c) s += B(r, c) * xj[c];
                yi[r] += alpha * s;
            }
        }
    }
}
// multiply_mv (sparseblockmatrix.tpp:288-301): y := A*x
static void multiply_mv(const SBM& A, const double* x, double* y) {
    const int P = A.P, Q = A.Q;
    for (int i = 0; i < A.blockRows(); ++i) {
        double* yi = y + (size_t)P * i;
        for (int r = 0; r < P; ++r) yi[r] = 0.0;
        for (int j : A.colsInRow(i)) {
            const Mat& B = A.get(i, j);
            const double* xj = x + (size_t)Q * j;
            for (int r = 0; r < P; ++r) {
                double s = 0.0;
                for (int c = 0; c < Q; ++c) s += B(r, c) * xj[c];
                yi[r] += s;
            }
        }
    }
}
// multiply_mv_t (sparseblockmatrix.tpp:322-335): y := A^T*x
static void multiply_mv_t(const SBM& A, const double* x, double* y) {
    const int P = A.P, Q = A.Q;
    for (int i = 0; i < A.blockCols(); ++i) {
        double* yi = y + (size_t)Q * i;
        for (int c = 0; c < Q; ++c) yi[c] = 0.0;
        for (int j : A.rowsInCol(i)) {
            const Mat& B = A.get(j, i);
            const double* xj = x + (size_t)P * j;
            for (int c = 0; c < Q; ++c) {
                double s = 0.0;
                for (int r = 0; r < P; ++r) s += B(r, c) * xj[r];
                yi[c] += s;
            }
        }
    }
}

// ------------------------------------------------------------- quadtree --
// Quadtree<2> (quadtree.h:92-223, quadtree.tpp)
struct Cell {
    double lo[2] = {0, 0}, hi[2] = {1, 1};
    double width(int d) const { return hi[d] - lo[d]; }
    double volume() const { double v = 1; for (int i = 0; i < NDIM; ++i) v *= width(i); return v; }
};
static bool cell_eq(const Cell& a, const Cell& b) {
    for (int i = 0; i < NDIM; ++i)
        if (a.lo[i] != b.lo[i] || a.hi[i] != b.hi[i]) return false;
    return true;
}

enum Direction { kLeft, kRight };

struct Quadtree {
    struct Node {
        int id, level = 0, height = 0, parent;
        Cell cell;
        int children[4] = {-1, -1, -1, -1};
    };
    std::vector<Node> tree;
    int numLevels = 1;
    int strategy = ORC_COARSEN_EQUAL;
    bool periodic = false;
    std::function<double(const double*)> h;   // isotropic h(x)

    Quadtree(std::function<double(const double*)> h_, int strategy_, bool periodic_)
        : strategy(strategy_), periodic(periodic_), h(h_) {
        Node root;
        root.id = 0; root.parent = -1;
        tree.push_back(root);
        build(0, 0);
    }
    // quadtree.tpp:10-40
    void build(int id, int level) {
        numLevels = std::max(level + 1, numLevels);
        tree[id].level = level;
        tree[id].height = 0;
        double mid[2];
        for (int i = 0; i < NDIM; ++i) mid[i] = tree[id].cell.lo[i] + tree[id].cell.width(i) / 2;
        double hv = h(mid);
        bool refine = true;
        for (int i = 0; i < NDIM; ++i)
            if (!(tree[id].cell.width(i) > hv)) refine = false;
        if (refine) {
            for (int b0 = 0; b0 < 2; ++b0)
                for (int b1 = 0; b1 < 2; ++b1) {
                    int bits[2] = {b0, b1};
                    Cell c = tree[id].cell;
                    for (int i = 0; i < NDIM; ++i) {
                        if (bits[i]) c.lo[i] = mid[i];
                        else c.hi[i] = mid[i];
                    }
                    int next = (int)tree.size();
                    Node nd;
                    nd.id = next; nd.parent = id; nd.cell = c;
                    tree.push_back(nd);
                    tree[id].children[b0 * 2 + b1] = next;
                    build(next, level + 1);
                }
            for (int k = 0; k < 4; ++k)
                tree[id].height = std::max(tree[tree[id].children[k]].height, tree[id].height);
            tree[id].height++;
        }
    }
    // Extension (the reference does not balance its trees): 2:1 face
    // balance.  A leaf is split while a face neighbour leaf is two or more
    // levels finer; only forced splits are made, so the result is the
    // unique coarsest balanced refinement.
    void split(int id) {
        double mid[2];
        for (int i = 0; i < NDIM; ++i) mid[i] = tree[id].cell.lo[i] + tree[id].cell.width(i) / 2;
        for (int b0 = 0; b0 < 2; ++b0)
            for (int b1 = 0; b1 < 2; ++b1) {
                int bits[2] = {b0, b1};
                Cell c = tree[id].cell;
                for (int i = 0; i < NDIM; ++i) {
                    if (bits[i]) c.lo[i] = mid[i];
                    else c.hi[i] = mid[i];
                }
                Node nd;
                nd.id = (int)tree.size(); nd.parent = id; nd.cell = c;
                nd.level = tree[id].level + 1;
                tree.push_back(nd);
                tree[id].children[b0 * 2 + b1] = nd.id;
            }
        numLevels = std::max(numLevels, tree[id].level + 2);
        for (int a = id; a >= 0; a = tree[a].parent) {
            int h = 0;
            for (int k = 0; k < 4; ++k) h = std::max(h, tree[tree[a].children[k]].height + 1);
            if (tree[a].height == h && a != id) break;
            tree[a].height = h;
        }
    }
    void balance() {
        bool changed = true;
        while (changed) {
            changed = false;
            std::vector<int> leaves;
            for (const Node& nd : tree)
                if (nd.children[0] < 0) leaves.push_back(nd.id);
            for (int id : leaves) {
                bool need = false;
                for (int i = 0; i < NDIM && !need; ++i)
                    for (Direction dir : {kLeft, kRight}) {
                        for (int nb : neighbors(id, i, dir, 0))
                            if (tree[nb].level >= tree[id].level + 2) need = true;
                        if (need) break;
                    }
                if (need) {
                    split(id);
                    changed = true;
                }
            }
        }
    }
    // quadtree.h:164-173
    bool isLeaf(const Node& node, int coarsening) const {
        if (strategy == ORC_COARSEN_RAPID) {
            return node.height == coarsening ||
                   (node.height < coarsening && node.parent >= 0 && tree[node.parent].height > coarsening);
        }
        int clevel = numLevels - 1 - coarsening;
        return node.level == clevel || (node.level < clevel && node.height == 0);
    }
    template <typename F>
    void dfs(const F& f, int id, int coarsening) const {
        f(tree[id]);
        if (!isLeaf(tree[id], coarsening))
            for (int k = 0; k < 4; ++k) dfs(f, tree[id].children[k], coarsening);
    }
    // quadtree.h:176-186
    std::vector<int> layer(int l) const {
        std::vector<int> out;
        dfs([&](const Node& nd) { if (isLeaf(nd, l)) out.push_back(nd.id); }, 0, l);
        return out;
    }
    // quadtree.tpp:58-87
    bool isNeighbor(const Node& a, const Node& b, int dim, Direction dir) const {
        double planeA = (dir == kLeft) ? a.cell.lo[dim] : a.cell.hi[dim];
        double planeB = (dir == kLeft) ? b.cell.hi[dim] : b.cell.lo[dim];
        if (periodic) {
            double doml = tree[0].cell.lo[dim], domu = tree[0].cell.hi[dim];
            if ((dir == kLeft && planeA == doml && planeB == domu) ||
                (dir == kRight && planeA == domu && planeB == doml))
                planeB = planeA;
        }
        if (planeA != planeB) return false;
        for (int i = 0; i < NDIM; ++i)
            if (i != dim)
                if (!(b.cell.hi[i] > a.cell.lo[i] && b.cell.lo[i] < a.cell.hi[i])) return false;
        return true;
    }
    // quadtree.tpp:90-98
    bool isParent(const Node& a, const Node& b) const {
        bool ge = true, le = true, eq = true;
        for (int i = 0; i < NDIM; ++i) {
            if (!(a.cell.lo[i] >= b.cell.lo[i])) ge = false;
            if (!(a.cell.hi[i] <= b.cell.hi[i])) le = false;
            if (!(a.cell.lo[i] == b.cell.lo[i] && a.cell.hi[i] == b.cell.hi[i])) eq = false;
        }
        return ge && le && !eq;
    }
    // quadtree.tpp:44-56 and 100-114
    void search(int aid, int dim, Direction dir, int id, int coarsening, std::vector<int>& v) const {
        const Node& a = tree[aid];
        const Node& nd = tree[id];
        if (isNeighbor(a, nd, dim, dir) || isParent(a, nd)) {
            if (!isLeaf(nd, coarsening)) {
                for (int k = 0; k < 4; ++k) search(aid, dim, dir, nd.children[k], coarsening, v);
            } else {
                v.push_back(nd.id);
            }
        }
    }
    std::vector<int> neighbors(int id, int dim, Direction dir, int coarsening) const {
        std::vector<int> v;
        search(id, dim, dir, 0, coarsening, v);
        return v;
    }
};

// ----------------------------------------------------------------- mesh --
// Face / Element / Mesh (mesh.h:17-374)
struct Face {
    int left, right, dim;
    double normal;      // normal[dim]; the other components are zero
    Cell cell;
    bool canonical = true;
    double xl[QF][2], xr[QF][2];
    bool interiorQ() const { return right >= 0; }
    bool boundaryQ() const { return right < 0; }
    int boundary() const { return boundaryQ() ? right : 0; }
    double area() const {
        double a = 1;
        for (int i = 0; i < NDIM; ++i) if (i != dim) a *= cell.width(i);
        return a;
    }
};

struct Mesh {
    int P = 0, npl = 0;
    std::vector<Cell> elements;       // lid -> cell
    std::vector<int> L2G;
    std::unordered_map<int, int> G2L;
    std::vector<Face> faces;
    std::vector<int> boundaryIndices;
    int nb = 0;
    std::vector<double> qx, qw;       // Quadrature<10>

    Mesh(const Quadtree& qt, int P_) : P(P_), npl(P_ * P_) {
        quadrature(QF, qx, qw);
        for (int i = 0; i < NDIM; ++i) {
            int index = 2 * i + 1;
            boundaryIndices.push_back(-index);
            boundaryIndices.push_back(-(index + 1));
        }
        std::vector<int> ids = qt.layer(0);
        L2G.resize(ids.size());
        for (int gid : ids) {
            int lid = (int)elements.size();
            G2L[gid] = lid;
            L2G[lid] = gid;
            elements.push_back(qt.tree[gid].cell);
        }
        // mesh.h:210-261
        for (int lid = 0; lid < (int)elements.size(); ++lid) {
            int gid = L2G[lid];
            for (int i = 0; i < NDIM; ++i) {
                for (Direction dir : {kLeft, kRight}) {
                    std::vector<int> nbrs = qt.neighbors(gid, i, dir, 0);
                    if (nbrs.empty()) {
                        double outward = (dir == kLeft) ? -1 : 1;
                        Cell fc = elements[lid];
                        if (dir == kLeft) fc.hi[i] = fc.lo[i]; else fc.lo[i] = fc.hi[i];
                        int bnd = boundaryIndices[2 * i + (dir == kRight)];
                        faces.push_back(make_face(lid, bnd, i, outward, fc));
                        nb++;
                    } else {
                        for (int ngid : nbrs) {
                            int nlid = G2L.at(ngid);
                            if (lid < nlid) {
                                int left = (dir == kLeft) ? nlid : lid;
                                int right = (dir == kRight) ? nlid : lid;
                                Cell fc;
                                for (int d = 0; d < NDIM; ++d) {
                                    fc.lo[d] = std::max(elements[left].lo[d], elements[right].lo[d]);
                                    fc.hi[d] = std::min(elements[left].hi[d], elements[right].hi[d]);
                                }
                                fc.lo[i] = elements[right].lo[i];
                                fc.hi[i] = elements[left].hi[i];
                                faces.push_back(make_face(left, right, i, 1.0, fc));
                            }
                        }
                    }
                }
            }
        }
    }

    // Face constructor (mesh.h:21-79)
    Face make_face(int left, int right, int dim, double normal, const Cell& cell) const {
        Face f;
        f.left = left; f.right = right; f.dim = dim; f.normal = normal; f.cell = cell;
        f.canonical = true;
        if (f.interiorQ()) {
            Cell lcell = elements[left], rcell = elements[right];
            lcell.lo[dim] = lcell.hi[dim];
            rcell.hi[dim] = rcell.lo[dim];
            f.canonical = cell_eq(lcell, rcell);
            if (!f.canonical) {
                double al[2], bl[2], ar[2], br[2];
                for (int i = 0; i < NDIM; ++i) {
                    al[i] = cell.lo[i] - lcell.lo[i];
                    bl[i] = cell.hi[i] - lcell.lo[i];
                    ar[i] = cell.lo[i] - rcell.lo[i];
                    br[i] = cell.hi[i] - rcell.lo[i];
                }
                for (int i = 0; i < NDIM; ++i) {
                    if (i != dim) {
                        al[i] /= lcell.width(i);
                        bl[i] /= lcell.width(i);
                        ar[i] /= rcell.width(i);
                        br[i] /= rcell.width(i);
                    }
                }
                for (int q = 0; q < QF; ++q) {
                    double x = qx[q];
                    int kk = 0 + (0 >= dim);   // the single tangential dimension
                    f.xl[q][kk] = al[kk] + (bl[kk] - al[kk]) * x;
                    f.xr[q][kk] = ar[kk] + (br[kk] - ar[kk]) * x;
                    f.xl[q][dim] = 1;
                    f.xr[q][dim] = 0;
                }
            }
        }
        return f;
    }

    double volume(int e) const { return elements[e].volume(); }
    Mat mass(int e) const {
        Mat M = tensor2(tables(P).mass, P);
        return scaled(volume(e), M);
    }
    Mat invmass(int e) const {
        Mat M = tensor2(tables(P).invmass, P);
        double jac = 1 / volume(e);
        return scaled(jac, M);
    }

    // lift (mesh.h:282-352).  L is returned as npl x QF (test from left).
    void lift(const Face& f, Mat* L, Mat* R, Mat* LL, Mat* RR, Mat* RL) const {
        const Tables& T = tables(P);
        if (f.canonical && !f.boundaryQ()) {
            // face mass = Master<1,P>::mass * area; slicing onto the traces
            double area = f.area();
            int jl[8], jr[8];
            for (int a = 0; a < P; ++a) {
                int jt[2];
                jt[1 - f.dim] = a;   // tangential index
                jt[f.dim] = (f.normal > 0) ? P - 1 : 0;
                jl[a] = jt[0] * P + jt[1];
                jt[f.dim] = (f.normal > 0) ? 0 : P - 1;
                jr[a] = jt[0] * P + jt[1];
            }
            if (LL) *LL = Mat(npl, npl);
            if (RR) *RR = Mat(npl, npl);
            if (RL) *RL = Mat(npl, npl);
            for (int a = 0; a < P; ++a)
                for (int c = 0; c < P; ++c) {
                    double m = T.mass[(size_t)a * P + c] * area;
                    if (LL) (*LL)(jl[a], jl[c]) = m;
                    if (RR) (*RR)(jr[a], jr[c]) = m;
                    if (RL) (*RL)(jr[a], jl[c]) = m;
                }
        } else {
            Mat phl(QF, npl), phr(QF, npl);
            std::vector<double> w(QF);
            for (int q = 0; q < QF; ++q) {
                double ql[2], qr[2];
                if (f.canonical) {
                    int kk = 0 + (0 >= f.dim);
                    ql[kk] = qx[q];
                    qr[kk] = qx[q];
                    ql[f.dim] = (f.normal > 0) ? 1 : 0;
                    qr[f.dim] = (f.normal > 0) ? 0 : 1;
                } else {
                    ql[0] = f.xl[q][0]; ql[1] = f.xl[q][1];
                    qr[0] = f.xr[q][0]; qr[1] = f.xr[q][1];
                }
                lagrange2(P, ql, &phl(q, 0));
                lagrange2(P, qr, &phr(q, 0));
                w[q] = 1;
                w[q] *= qw[q];
            }
            double area = f.area();
            for (int q = 0; q < QF; ++q) w[q] *= area;
            Mat Lm(npl, QF), Rm(npl, QF);
            for (int a = 0; a < npl; ++a)
                for (int q = 0; q < QF; ++q) {
                    Lm(a, q) = phl(q, a) * w[q];
                    Rm(a, q) = phr(q, a) * w[q];
                }
            if (L) *L = Lm;
            if (R) *R = Rm;
            if (LL) *LL = matmul(Lm, phl);
            if (RR) *RR = matmul(Rm, phr);
            if (RL) *RL = matmul(Rm, phl);
        }
    }
};

// ---------------------------------------------------------- LDG operators --
// LDGOperators<N,P> (ldgpoisson.h:15-53)
struct Ops {
    SBM M, G[3], T, A;
    int ndim = NDIM;   // 3 for tetrahedral meshes
    std::vector<LDLT> Minv;
    bool has_MGT = false;
    // construct_laplacian (ldgpoisson.h:34-52): A = T + sum_d G_d^T M G_d
    void construct_laplacian() {
        A = T;
        for (int d = 0; d < ndim; ++d) {
            for (int k = 0; k < M.blockRows(); ++k) {
                const auto& cols = G[d].colsInRow(k);
                for (int i : cols) {
                    Mat GT_M = matmul_tn(G[d].get(k, i), M.get(k, k));
                    for (int j : cols) A.add(i, j, matmul(GT_M, G[d].get(k, j)));
                }
            }
        }
    }
};

enum BCType { kDirichlet = 0, kNeumann = 1, kPeriodic = 2 };

struct Problem {
    int P, npl;
    std::unique_ptr<Quadtree> qt;
    std::unique_ptr<Mesh> mesh;
    std::shared_ptr<Ops> ops;
    int bctype;
    std::function<double(const double*)> bcfun;   // boundary value
    double tau0, tauD;
    bool tau_per_face = false;   // extension: tau0 / min(h_L, h_R), tauD / h_L
    std::vector<double> rhs, utrue;
    std::vector<std::vector<Mat>> Tl;   // unused placeholder
    std::vector<SBM> hier;             // InterpolationHierarchy<2,P>::T
    // simplex meshes (no quadtree / Cartesian mesh)
    bool simplex = false;
    int s_ne = 0, s_nf = 0, s_nb = 0;
    std::vector<std::vector<int>> agg;   // per agglomeration level: aggregate of each finer element
    struct AggQuality {
        int n;
        double mean_ratio, max_ratio;
    };
    std::vector<AggQuality> agg_quality;   // per agglomeration level
    std::vector<double> s_xy;            // node coordinates (s_dim per DOF) in DOF order
    int s_dim = 2;
};

// LDGPoisson<N,P>::discretize (ldgpoisson.tpp:14-24) and its parts
static void discretize(Problem& pr, std::vector<double>& rhs) {
    const Mesh& mesh = *pr.mesh;
    Ops& ops = *pr.ops;
    int ne = (int)mesh.elements.size(), npl = pr.npl, P = pr.P;
    ops.M = SBM(ne, ne, npl, npl);
    ops.T = SBM(ne, ne, npl, npl);
    for (int d = 0; d < NDIM; ++d) ops.G[d] = SBM(ne, ne, npl, npl);
    std::vector<double> Jg[2];
    for (int d = 0; d < NDIM; ++d) Jg[d].assign((size_t)ne * npl, 0.0);
    rhs.assign((size_t)ne * npl, 0.0);

    // construct_mass_matrix (ldgpoisson.tpp:27-39)
    for (int e = 0; e < ne; ++e) {
        Mat Me = mesh.mass(e);
        ops.M.set(e, e, Me);
        ops.Minv.emplace_back(Me);
    }
    // construct_broken_gradient (ldgpoisson.tpp:42-60)
    for (int i = 0; i < NDIM; ++i) {
        Mat diff = master_diff(P, i);
        for (int e = 0; e < ne; ++e) {
            double jac = 1.0 / mesh.elements[e].width(i);
            ops.G[i].add(e, e, scaled(jac, diff));
        }
    }
    // construct_lifting_terms (ldgpoisson.tpp:63-100)
    for (const Face& f : mesh.faces) {
        Mat LL, RR, RL;
        mesh.lift(f, nullptr, nullptr, &LL, &RR, &RL);
        double n = f.normal;
        if (f.interiorQ()) {
            Mat MinvR = mesh.invmass(f.right);
            ops.G[f.dim].add(f.right, f.right, matmul(scaled(n, MinvR), RR));
            ops.G[f.dim].add(f.right, f.left, matmul(scaled(-n, MinvR), RL));
            double tau = pr.tau0;
            if (pr.tau_per_face)
                tau = pr.tau0 / std::min(mesh.elements[f.left].width(0), mesh.elements[f.right].width(0));
            ops.T.add(f.right, f.right, scaled(tau, RR));
            ops.T.add(f.left, f.left, scaled(tau, LL));
            ops.T.add(f.right, f.left, scaled(-tau, RL));
            ops.T.add(f.left, f.right, scaled(-tau, transpose(RL)));
        } else if (pr.bctype == kDirichlet) {
            Mat MinvL = mesh.invmass(f.left);
            ops.G[f.dim].add(f.left, f.left, matmul(scaled(-n, MinvL), LL));
            double tauD = pr.tau_per_face ? pr.tauD / mesh.elements[f.left].width(0) : pr.tauD;
            ops.T.add(f.left, f.left, scaled(tauD, LL));
        }
    }
    ops.construct_laplacian();
    ops.has_MGT = true;

    // add_source_terms (ldgpoisson.tpp:103-161)
    for (const Face& f : mesh.faces) {
        if (!f.boundaryQ()) continue;
        Mat L;
        mesh.lift(f, &L, nullptr, nullptr, nullptr, nullptr);
        double n = f.normal;
        std::vector<double> bc(QF);
        for (int q = 0; q < QF; ++q) {
            double xq[2];
            int kk = 0 + (0 >= f.dim);
            xq[kk] = f.cell.lo[kk] + f.cell.width(kk) * mesh.qx[q];
            xq[f.dim] = f.cell.lo[f.dim];
            bc[q] = pr.bcfun(xq);
        }
        std::vector<double> Lbc(npl, 0.0);
        for (int a = 0; a < npl; ++a) {
            double s = 0;
            for (int q = 0; q < QF; ++q) s += L(a, q) * bc[q];
            Lbc[a] = s;
        }
        if (pr.bctype == kDirichlet) {
            for (int a = 0; a < npl; ++a) {
                Jg[f.dim][(size_t)npl * f.left + a] += n * Lbc[a];
                rhs[(size_t)npl * f.left + a] +=
                    (pr.tau_per_face ? pr.tauD / mesh.elements[f.left].width(0) : pr.tauD) * Lbc[a];
            }
        } else if (pr.bctype == kNeumann) {
            for (int a = 0; a < npl; ++a) rhs[(size_t)npl * f.left + a] += Lbc[a];
        } else {
            throw std::invalid_argument("Unknown boundary condition.");
        }
    }
    for (int e = 0; e < ne; ++e) {
        for (int d = 0; d < NDIM; ++d) {
            for (int i : ops.G[d].rowsInCol(e)) {
                const Mat& B = ops.G[d].get(i, e);
                const double* jg = Jg[d].data() + (size_t)npl * i;
                for (int c = 0; c < npl; ++c) {
                    double s = 0;
                    for (int r = 0; r < npl; ++r) s += B(r, c) * jg[r];
                    rhs[(size_t)npl * e + c] -= s;
                }
            }
        }
    }
}

// InterpolationHierarchy<N,P> (interpolationhierarchy.h:30-82), for any
// degree P on the problem's quadtree
static std::vector<SBM> h_hierarchy(const Quadtree& qt, int P) {
    std::vector<SBM> out;
    int npl = P * P;
    const Tables& T = tables(P);
    for (int l = 0; l < qt.numLevels - 1; ++l) {
        std::vector<int> fine = qt.layer(l), coarse = qt.layer(l + 1);
        std::unordered_map<int, int> cg2l;
        int clid = 0;
        for (int g : coarse) cg2l[g] = clid++;
        out.emplace_back((int)fine.size(), (int)coarse.size(), npl, npl);
        SBM& Tm = out.back();
        int flid = 0;
        for (int fg : fine) {
            if (qt.isLeaf(qt.tree[fg], l + 1)) {
                Tm.set(flid, cg2l[fg], identity(npl));
                flid++;
            } else {
                int cg = qt.tree[fg].parent;
                const Cell& fc = qt.tree[fg].cell;
                const Cell& cc = qt.tree[cg].cell;
                Cell rel;
                for (int i = 0; i < NDIM; ++i) {
                    rel.lo[i] = (fc.lo[i] - cc.lo[i]) / cc.width(i);
                    rel.hi[i] = (fc.hi[i] - cc.lo[i]) / cc.width(i);
                }
                Mat E(npl, npl);
                for (int i0 = 0; i0 < P; ++i0)
                    for (int i1 = 0; i1 < P; ++i1) {
                        double node[2];
                        int idx[2] = {i0, i1};
                        for (int i = 0; i < NDIM; ++i)
                            node[i] = rel.lo[i] + rel.width(i) * T.nodes[idx[i]];
                        lagrange2(P, node, &E(i0 * P + i1, 0));
                    }
                Tm.set(flid++, cg2l[cg], E);
            }
        }
    }
    return out;
}

static void build_hierarchy(Problem& pr) { pr.hier = h_hierarchy(*pr.qt, pr.P); }

// p-interpolation from degree P2 to degree P1 on the same elements
// (InterpolationHierarchy<N,P1,P2>, interpolationhierarchy.h:109-129): the
// block-diagonal operator whose block evaluates the P2 Lagrange basis at the
// P1 nodes of the master element
static SBM p_transfer(int ne, int P1, int P2) {
    int b1 = P1 * P1, b2 = P2 * P2;
    const Tables& T1 = tables(P1);
    Mat E(b1, b2);
    for (int i0 = 0; i0 < P1; ++i0)
        for (int i1 = 0; i1 < P1; ++i1) {
            double node[2] = {T1.nodes[i0], T1.nodes[i1]};
            lagrange2(P2, node, &E(i0 * P1 + i1, 0));
        }
    SBM Tm(ne, ne, b1, b2);
    for (int i = 0; i < ne; ++i) Tm.set(i, i, E);
    return Tm;
}

// Gaussian-sum forcing: 8 Gaussians, centres U[0,1]^2, widths U[0.05,0.2],
// amplitudes N(0,1); mt19937_64 with 53-bit uniforms and Box-Muller normals.
struct Gauss8 { double cx[8], cy[8], w[8], a[8]; };
static Gauss8 gaussian_params(uint64_t seed) {
    std::mt19937_64 g(seed);
    auto uni = [&]() { return (double)(g() >> 11) * 0x1.0p-53; };
    Gauss8 p;
    for (int k = 0; k < 8; ++k) {
        p.cx[k] = uni();
        p.cy[k] = uni();
        p.w[k] = 0.05 + 0.15 * uni();
        double u1;
        do { u1 = uni(); } while (u1 <= 0.0);
        double u2 = uni();
        p.a[k] = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
    }
    return p;
}
static double gaussian_eval(const Gauss8& p, const double* x) {
    double s = 0;
    for (int k = 0; k < 8; ++k) {
        double dx = x[0] - p.cx[k], dy = x[1] - p.cy[k];
        s += p.a[k] * std::exp(-(dx * dx + dy * dy) / (2.0 * p.w[k] * p.w[k]));
    }
    return s;
}

// Function<N,P> nodal interpolant (function.h:42-53)
static std::vector<double> interpolate(const Mesh& mesh, const std::function<double(const double*)>& f) {
    int P = mesh.P, npl = mesh.npl;
    const Tables& T = tables(P);
    std::vector<double> v((size_t)mesh.elements.size() * npl);
    for (size_t e = 0; e < mesh.elements.size(); ++e) {
        const Cell& c = mesh.elements[e];
        for (int i0 = 0; i0 < P; ++i0)
            for (int i1 = 0; i1 < P; ++i1) {
                double x[2] = {c.lo[0] + c.width(0) * T.nodes[i0], c.lo[1] + c.width(1) * T.nodes[i1]};
                v[e * npl + i0 * P + i1] = f(x);
            }
    }
    return v;
}

static Problem* problem_create_h(int P, const std::function<double(const double*)>& h, int balance,
                                 int tau_per_face, int coarsening, int bctype, int test, double tau0,
                                 double tauD, uint64_t seed);

static Problem* problem_create(int P, double dx, int refine, int coarsening, int bctype, int test,
                               double tau0, double tauD, uint64_t seed) {
    std::function<double(const double*)> h;
    if (refine == ORC_REFINE_UNIFORM) {
        h = [dx](const double*) { return dx; };
    } else {
        // h_adaptive (dg_tests.cpp:212-215)
        h = [dx](const double* x) { return (x[0] > 0.5) ? dx : (x[0] > 0.25) ? 0.25 * dx : 0.5 * dx; };
    }
    return problem_create_h(P, h, 0, 0, coarsening, bctype, test, tau0, tauD, seed);
}

// Seeded points: mt19937_64 with 53-bit uniforms, (x, y) pairs.
static std::vector<double> seeded_points(uint64_t seed, int n) {
    std::mt19937_64 g(seed);
    std::vector<double> p(2 * (size_t)n);
    for (auto& v : p) v = (double)(g() >> 11) * 0x1.0p-53;
    return p;
}

// Mesh size of the seeded-points refinement: a cell of width
// w = 2^-(base + l) is split while l < extra and its centre lies within
// radius * 2^-l of a point; as an h(x) callback (split iff w > h(centre)):
// h = min(2^-base, max(2^-(base+extra), d / (radius 2^base))).
static double points_h(const std::vector<double>& pts, int base, int extra, double radius, const double* x) {
    double d = 1e300;
    for (size_t k = 0; k + 1 < pts.size(); k += 2) {
        const double dx = x[0] - pts[k], dy = x[1] - pts[k + 1];
        d = std::min(d, std::sqrt(dx * dx + dy * dy));
    }
    const double lo = std::ldexp(1.0, -(base + extra)), hi = std::ldexp(1.0, -base);
    return std::min(hi, std::max(lo, d / (radius * std::ldexp(1.0, base))));
}

static Problem* problem_create_h(int P, const std::function<double(const double*)>& h, int balance,
                                 int tau_per_face, int coarsening, int bctype, int test, double tau0,
                                 double tauD, uint64_t seed) {
    std::unique_ptr<Problem> pr(new Problem());
    pr->P = P; pr->npl = P * P; pr->bctype = bctype; pr->tau0 = tau0; pr->tauD = tauD;
    pr->tau_per_face = tau_per_face != 0;
    pr->qt.reset(new Quadtree(h, coarsening, bctype == kPeriodic));
    if (balance) pr->qt->balance();
    pr->mesh.reset(new Mesh(*pr->qt, P));
    pr->ops = std::make_shared<Ops>();
    const double PI = 3.14159265358979323846;
    std::function<double(const double*)> ufun, ffun;
    pr->bcfun = [](const double*) { return 0.0; };
    if (test == ORC_TEST_SOLUTION) {
        // dg_tests.cpp:232-254
        if (bctype == kDirichlet) {
            ufun = [PI](const double* x) { return std::cos(2 * PI * x[0]) * std::cos(2 * PI * x[1]) + x[0] + x[1]; };
            ffun = [PI](const double* x) { return 8 * PI * PI * std::cos(2 * PI * x[0]) * std::cos(2 * PI * x[1]); };
            pr->bcfun = ufun;
        } else if (bctype == kNeumann) {
            ufun = [PI](const double* x) { return std::cos(2 * PI * x[0]) * std::cos(2 * PI * x[1]) + x[0] * (1 - x[0]) + x[1] * (1 - x[1]); };
            ffun = [PI](const double* x) { return 8 * PI * PI * std::cos(2 * PI * x[0]) * std::cos(2 * PI * x[1]) + 4.0; };
            pr->bcfun = [](const double*) { return -1.0; };
        } else {
            ufun = [PI](const double* x) { return std::sin(2 * PI * x[0]) * std::sin(2 * PI * x[1]); };
            ffun = [PI](const double* x) { return 8 * PI * PI * std::sin(2 * PI * x[0]) * std::sin(2 * PI * x[1]); };
        }
    } else if (test == ORC_TEST_GAUSSIAN) {
        Gauss8 gp = gaussian_params(seed);
        ffun = [gp](const double* x) { return gaussian_eval(gp, x); };
        ufun = [](const double*) { return 0.0; };
    } else {
        ffun = [](const double*) { return 0.0; };
        ufun = [](const double*) { return 0.0; };
    }
    std::vector<double> rhs_bc;
    discretize(*pr, rhs_bc);
    // computeRHS (ldgpoisson.tpp:167-176)
    std::vector<double> fv = interpolate(*pr->mesh, ffun);
    int ne = (int)pr->mesh->elements.size(), npl = pr->npl;
    pr->rhs.assign((size_t)ne * npl, 0.0);
    for (int e = 0; e < ne; ++e) {
        const Mat& Me = pr->ops->M.get(e, e);
        for (int r = 0; r < npl; ++r) {
            double s = 0;
            for (int c = 0; c < npl; ++c) s += Me(r, c) * fv[(size_t)e * npl + c];
            pr->rhs[(size_t)e * npl + r] = rhs_bc[(size_t)e * npl + r] + s;
        }
    }
    // meanZero for Neumann / periodic (dg_tests.cpp:283-286, function.h:154-167)
    if (bctype == kNeumann || bctype == kPeriodic) {
        double mean = 0;
        for (double v : pr->rhs) mean += v;
        mean /= (double)pr->rhs.size();
        for (double& v : pr->rhs) v -= mean;
    }
    pr->utrue = interpolate(*pr->mesh, ufun);
    if (pr->qt->numLevels > 1) build_hierarchy(*pr);
    return pr.release();
}

// ------------------------------------------------------------ multigrid --
// Level<N,P> and Multigrid<N,P> (multigrid.h:65-433)
struct Level {
    std::shared_ptr<Ops> ops;
    std::vector<LDLT> Dinv;
    std::vector<double> x, b, r;
    int npl = 0;
    // dense Cholesky of the whole level matrix (coarsest-level extension)
    std::vector<double> chol;
    std::vector<char> absent;   // unknowns with zero rows and columns (dense solve)
    int nchol = 0;
};

struct MG {
    int relaxation, solver, npre, npost, restriction;
    double omega;
    bool mean_project;
    const Problem* pr;
    std::vector<std::unique_ptr<Level>> levels;
    std::vector<SBM> Ts;   // Ts[i] interpolates level i+1 to level i

    // Level(fineOps) (multigrid.h:83-96)
    void fine_level(std::shared_ptr<Ops> ops) {
        std::unique_ptr<Level> L(new Level());
        L->ops = ops;
        L->npl = ops->A.P;
        L->x.assign(ops->A.cols(), 0.0);
        L->b.assign(ops->A.cols(), 0.0);
        L->r.assign(ops->A.cols(), 0.0);
        for (int i = 0; i < ops->A.blockRows(); ++i) L->Dinv.emplace_back(ops->A.get(i, i));
        levels.push_back(std::move(L));
    }
    // Level(fineOps, T) (multigrid.h:105-171)
    void coarse_level(const Ops& f, const SBM& T) {
        std::unique_ptr<Level> L(new Level());
        L->ops = std::make_shared<Ops>();
        Ops& o = *L->ops;
        int npl = T.Q;
        L->npl = npl;
        L->x.assign(T.cols(), 0.0);
        L->b.assign(T.cols(), 0.0);
        L->r.assign(T.cols(), 0.0);
        if (restriction == ORC_RESTRICT_RATRAT) {
            if (!f.has_MGT) throw std::invalid_argument("RATRAT needs M, G, T on the finer level");
            o.M = SBM(T.blockCols(), T.blockCols(), npl, npl);
            for (int k = 0; k < f.M.blockRows(); ++k) {
                const auto& cols = T.colsInRow(k);
                for (int i : cols) {
                    Mat TT_M = matmul_tn(T.get(k, i), f.M.get(k, k));
                    for (int j : cols) o.M.add(i, j, matmul(TT_M, T.get(k, j)));
                }
            }
            for (int i = 0; i < o.M.blockRows(); ++i) o.Minv.emplace_back(o.M.get(i, i));
            SBM temp1, temp2;
            o.ndim = f.ndim;
            for (int d = 0; d < f.ndim; ++d) {
                multiply_mm(f.G[d], T, temp1);
                multiply_mm(f.M, temp1, temp2);
                multiply_mm_t(T, temp2, o.G[d]);
                for (int i = 0; i < o.M.blockRows(); ++i) {
                    const auto& cols = o.G[d].colsInRow(i);
                    for (int j : cols) o.G[d].set(i, j, o.Minv[i].solve(o.G[d].get(i, j)));
                }
            }
            multiply_mm(f.T, T, temp1);
            multiply_mm_t(T, temp1, o.T);
            o.construct_laplacian();
            o.has_MGT = true;
        } else if (restriction == ORC_RESTRICT_RAT) {
            SBM temp1;
            multiply_mm(f.A, T, temp1);
            multiply_mm_t(T, temp1, o.A);
        } else {
            throw std::invalid_argument("Unknown restriction method.");
        }
        for (int i = 0; i < o.A.blockRows(); ++i) L->Dinv.emplace_back(o.A.get(i, i));
        levels.push_back(std::move(L));
    }
    void dense_factor(Level& L) {
        const SBM& A = L.ops->A;
        int n = A.rows(), b = A.P;
        L.nchol = n;
        std::vector<double> D((size_t)n * n, 0.0);
        for (const auto& kv : A.map)
            for (int r = 0; r < b; ++r)
                for (int c = 0; c < b; ++c)
                    D[(size_t)(kv.first.i * b + r) * n + kv.first.j * b + c] = kv.second(r, c);
        // unknowns with exactly zero rows and columns are absent (unit
        // diagonal, zero solution), as in LDLT
        L.absent.assign(n, 0);
        for (int i = 0; i < n; ++i) {
            bool z = true;
            for (int j = 0; j < n && z; ++j) z = D[(size_t)i * n + j] == 0.0 && D[(size_t)j * n + i] == 0.0;
            if (z) {
                L.absent[i] = 1;
                D[(size_t)i * n + i] = 1.0;
            }
        }
        for (int j = 0; j < n; ++j) {
            double s = D[(size_t)j * n + j];
            for (int k = 0; k < j; ++k) s -= D[(size_t)j * n + k] * D[(size_t)j * n + k];
            if (!(s > 0)) throw std::runtime_error("coarse matrix not SPD");
            double ljj = std::sqrt(s);
            D[(size_t)j * n + j] = ljj;
            for (int i = j + 1; i < n; ++i) {
                double t = D[(size_t)i * n + j];
                for (int k = 0; k < j; ++k) t -= D[(size_t)i * n + k] * D[(size_t)j * n + k];
                D[(size_t)i * n + j] = t / ljj;
            }
        }
        L.chol.swap(D);
    }

    void computeResidual(Level& L) {   // multigrid.h:174-178
        L.r = L.b;
        multiply_add_mv(-1.0, L.ops->A, L.x.data(), 1.0, L.r.data());
    }
    void jacobi(Level& L) {             // multigrid.h:223-229
        computeResidual(L);
        int npl = L.npl;
        for (int i = 0; i < L.ops->A.blockRows(); ++i) {
            std::vector<double> z = L.Dinv[i].solve(L.r.data() + (size_t)npl * i);
            for (int a = 0; a < npl; ++a) L.x[(size_t)npl * i + a] += omega * z[a];
        }
    }
    void gs_row(Level& L, int i, std::vector<double>& temp) {
        int npl = L.npl;
        const SBM& A = L.ops->A;
        std::fill(temp.begin(), temp.end(), 0.0);
        for (int j : A.colsInRow(i)) {
            if (j == i) continue;
            const Mat& B = A.get(i, j);
            const double* xj = L.x.data() + (size_t)npl * j;
            for (int r = 0; r < npl; ++r) {
                double s = 0;
                for (int c = 0; c < npl; ++c) s += B(r, c) * xj[c];
                temp[r] += s;
            }
        }
        std::vector<double> t(npl);
        for (int a = 0; a < npl; ++a) t[a] = L.b[(size_t)npl * i + a] - temp[a];
        L.Dinv[i].solve_inplace(t.data());
        for (int a = 0; a < npl; ++a) {
            double& xi = L.x[(size_t)npl * i + a];
            xi += omega * (t[a] - xi);
        }
    }
    void gauss_seidel(Level& L, bool reverse) {   // multigrid.h:236-262
        std::vector<double> temp(L.npl);
        int nb = L.ops->A.blockRows();
        if (!reverse) for (int i = 0; i < nb; ++i) gs_row(L, i, temp);
        else for (int i = nb - 1; i >= 0; --i) gs_row(L, i, temp);
    }
    void relax(Level& L, int n, bool reverse) {   // multigrid.h:202-216
        for (int i = 0; i < n; ++i) {
            if (relaxation == ORC_RELAX_JACOBI) jacobi(L);
            else if (relaxation == ORC_RELAX_GS) gauss_seidel(L, reverse);
            else throw std::invalid_argument("Unknown relaxation method.");
        }
    }
    void solve(Level& L) {   // multigrid.h:181-195 (+ dense Cholesky extension)
        if (solver == ORC_COARSE_RELAX) {
            relax(L, npre, false);
            relax(L, npost, true);
        } else if (solver == ORC_COARSE_CHOLESKY) {
            if (L.ops->A.blockRows() != 1) throw std::invalid_argument("Cholesky coarse solve needs one element");
            L.x = L.Dinv[0].solve(L.b.data());
        } else if (solver == ORC_COARSE_DENSE) {
            int n = L.nchol;
            std::vector<double> y(L.b);
            for (int i = 0; i < n; ++i) {
                double s = y[i];
                for (int k = 0; k < i; ++k) s -= L.chol[(size_t)i * n + k] * y[k];
                y[i] = s / L.chol[(size_t)i * n + i];
            }
            for (int i = n - 1; i >= 0; --i) {
                double s = y[i];
                for (int k = i + 1; k < n; ++k) s -= L.chol[(size_t)k * n + i] * y[k];
                y[i] = s / L.chol[(size_t)i * n + i];
            }
            for (int i = 0; i < n; ++i)
                if (L.absent[i]) y[i] = 0.0;
            L.x = y;
        } else {
            throw std::invalid_argument("Unknown coarse solver.");
        }
    }
    void vcycle(int i) {   // multigrid.h:361-383
        Level& L = *levels[i];
        if (i == (int)levels.size() - 1) {
            if (mean_project) {
                double mean = 0;
                for (double v : L.b) mean += v;
                mean /= (double)L.b.size();
                for (double& v : L.b) v -= mean;
            }
            solve(L);
        } else {
            relax(L, npre, false);
            computeResidual(L);
            Level& C = *levels[i + 1];
            multiply_mv_t(Ts[i], L.r.data(), C.b.data());   // restrictResidual :414-418
            std::fill(C.x.begin(), C.x.end(), 0.0);
            vcycle(i + 1);
            multiply_add_mv(1.0, Ts[i], C.x.data(), 1.0, L.x.data());   // correctSolution :421-425
            relax(L, npost, true);
        }
    }
};

static double dot(const std::vector<double>& a, const std::vector<double>& b) {
    double s = 0;
    for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
}

// pcg (krylov.h:22-68)
static int pcg(const SBM& A, const std::vector<double>& b, std::vector<double>& x,
               const std::function<std::vector<double>(const std::vector<double>&)>& precon,
               double tol, int maxit, double* hist, double* dhist) {
    size_t n = b.size();
    std::vector<double> r(b), d, q(n), s;
    multiply_add_mv(-1.0, A, x.data(), 1.0, r.data());
    d = precon(r);
    double delta_new = dot(r, d), delta_0 = delta_new, delta_old, alpha, beta;
    int i = 0;
    while (i < maxit && delta_new > tol * tol * delta_0) {
        multiply_mv(A, d.data(), q.data());
        alpha = delta_new / dot(d, q);
        for (size_t k = 0; k < n; ++k) x[k] += alpha * d[k];
        if (i % 50 == 0) {
            r = b;
            multiply_add_mv(-1.0, A, x.data(), 1.0, r.data());
        } else {
            for (size_t k = 0; k < n; ++k) r[k] -= alpha * q[k];
        }
        s = precon(r);
        delta_old = delta_new;
        delta_new = dot(r, s);
        beta = delta_new / delta_old;
        for (size_t k = 0; k < n; ++k) d[k] = s[k] + beta * d[k];
        if (hist) hist[i] = std::sqrt(dot(r, r));
        if (dhist) dhist[i] = delta_new;
        ++i;
    }
    return i;
}

static const SBM& op_of(const Ops& o, int which) {
    switch (which) {
        case 0: return o.M;
        case 1: return o.G[0];
        case 2: return o.G[1];
        case 3: return o.T;
        case 4: return o.A;
        case 5: if (o.ndim > 2) return o.G[2]; break;
    }
    throw std::invalid_argument("bad operator id");
}

static void export_csr(const SBM& A, int* row_ptr, int* col_idx, double* vals) {
    long pos = 0;
    size_t bs = (size_t)A.P * A.Q;
    for (int i = 0; i < A.blockRows(); ++i) {
        if (row_ptr) row_ptr[i] = (int)pos;
        std::vector<int> cols(A.colsInRow(i).begin(), A.colsInRow(i).end());
        std::sort(cols.begin(), cols.end());
        for (int j : cols) {
            if (col_idx) col_idx[pos] = j;
            if (vals) std::memcpy(vals + pos * bs, A.get(i, j).a.data(), bs * sizeof(double));
            ++pos;
        }
    }
    if (row_ptr) row_ptr[A.blockRows()] = (int)pos;
}

}  // namespace orc

// =================================================================== C API ==
using namespace orc;

struct orc_problem { Problem* p; };
struct orc_mg { MG* m; };
struct orc_sbm { SBM s; };

#define ORC_TRY(...) try { __VA_ARGS__; return 0; } catch (...) { return 1; }

#include "unstructured.inc"

extern "C" {

int orc_master_tables(int P, double* nodes, double* denom, double* mass, double* invmass, double* diff) {
    ORC_TRY({
        const Tables& T = tables(P);
        if (nodes) std::memcpy(nodes, T.nodes.data(), P * sizeof(double));
        if (denom) std::memcpy(denom, T.denom.data(), P * sizeof(double));
        if (mass) std::memcpy(mass, T.mass.data(), (size_t)P * P * sizeof(double));
        if (invmass) std::memcpy(invmass, T.invmass.data(), (size_t)P * P * sizeof(double));
        if (diff) std::memcpy(diff, T.diff.data(), (size_t)P * P * sizeof(double));
    })
}

int orc_quadrature(int Q, double* nodes, double* weights) {
    ORC_TRY({
        if (Q < 1 || Q > 12) throw std::invalid_argument("Q");
        std::vector<double> x, w;
        quadrature(Q, x, w);
        std::memcpy(nodes, x.data(), Q * sizeof(double));
        std::memcpy(weights, w.data(), Q * sizeof(double));
    })
}

int orc_sbm_create(int m, int n, int P, int Q, orc_sbm** out) {
    ORC_TRY({ *out = new orc_sbm{SBM(m, n, P, Q)}; })
}
int orc_sbm_set_block(orc_sbm* A, int i, int j, const double* blk) {
    ORC_TRY({
        Mat B(A->s.P, A->s.Q);
        std::memcpy(B.a.data(), blk, B.a.size() * sizeof(double));
        A->s.set(i, j, B);
    })
}
int orc_sbm_add_block(orc_sbm* A, int i, int j, const double* blk) {
    ORC_TRY({
        Mat B(A->s.P, A->s.Q);
        std::memcpy(B.a.data(), blk, B.a.size() * sizeof(double));
        A->s.add(i, j, B);
    })
}
int orc_sbm_mv(const orc_sbm* A, double alpha, const double* x, double beta, double* y) {
    ORC_TRY({ multiply_add_mv(alpha, A->s, x, beta, y); })
}
int orc_sbm_mv_t(const orc_sbm* A, const double* x, double* y) {
    ORC_TRY({ multiply_mv_t(A->s, x, y); })
}
int orc_sbm_destroy(orc_sbm* A) { delete A; return 0; }

int orc_problem_create(int P, double dx, int refine, int coarsening, int bctype, int test,
                       double tau0, double tauD, uint64_t seed, orc_problem** out) {
    ORC_TRY({
        *out = new orc_problem{problem_create(P, dx, refine, coarsening, bctype, test, tau0, tauD, seed)};
    })
}
int orc_problem_create_points(int P, int base_level, int extra_levels, int npoints, uint64_t point_seed,
                              double radius, int balance, int tau_per_face, double tau0, double tauD,
                              uint64_t rhs_seed, orc_problem** out) {
    ORC_TRY({
        if (base_level < 0 || extra_levels < 0 || base_level + extra_levels > 20 || npoints < 1 || !(radius > 0))
            throw std::invalid_argument("bad points rule");
        std::vector<double> pts = seeded_points(point_seed, npoints);
        std::function<double(const double*)> h = [pts, base_level, extra_levels, radius](const double* x) {
            return points_h(pts, base_level, extra_levels, radius, x);
        };
        *out = new orc_problem{problem_create_h(P, h, balance, tau_per_face, ORC_COARSEN_EQUAL, kDirichlet,
                                                ORC_TEST_GAUSSIAN, tau0, tauD, rhs_seed)};
    })
}
int orc_seeded_points(uint64_t seed, int n, double* xy) {
    ORC_TRY({
        std::vector<double> p = seeded_points(seed, n);
        std::copy(p.begin(), p.end(), xy);
    })
}
int orc_problem_destroy(orc_problem* pr) {
    if (pr) { delete pr->p; delete pr; }
    return 0;
}
int orc_problem_info(const orc_problem* pr, int* ne, int* npl, int* ndof, int* nlevels, int* nfaces,
                     int* nbfaces) {
    ORC_TRY({
        const Problem& p = *pr->p;
        int e = p.simplex ? p.s_ne : (int)p.mesh->elements.size();
        if (ne) *ne = e;
        if (npl) *npl = p.npl;
        if (ndof) *ndof = e * p.npl;
        if (nlevels) *nlevels = p.simplex ? (int)p.hier.size() + 1 : p.qt->numLevels;
        if (nfaces) *nfaces = p.simplex ? p.s_nf : (int)p.mesh->faces.size();
        if (nbfaces) *nbfaces = p.simplex ? p.s_nb : p.mesh->nb;
    })
}
int orc_problem_elements(const orc_problem* pr, double* lower, double* upper) {
    ORC_TRY({
        const auto& el = pr->p->mesh->elements;
        for (size_t e = 0; e < el.size(); ++e)
            for (int d = 0; d < NDIM; ++d) {
                lower[e * NDIM + d] = el[e].lo[d];
                upper[e * NDIM + d] = el[e].hi[d];
            }
    })
}
int orc_problem_nnzb(const orc_problem* pr, int which, int* nnzb) {
    ORC_TRY({ *nnzb = (int)op_of(*pr->p->ops, which).nnzb(); })
}
int orc_problem_export(const orc_problem* pr, int which, int* row_ptr, int* col_idx, double* vals) {
    ORC_TRY({ export_csr(op_of(*pr->p->ops, which), row_ptr, col_idx, vals); })
}
int orc_problem_rhs(const orc_problem* pr, double* b) {
    ORC_TRY({ std::memcpy(b, pr->p->rhs.data(), pr->p->rhs.size() * sizeof(double)); })
}
int orc_problem_utrue(const orc_problem* pr, double* u) {
    ORC_TRY({ std::memcpy(u, pr->p->utrue.data(), pr->p->utrue.size() * sizeof(double)); })
}
int orc_hier_size(const orc_problem* pr, int* nT) {
    ORC_TRY({ *nT = (int)pr->p->hier.size(); })
}
int orc_hier_shape(const orc_problem* pr, int l, int* nbr, int* nbc, int* nnzb) {
    ORC_TRY({
        const SBM& T = pr->p->hier.at(l);
        if (nbr) *nbr = T.blockRows();
        if (nbc) *nbc = T.blockCols();
        if (nnzb) *nnzb = (int)T.nnzb();
    })
}
int orc_hier_export(const orc_problem* pr, int l, int* row_ptr, int* col_idx, double* vals) {
    ORC_TRY({ export_csr(pr->p->hier.at(l), row_ptr, col_idx, vals); })
}
int orc_gaussian_params(uint64_t seed, double* cx, double* cy, double* w, double* a) {
    ORC_TRY({
        Gauss8 g = gaussian_params(seed);
        std::memcpy(cx, g.cx, sizeof g.cx);
        std::memcpy(cy, g.cy, sizeof g.cy);
        std::memcpy(w, g.w, sizeof g.w);
        std::memcpy(a, g.a, sizeof g.a);
    })
}

int orc_mg_create(const orc_problem* pr, int relaxation, double omega, int solver, int npre, int npost,
                  int restriction, int nlevels, int mean_project, orc_mg** out) {
    ORC_TRY({
        std::unique_ptr<MG> m(new MG());
        m->relaxation = relaxation; m->omega = omega; m->solver = solver;
        m->npre = npre; m->npost = npost; m->restriction = restriction;
        m->mean_project = mean_project != 0;
        m->pr = pr->p;
        m->fine_level(pr->p->ops);
        int nT = (int)pr->p->hier.size();
        int use = (nlevels <= 0) ? nT : std::min(nT, nlevels - 1);
        for (int i = 0; i < use; ++i) m->Ts.push_back(pr->p->hier[i]);
        for (int i = 0; i < use; ++i) m->coarse_level(*m->levels[i]->ops, m->Ts[i]);
        if (solver == ORC_COARSE_DENSE) m->dense_factor(*m->levels.back());
        *out = new orc_mg{m.release()};
    })
}

// hp-multigrid (Multigrid<N,P1,P2,...>, multigrid.h:436-560): p-levels
// degrees[0] (the problem's P) -> degrees[1] -> ... on the fine mesh, then
// nh h-levels at the last degree (InterpolationHierarchy<N,Pk>)
int orc_mg_create_hp(const orc_problem* pr, const int* degrees, int ndeg, int nh, int relaxation, double omega,
                     int solver, int npre, int npost, int restriction, int mean_project, orc_mg** out) {
    ORC_TRY({
        const Problem& p = *pr->p;
        if (ndeg < 1 || degrees[0] != p.P) throw std::invalid_argument("degrees[0] must be the problem's P");
        std::unique_ptr<MG> m(new MG());
        m->relaxation = relaxation; m->omega = omega; m->solver = solver;
        m->npre = npre; m->npost = npost; m->restriction = restriction;
        m->mean_project = mean_project != 0;
        m->pr = pr->p;
        m->fine_level(p.ops);
        const int ne = (int)p.mesh->elements.size();
        for (int k = 1; k < ndeg; ++k) m->Ts.push_back(p_transfer(ne, degrees[k - 1], degrees[k]));
        if (nh > 0) {
            std::vector<SBM> h = h_hierarchy(*p.qt, degrees[ndeg - 1]);
            for (int i = 0; i < nh && i < (int)h.size(); ++i) m->Ts.push_back(h[i]);
        }
        for (size_t i = 0; i < m->Ts.size(); ++i) m->coarse_level(*m->levels[i]->ops, m->Ts[i]);
        if (solver == ORC_COARSE_DENSE) m->dense_factor(*m->levels.back());
        *out = new orc_mg{m.release()};
    })
}

// T[l] of the hp hierarchy built by orc_mg_create_hp / orc_mg_create
int orc_mg_transfer_shape(const orc_mg* mg, int l, int* nbr, int* nbc, int* br, int* bc, int* nnzb) {
    ORC_TRY({
        const SBM& T = mg->m->Ts.at(l);
        if (nbr) *nbr = T.blockRows();
        if (nbc) *nbc = T.blockCols();
        if (br) *br = T.P;
        if (bc) *bc = T.Q;
        if (nnzb) *nnzb = (int)T.nnzb();
    })
}
int orc_mg_transfer_export(const orc_mg* mg, int l, int* row_ptr, int* col_idx, double* vals) {
    ORC_TRY({ export_csr(mg->m->Ts.at(l), row_ptr, col_idx, vals); })
}
int orc_mg_destroy(orc_mg* mg) {
    if (mg) { delete mg->m; delete mg; }
    return 0;
}
int orc_mg_nlevels(const orc_mg* mg, int* n) {
    ORC_TRY({ *n = (int)mg->m->levels.size(); })
}
int orc_mg_level_nnzb(const orc_mg* mg, int l, int which, int* nbr, int* nnzb) {
    ORC_TRY({
        const SBM& A = op_of(*mg->m->levels.at(l)->ops, which);
        if (nbr) *nbr = A.blockRows();
        if (nnzb) *nnzb = (int)A.nnzb();
    })
}
int orc_mg_level_block(const orc_mg* mg, int l, int* b) {
    ORC_TRY({ *b = mg->m->levels.at(l)->npl; })
}
int orc_mg_level_export(const orc_mg* mg, int l, int which, int* row_ptr, int* col_idx, double* vals) {
    ORC_TRY({ export_csr(op_of(*mg->m->levels.at(l)->ops, which), row_ptr, col_idx, vals); })
}
int orc_mg_vcycle(orc_mg* mg, const double* b, double* x) {
    ORC_TRY({
        Level& L = *mg->m->levels[0];
        std::memcpy(L.b.data(), b, L.b.size() * sizeof(double));
        std::memcpy(L.x.data(), x, L.x.size() * sizeof(double));
        mg->m->vcycle(0);
        std::memcpy(x, L.x.data(), L.x.size() * sizeof(double));
    })
}
int orc_mg_relax(orc_mg* mg, int l, int n, int reverse, const double* b, double* x) {
    ORC_TRY({
        Level& L = *mg->m->levels.at(l);
        std::memcpy(L.b.data(), b, L.b.size() * sizeof(double));
        std::memcpy(L.x.data(), x, L.x.size() * sizeof(double));
        mg->m->relax(L, n, reverse != 0);
        std::memcpy(x, L.x.data(), L.x.size() * sizeof(double));
    })
}
int orc_pcg(const orc_problem* pr, orc_mg* mg, const double* b, double* x, double tol, int maxit,
            int* iters, double* hist, double* delta_hist) {
    ORC_TRY({
        const SBM& A = pr->p->ops->A;
        size_t n = (size_t)A.rows();
        std::vector<double> bv(b, b + n), xv(x, x + n);
        int it;
        if (mg) {
            MG* m = mg->m;
            // preconditioner closure (dg_tests.cpp:300-305)
            auto precon = [m](const std::vector<double>& r) {
                Level& L = *m->levels[0];
                std::fill(L.x.begin(), L.x.end(), 0.0);
                L.b = r;
                m->vcycle(0);
                return L.x;
            };
            it = pcg(A, bv, xv, precon, tol, maxit, hist, delta_hist);
        } else {
            it = pcg(A, bv, xv, [](const std::vector<double>& r) { return r; }, tol, maxit, hist, delta_hist);
        }
        std::memcpy(x, xv.data(), n * sizeof(double));
        if (iters) *iters = it;
    })
}
// SparseBlockMatrix::write (sparseblockmatrix.tpp:145-164): block-map order
int orc_problem_write_mtx(const orc_problem* pr, int which, const char* path) {
    ORC_TRY({
        const SBM& A = op_of(*pr->p->ops, which);
        std::ofstream ofs(path);
        ofs.precision(std::numeric_limits<double>::max_digits10);
        ofs << "%%MatrixMarket matrix coordinate real general" << std::endl;
        ofs << A.rows() << " " << A.cols() << " " << (long)A.P * A.Q * A.nnzb() << std::endl;
        for (auto it = A.map.begin(); it != A.map.end(); ++it) {
            int bi = it->first.i * A.P, bj = it->first.j * A.Q;
            for (int i = 0; i < A.P; ++i)
                for (int j = 0; j < A.Q; ++j) ofs << bi + i + 1 << " " << bj + j + 1 << " " << it->second(i, j) << std::endl;
        }
        if (!ofs) throw std::runtime_error("write failed");
    })
}
// Function::write (function.h:173-190)
int orc_problem_write_fun(const orc_problem* pr, const double* u, const char* path) {
    ORC_TRY({
        const Problem& p = *pr->p;
        const Tables& T = tables(p.P);
        std::ofstream ofs(path);
        ofs.precision(std::numeric_limits<double>::max_digits10);
        if (p.simplex) {
            // unstructured Function::write (src/unstructured/dg/function.h:159-176)
            ofs << p.P << " " << p.s_dim << " " << p.s_ne << std::endl;
            for (int e = 0; e < p.s_ne; ++e) {
                for (int i = 0; i < p.npl; ++i) {
                    size_t k = (size_t)e * p.npl + i;
                    for (int d = 0; d < p.s_dim; ++d) ofs << p.s_xy[k * p.s_dim + d] << " ";
                    ofs << u[k] << std::endl;
                }
                ofs << std::endl;
            }
            if (!ofs) throw std::runtime_error("write failed");
            return 0;
        }
        int ne = (int)p.mesh->elements.size();
        ofs << p.P << " " << NDIM << " " << ne << std::endl;
        for (int e = 0; e < ne; ++e) {
            const Cell& c = p.mesh->elements[e];
            for (int i0 = 0; i0 < p.P; ++i0)
                for (int i1 = 0; i1 < p.P; ++i1) {
                    double x = c.lo[0] + c.width(0) * T.nodes[i0], y = c.lo[1] + c.width(1) * T.nodes[i1];
                    ofs << x << " " << y << " " << u[(size_t)e * p.npl + i0 * p.P + i1] << std::endl;
                }
            ofs << std::endl;
        }
        if (!ofs) throw std::runtime_error("write failed");
    })
}

int orc_problem_mv(const orc_problem* pr, int which, double alpha, const double* x, double beta, double* y) {
    ORC_TRY({ multiply_add_mv(alpha, op_of(*pr->p->ops, which), x, beta, y); })
}

}  // extern "C"

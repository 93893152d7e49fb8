// reference_stub.h -- the few reference types the C++ binding touches,
// reduced to their interfaces (TEST INFRASTRUCTURE ONLY).
//
// The binding in dg_binding.cpp is written against the reference's own
// classes: DG::SparseBlockMatrix<P,Q> (src/cartesian/util/
// sparseblockmatrix.h:62-165: blockRows, blockCols, colsInRow, getBlock),
// DG::LDGPoisson<N,P>::ops() (src/cartesian/dg/ldgpoisson.h:15-31, 94-97),
// DG::InterpolationHierarchy<N,P>::T (src/cartesian/multigrid/
// interpolationhierarchy.h:91), DG::MG::Parameters (src/cartesian/multigrid/
// multigrid.h:48-62) and DG::Vector.  The reference needs Eigen 3 and MKL,
// which this machine lacks, so these stand-ins keep the same member names
// and types a caller uses, so that the binding compiles unchanged.
#pragma once
#include <array>
#include <map>
#include <memory>
#include <set>
#include <vector>

namespace DG {

using Vector = std::vector<double>;

// row-major dense block with data() like Eigen's RowMajor Mat<P,Q>
template <int P, int Q>
struct Mat {
    std::array<double, P * Q> a{};
    const double* data() const { return a.data(); }
    double& operator()(int r, int c) { return a[r * Q + c]; }
};

template <int P, int Q>
class SparseBlockMatrix {
public:
    SparseBlockMatrix(int m = 0, int n = 0) : m_(m), n_(n) {}
    int blockRows() const { return m_; }
    int blockCols() const { return n_; }
    const std::set<int>& colsInRow(int i) const {
        static const std::set<int> none;
        auto it = cols_.find(i);
        return it == cols_.end() ? none : it->second;
    }
    const Mat<P, Q>& getBlock(int i, int j) const { return blocks_.at({i, j}); }
    void addToBlock(int i, int j, const Mat<P, Q>& b) {
        auto& d = blocks_[{i, j}];
        for (int k = 0; k < P * Q; ++k) d.a[k] += b.a[k];
        cols_[i].insert(j);
    }

private:
    int m_, n_;
    std::map<std::pair<int, int>, Mat<P, Q>> blocks_;
    std::map<int, std::set<int>> cols_;
};

template <int N, int P>
struct LDGOperators {
    SparseBlockMatrix<P, P> M, T;
    std::array<SparseBlockMatrix<P, P>, N> G;
};

template <int N, int P>
struct LDGPoisson {
    std::shared_ptr<LDGOperators<N, P>> ops_ = std::make_shared<LDGOperators<N, P>>();
    std::shared_ptr<LDGOperators<N, P>> ops() const { return ops_; }
};

template <int N, int P>
struct InterpolationHierarchy {
    std::vector<SparseBlockMatrix<P, P>> T;
};

namespace MG {
enum RelaxationMethod { kJacobi, kGaussSeidel };
enum CoarseSolver { kCholesky, kRelaxation };
enum RestrictionMethod { kRAT, kRATRAT };
struct Parameters {
    RelaxationMethod relaxation = kGaussSeidel;
    double omega = 0.8;
    CoarseSolver solver = kCholesky;
    int npre = 3, npost = 3;
    RestrictionMethod restriction = kRATRAT;
};
}  // namespace MG

}  // namespace DG

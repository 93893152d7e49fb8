// simplex.cu -- unstructured triangle meshes: mesh input (.mesh files and a
// disk mesher), P_{P-1} LDG operators assembled on the GPU, and an
// agglomeration hierarchy with tensor-product coarse spaces.
//
// Reference: Wireframe (src/unstructured/mesh/wireframe.h:24-67), Mesh and
// Face (mesh.h:20-300), Master<N,P> (dg/master.h:12-60),
// LDGPoisson::discretize (dg/ldgpoisson.tpp:27-100) and the agglomerated
// InterpolationHierarchy (multigrid/interpolationhierarchy.h:89-210).
//
// The master element is computed here from a monomial basis in long double
// (nodal Lagrange basis on the equispaced simplex nodes, exact monomial
// integrals), not from the reference's orthonormal Koornwinder basis; the
// nodal basis and its mass and differentiation matrices are the same.  The
// GPU computes every element and interior-face block from the element
// geometry (k_simplex_elem, k_simplex_face); the host lists, per stored
// block, its contributions in the reference's order and k_sum_blocks adds
// them.  Departures from the reference, shared with the oracle: faces in
// first-encounter order (element ascending, local face j = {t[j], t[j+1]})
// instead of an unordered_map's order; bounding boxes start from the first
// point (the reference starts from the unit cell); aggregates from the
// greedy seeded agglomeration below instead of MGridGen.  All boundary faces
// are homogeneous Dirichlet.
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <random>
#include <sstream>
#include <unordered_map>

#include "api.cuh"
#include "ldg_build.cuh"

using namespace mg;

namespace mg {

typedef long double LD;

static void ld_inverse(std::vector<LD>& A, int n) {
    std::vector<LD> I((size_t)n * n, 0);
    for (int i = 0; i < n; ++i) I[(size_t)i * n + i] = 1;
    for (int c = 0; c < n; ++c) {
        int piv = c;
        for (int r = c + 1; r < n; ++r)
            if (std::fabs(A[(size_t)r * n + c]) > std::fabs(A[(size_t)piv * n + c])) piv = r;
        MG_REQUIRE(A[(size_t)piv * n + c] != 0, MGLDG_ERR_NOT_SPD, "singular master-element matrix");
        for (int j = 0; j < n; ++j) {
            std::swap(A[(size_t)c * n + j], A[(size_t)piv * n + j]);
            std::swap(I[(size_t)c * n + j], I[(size_t)piv * n + j]);
        }
        const LD d = A[(size_t)c * n + c];
        for (int j = 0; j < n; ++j) {
            A[(size_t)c * n + j] /= d;
            I[(size_t)c * n + j] /= d;
        }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            const LD f = A[(size_t)r * n + c];
            if (f == 0) continue;
            for (int j = 0; j < n; ++j) {
                A[(size_t)r * n + j] -= f * A[(size_t)c * n + j];
                I[(size_t)r * n + j] -= f * I[(size_t)c * n + j];
            }
        }
    }
    A = I;
}

static LD lfact(int n) {
    LD f = 1;
    for (int i = 2; i <= n; ++i) f *= i;
    return f;
}

// Master<N,P> for N = 1, 2, 3: equispaced nodes in SimplexRange order (last
// index fastest, index sum < P), nodal basis phi_i = sum_m C(m,i) x^a y^b z^c
struct SMaster {
    int N = 0, P = 0, b = 0;
    double volume = 0;
    std::vector<std::array<int, 3>> idx;     // node multi-indices
    std::vector<std::array<int, 3>> mono;    // monomial exponents
    std::vector<LD> C;                       // b x b, C[m*b + i]
    std::vector<double> Cd;                  // C rounded to double (for eval)
    std::vector<double> nodes;               // b x N
    std::vector<double> mass, invmass, diff[3];
    SMaster(int N_, int P_) : N(N_), P(P_) {
        for (int i0 = 0; i0 < P; ++i0)
            for (int i1 = 0; i1 < (N >= 2 ? P - i0 : 1); ++i1)
                for (int i2 = 0; i2 < (N >= 3 ? P - i0 - i1 : 1); ++i2)
                    idx.push_back({i0, N >= 2 ? i1 : 0, N >= 3 ? i2 : 0});
        b = (int)idx.size();
        for (int d = 0; d < P; ++d)
            for (int a = d; a >= 0; --a)
                for (int c = 0; c <= d - a; ++c) {
                    const int bb = d - a - c;
                    if (N == 1 && (bb || c)) continue;
                    if (N == 2 && c) continue;
                    mono.push_back({a, bb, c});
                }
        volume = (double)(1 / lfact(N));
        std::vector<LD> xn((size_t)b * 3, 0);
        for (int q = 0; q < b; ++q)
            for (int d = 0; d < N; ++d)
                xn[(size_t)q * 3 + d] = (P == 1) ? (LD)1 / 3 : (LD)idx[q][d] / (P - 1);   // simplexNodes<N,1>: 1/3
        for (int q = 0; q < b; ++q)
            for (int d = 0; d < N; ++d) nodes.push_back((double)xn[(size_t)q * 3 + d]);
        // V(q, m) = mono_m(x_q); C = V^-1
        C.assign((size_t)b * b, 0);
        for (int q = 0; q < b; ++q)
            for (int m = 0; m < b; ++m) C[(size_t)q * b + m] = mono_val(m, &xn[(size_t)q * 3]);
        ld_inverse(C, b);
        Cd.assign(C.begin(), C.end());
        // mass: exact monomial integrals over the master simplex
        // (a! b! c! / (a + b + c + N)!)
        auto integral = [&](int a0, int a1, int a2) -> LD {
            return lfact(a0) * lfact(a1) * lfact(a2) / lfact(a0 + a1 + a2 + N);
        };
        std::vector<LD> Mm((size_t)b * b);
        for (int m = 0; m < b; ++m)
            for (int n = 0; n < b; ++n)
                Mm[(size_t)m * b + n] =
                    integral(mono[m][0] + mono[n][0], mono[m][1] + mono[n][1], mono[m][2] + mono[n][2]);
        std::vector<LD> Ml((size_t)b * b, 0);
        for (int i = 0; i < b; ++i)
            for (int j = 0; j < b; ++j) {
                LD sum = 0;
                for (int m = 0; m < b; ++m)
                    for (int n = 0; n < b; ++n) sum += C[(size_t)m * b + i] * Mm[(size_t)m * b + n] * C[(size_t)n * b + j];
                Ml[(size_t)i * b + j] = sum;
            }
        mass.resize((size_t)b * b);
        for (size_t k = 0; k < Ml.size(); ++k) mass[k] = (double)Ml[k];
        ld_inverse(Ml, b);
        invmass.resize((size_t)b * b);
        for (size_t k = 0; k < Ml.size(); ++k) invmass[k] = (double)Ml[k];
        // diff[d](q, i) = d phi_i / d x_d at node q
        for (int d = 0; d < N; ++d) {
            diff[d].assign((size_t)b * b, 0.0);
            for (int q = 0; q < b; ++q)
                for (int i = 0; i < b; ++i) {
                    LD sum = 0;
                    for (int m = 0; m < b; ++m) sum += C[(size_t)m * b + i] * dmono_val(m, d, &xn[(size_t)q * 3]);
                    diff[d][(size_t)q * b + i] = (double)sum;
                }
        }
    }
    LD mono_val(int m, const LD* x) const {
        LD v = 1;
        for (int d = 0; d < 3; ++d)
            for (int k = 0; k < mono[m][d]; ++k) v *= x[d];
        return v;
    }
    LD dmono_val(int m, int d, const LD* x) const {
        const int e = mono[m][d];
        if (e == 0) return 0;
        LD v = e;
        for (int k = 0; k < e - 1; ++k) v *= x[d];
        for (int o = 0; o < 3; ++o)
            if (o != d)
                for (int k = 0; k < mono[m][o]; ++k) v *= x[o];
        return v;
    }
    // nodal basis at x (N doubles in), in double: the monomials at x once,
    // then phi_i = sum_m C(m,i) x^m (b <= 56, exponents <= 5)
    void eval(const double* x, double* out) const {
        double pw[3][8];
        for (int d = 0; d < 3; ++d) {
            pw[d][0] = 1.0;
            for (int k = 1; k < 8; ++k) pw[d][k] = pw[d][k - 1] * (d < N ? x[d] : 0.0);
        }
        double mv[64];
        for (int m = 0; m < b; ++m) mv[m] = pw[0][mono[m][0]] * pw[1][mono[m][1]] * pw[2][mono[m][2]];
        for (int i = 0; i < b; ++i) {
            double sum = 0;
            for (int m = 0; m < b; ++m) sum += Cd[(size_t)m * b + i] * mv[m];
            out[i] = sum;
        }
    }
    int index_of(int i0, int i1, int i2 = 0) const {
        for (int k = 0; k < b; ++k)
            if (idx[k][0] == i0 && idx[k][1] == i1 && idx[k][2] == i2) return k;
        return -1;
    }
};

// ------------------------------------------------------------ GPU kernels
// Element geometry, 22 doubles per element: p0[3], J[3][3] (J[d][i] =
// p_{i+1,d} - p_{0,d}), Jinv[3][3], volume.
constexpr int kGeom = 22;

// per element e: M_e = Mref vol / vref; G_d(e,e) = sum_j Jinv(j,d) D_j
// (ldgpoisson.tpp:27-60 of the unstructured tree)
__global__ void k_simplex_elem(int ne, int N, int b, const double* __restrict__ geom, const double* __restrict__ Mref,
                               const double* __restrict__ D, double vref, double* __restrict__ out) {
    const int bsz = b * b;
    const int64_t total = (int64_t)ne * bsz;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t / bsz), k = (int)(t - (int64_t)e * bsz);
        const double* g = geom + (size_t)e * kGeom;
        const double* Jinv = g + 12;
        out[(size_t)e * bsz + k] = Mref[k] * (g[21] / vref);
        for (int d = 0; d < N; ++d) {
            double v = Jinv[0 * 3 + d] * D[k];
            for (int j = 1; j < N; ++j) v += Jinv[j * 3 + d] * D[(size_t)j * bsz + k];
            out[((size_t)(1 + d) * ne + e) * bsz + k] = v;
        }
    }
}

struct FaceDev {
    int left, right;
    double n[3], jac, volR;   // jac = face area / master face volume
    int sl[10], sr[10];       // element node of face node a, left / right
};

// per interior face, 2N + 4 blocks: G_d(R,R) = (n_d MinvR) RR, G_d(R,L) =
// (-n_d MinvR) RL for d < N, then T(R,R) = tau RR, T(L,L) = tau LL,
// T(R,L) = -tau RL, T(L,R) = -tau RL^T, with RR = S_r^T (Mf jac) S_r etc.
// (ldgpoisson.tpp:63-100, mesh.h:270-283)
__global__ void k_simplex_face(int nf, int N, int b, int P1, const FaceDev* __restrict__ faces,
                               const double* __restrict__ Mf, const double* __restrict__ Minv, double vref,
                               double tau0, double* __restrict__ out) {
    const int bsz = b * b;
    const int nk = 2 * N + 4;
    const int64_t total = (int64_t)nf * nk * bsz;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(t / ((int64_t)nk * bsz));
        const int rem = (int)(t - (int64_t)f * nk * bsz);
        const int kind = rem / bsz, k = rem - kind * bsz;
        const int r = k / b, c = k - r * b;
        const FaceDev& F = faces[f];
        double v = 0;
        if (kind < 2 * N) {
            // (s n_d MinvR)(S_r^T fm S_x), column c must be a face node of the
            // trial side x (right for RR, left for RL)
            const int d = kind >> 1;
            const bool rl = kind & 1;
            const double s = rl ? -F.n[d] : F.n[d];
            const int* sx = rl ? F.sl : F.sr;
            int cc = -1;
            for (int a = 0; a < P1; ++a)
                if (sx[a] == c) cc = a;
            if (cc >= 0) {
                // sum over the element nodes k = sr[a] in ascending order
                int ord[10];
                for (int a = 0; a < P1; ++a) ord[a] = a;
                for (int i = 1; i < P1; ++i)
                    for (int j = i; j > 0 && F.sr[ord[j]] < F.sr[ord[j - 1]]; --j) {
                        int tmp = ord[j]; ord[j] = ord[j - 1]; ord[j - 1] = tmp;
                    }
                const double jac = vref / F.volR;
                for (int q = 0; q < P1; ++q) {
                    const int a = ord[q];
                    const double minv = s * (Minv[r * b + F.sr[a]] * jac);
                    v += minv * (Mf[a * P1 + cc] * F.jac);
                }
            }
        } else {
            const int kk = kind - 2 * N;
            const int* srow = (kk == 1 || kk == 3) ? F.sl : F.sr;
            const int* scol = (kk == 0 || kk == 3) ? F.sr : F.sl;
            int ra = -1, cb = -1;
            for (int a = 0; a < P1; ++a) {
                if (srow[a] == r) ra = a;
                if (scol[a] == c) cb = a;
            }
            if (ra >= 0 && cb >= 0) {
                // T(L,R) = -tau RL^T: entry (r, c) = -tau fm(c-face-node, r-face-node)
                const double m = (kk == 3) ? Mf[cb * P1 + ra] * F.jac : Mf[ra * P1 + cb] * F.jac;
                const double tau = (kk <= 1) ? tau0 : -tau0;
                v = tau * m;
            }
        }
        out[(size_t)f * nk * bsz + (size_t)kind * bsz + k] = v;
    }
}

// b_e = M_e f at the element's nodes, f a Gaussian sum centred in the unit
// ball of dimension N (seed 0: f = 1)
struct GaussDevS {
    double c[3][8], w[8], a[8];
    int constant_one;
};
__global__ void k_rhs_simplex(int ne, int N, int b, const double* __restrict__ geom, const double* __restrict__ nodes,
                              const double* __restrict__ Mref, double vref, GaussDevS g, double* __restrict__ out) {
    extern __shared__ double sf[];
    for (int e = blockIdx.x; e < ne; e += gridDim.x) {
        const double* gm = geom + (size_t)e * kGeom;
        for (int q = threadIdx.x; q < b; q += blockDim.x) {
            double x[3] = {0, 0, 0};
            for (int d = 0; d < N; ++d) {
                double acc = gm[3 + d * 3 + 0] * nodes[N * q + 0];
                for (int j = 1; j < N; ++j) acc += gm[3 + d * 3 + j] * nodes[N * q + j];
                x[d] = gm[d] + acc;
            }
            double sum = 0;
            if (g.constant_one) {
                sum = 1.0;
            } else {
                for (int k = 0; k < 8; ++k) {
                    double r2 = 0;
                    for (int d = 0; d < N; ++d) {
                        const double dd = x[d] - g.c[d][k];
                        r2 += dd * dd;
                    }
                    sum += g.a[k] * exp(-r2 / (2.0 * g.w[k] * g.w[k]));
                }
            }
            sf[q] = sum;
        }
        __syncthreads();
        const double jac = gm[21] / vref;
        for (int r = threadIdx.x; r < b; r += blockDim.x) {
            double sum = 0;
            for (int c = 0; c < b; ++c) sum += (Mref[r * b + c] * jac) * sf[c];
            out[(size_t)e * b + r] = sum;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ host parts
struct SEl {
    double p[4][3];
    double J[3][3], Jinv[3][3], vol;
};

static SEl make_sel(int N, const double* pts, const int* t) {
    SEl s{};
    for (int j = 0; j <= N; ++j)
        for (int d = 0; d < N; ++d) s.p[j][d] = pts[(size_t)N * t[j] + d];
    for (int d = 0; d < N; ++d)
        for (int i = 0; i < N; ++i) s.J[d][i] = s.p[i + 1][d] - s.p[0][d];
    double det;
    if (N == 2) {
        det = s.J[0][0] * s.J[1][1] - s.J[0][1] * s.J[1][0];
        MG_REQUIRE(det != 0 && std::isfinite(det), MGLDG_ERR_ARG, "degenerate triangle");
        s.Jinv[0][0] = s.J[1][1] / det;
        s.Jinv[0][1] = -s.J[0][1] / det;
        s.Jinv[1][0] = -s.J[1][0] / det;
        s.Jinv[1][1] = s.J[0][0] / det;
        s.vol = std::fabs(det) / 2;
    } else {
        const double(&a)[3][3] = s.J;
        const double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
        const double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
        const double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
        det = a[0][0] * c00 + a[0][1] * c01 + a[0][2] * c02;
        MG_REQUIRE(det != 0 && std::isfinite(det), MGLDG_ERR_ARG, "degenerate tetrahedron");
        s.Jinv[0][0] = c00 / det;
        s.Jinv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
        s.Jinv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
        s.Jinv[1][0] = c01 / det;
        s.Jinv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
        s.Jinv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
        s.Jinv[2][0] = c02 / det;
        s.Jinv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
        s.Jinv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
        s.vol = std::fabs(det) / 6;
    }
    return s;
}

// Gaussian sum in the unit ball: centres by rejection from [-1,1]^N,
// widths U[0.05,0.2], amplitudes N(0,1) (Box-Muller, cosine branch)
static GaussDevS gaussian_ball(uint64_t seed, int N) {
    GaussDevS p{};
    if (seed == 0) {
        p.constant_one = 1;
        return p;
    }
    std::mt19937_64 g(seed);
    auto uni = [&]() { return (double)(g() >> 11) * 0x1.0p-53; };
    for (int k = 0; k < 8; ++k) {
        double x[3], r2;
        do {
            r2 = 0;
            for (int d = 0; d < N; ++d) {
                x[d] = 2 * uni() - 1;
                r2 += x[d] * x[d];
            }
        } while (r2 >= 1);
        for (int d = 0; d < N; ++d) p.c[d][k] = x[d];
        p.w[k] = 0.05 + 0.15 * uni();
        double u1;
        do { u1 = uni(); } while (u1 <= 0.0);
        const double u2 = uni();
        p.a[k] = std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * 3.14159265358979323846 * u2);
    }
    return p;
}

typedef std::vector<std::vector<std::pair<int, double>>> Graph;

// Greedy seeded agglomeration (no reference counterpart; stands in for
// MGridGen): nodes in the order of seeded keys (mt19937_64(seed), ties by
// index); an unassigned node starts an aggregate and grows it up to maxsize
// -- in two dimensions with its own unassigned neighbours, heaviest shared
// face first (ties: lower index); in three dimensions breadth-first, each
// time taking the unassigned node with the largest total face weight to the
// aggregate (ties: lower index).  An aggregate of fewer than minsize
// elements then joins the neighbouring aggregate it shares the most face
// weight with (ties: lower aggregate): a few elements' nodes need not
// determine the P^N tensor modes of their bounding box.  Aggregates keep
// their creation order.
static std::vector<int> greedy_agglomerate(int n, const Graph& adj, uint64_t seed, int N, int* ncoarse) {
    const int maxsize = N == 3 ? 8 : 4, minsize = N == 3 ? 6 : 3;
    std::mt19937_64 g(seed);
    std::vector<std::pair<uint64_t, int>> key(n);
    for (int u = 0; u < n; ++u) key[u] = {g(), u};
    std::sort(key.begin(), key.end());
    std::vector<int> agg(n, -1), size;
    std::vector<std::pair<int, double>> cand;
    for (auto& kv : key) {
        const int u = kv.second;
        if (agg[u] >= 0) continue;
        const int a = (int)size.size();
        size.push_back(1);
        agg[u] = a;
        if (N != 3) {
            cand.clear();
            for (auto& e : adj[u])
                if (agg[e.first] < 0) cand.push_back(e);
            std::sort(cand.begin(), cand.end(), [](const std::pair<int, double>& x, const std::pair<int, double>& y) {
                if (x.second != y.second) return x.second > y.second;
                return x.first < y.first;
            });
            for (size_t k = 0; k < cand.size() && (int)k < maxsize - 1; ++k) {
                agg[cand[k].first] = a;
                size[a]++;
            }
        } else {
            std::map<int, double> front;
            auto grow = [&](int m) {
                for (auto& e : adj[m])
                    if (agg[e.first] < 0) {
                        auto it = front.find(e.first);
                        if (it == front.end()) front[e.first] = e.second;
                        else it->second += e.second;
                    }
            };
            grow(u);
            while (size[a] < maxsize && !front.empty()) {
                int best = -1;
                double bw = -1;
                for (auto& kv2 : front)
                    if (kv2.second > bw) {
                        bw = kv2.second;
                        best = kv2.first;
                    }
                front.erase(best);
                agg[best] = a;
                size[a]++;
                grow(best);
            }
        }
    }
    std::vector<std::vector<int>> members(size.size());
    for (int u = 0; u < n; ++u) members[agg[u]].push_back(u);
    for (int a = 0; a < (int)size.size(); ++a) {
        if (size[a] == 0 || size[a] >= minsize) continue;
        std::map<int, double> wt;
        for (int u : members[a])
            for (auto& e : adj[u]) {
                const int c = agg[e.first];
                if (c == a) continue;
                auto it = wt.find(c);
                if (it == wt.end()) wt[c] = e.second;
                else it->second += e.second;
            }
        int best = -1;
        double bw = -1;
        for (auto& kv : wt)
            if (kv.second > bw) {
                bw = kv.second;
                best = kv.first;
            }
        if (best < 0) continue;
        for (int u : members[a]) {
            agg[u] = best;
            members[best].push_back(u);
        }
        members[a].clear();
        size[best] += size[a];
        size[a] = 0;
    }
    std::vector<int> renum(size.size(), -1);
    int nc = 0;
    for (int a = 0; a < (int)size.size(); ++a)
        if (size[a] > 0) renum[a] = nc++;
    for (int u = 0; u < n; ++u) agg[u] = renum[agg[u]];
    *ncoarse = nc;
    return agg;
}

static Graph coarse_graph(const Graph& adj, const std::vector<int>& agg, int nc) {
    std::vector<std::map<int, double>> m(nc);
    for (size_t u = 0; u < adj.size(); ++u)
        for (auto& e : adj[u]) {
            const int a = agg[u], c = agg[e.first];
            if (a == c) continue;
            auto it = m[a].find(c);
            if (it == m[a].end()) m[a][c] = e.second;
            else it->second += e.second;
        }
    Graph out(nc);
    for (int a = 0; a < nc; ++a)
        for (auto& kv : m[a]) out[a].push_back(kv);
    return out;
}

struct SBox {
    double lo[3], hi[3];
};

static mgldg_bsr* host_bsr(mgldg_ctx* ctx, int nbr, int nbc, int br, int bc, const std::vector<int>& col,
                           const std::vector<double>& vals) {
    std::vector<int> rp(nbr + 1);
    for (int k = 0; k <= nbr; ++k) rp[k] = k;
    mgldg_bsr* T = bsr_new(ctx, nbr, nbc, br, bc, rp, col);
    try {
        upload(ctx, T->val, vals.data(), vals.size());
    } catch (...) {
        delete T;
        throw;
    }
    return T;
}

// quadrature on the master face (an (N-1)-simplex), weights summing to 1:
// the 10-point Gauss-Legendre rule on an edge; on a triangle the collapsed
// 10 x 10 Gauss-Legendre product (Duffy), exact for degree 19
static void face_rule(int N, std::vector<double>& x, std::vector<double>& w) {
    x.clear();
    w.clear();
    if (N == 2) {
        for (int q = 0; q < MGLDG_QF; ++q) {
            x.push_back(kQuadNodes[q]);
            w.push_back(kQuadWeights[q]);
        }
        return;
    }
    for (int a = 0; a < MGLDG_QF; ++a)
        for (int c = 0; c < MGLDG_QF; ++c) {
            const double u = kQuadNodes[a], v = kQuadNodes[c];
            x.push_back(u);
            x.push_back(v * (1 - u));
            w.push_back(2 * kQuadWeights[a] * kQuadWeights[c] * (1 - u));
        }
}

// Cholesky factor of the aggregate's Gram matrix G = sum_u T_u^T M_u T_u
// (row-major lower triangle; pivots below 1e-13 of the diagonal are raised to
// that floor) and T_u <- T_u L^-T for its rows.  Plain double arithmetic in a
// fixed order, the same as the oracle's.
static void orthonormalize(const std::vector<int>& rows, std::vector<double>& vals, int br, int cb,
                           const std::vector<SEl>* el, const std::vector<double>& Mref, double vref, double* Lout) {
    std::vector<double> G((size_t)cb * cb, 0.0), MT((size_t)br * cb);
    for (int u : rows) {
        const double* T = &vals[(size_t)u * br * cb];
        if (el) {
            const double jac = (*el)[u].vol / vref;
            for (int r = 0; r < br; ++r)
                for (int c = 0; c < cb; ++c) {
                    double s = 0;
                    for (int k = 0; k < br; ++k) s += (Mref[(size_t)r * br + k] * jac) * T[(size_t)k * cb + c];
                    MT[(size_t)r * cb + c] = s;
                }
        } else {
            for (size_t k = 0; k < MT.size(); ++k) MT[k] = T[k];
        }
        for (int i = 0; i < cb; ++i)
            for (int j = 0; j < cb; ++j) {
                double s = 0;
                for (int r = 0; r < br; ++r) s += T[(size_t)r * cb + i] * MT[(size_t)r * cb + j];
                G[(size_t)i * cb + j] += s;
            }
    }
    // Cholesky G = L L^T with dropping: a column whose part M-orthogonal to
    // the earlier kept columns has squared norm <= kDrop of its own is
    // (numerically) in their span and is dropped -- its basis function
    // becomes exactly zero, L(j,j) = 0 and column j of L is zero.  The tensor
    // space interpolated at the nodes of a few simplices is rank deficient
    // (27 functions on aggregates of tetrahedra with fewer distinct nodes);
    // the kept columns span the same coarse space.  Row j of L keeps its
    // entries: the dropped function's coordinates in the kept basis.
    constexpr double kDrop = 1e-8;
    std::vector<double> L((size_t)cb * cb, 0.0);
    std::vector<char> kept(cb, 0);
    for (int j = 0; j < cb; ++j) {
        double d = G[(size_t)j * cb + j];
        for (int k = 0; k < j; ++k) d -= L[(size_t)j * cb + k] * L[(size_t)j * cb + k];
        if (!(d > kDrop * G[(size_t)j * cb + j])) continue;
        kept[j] = 1;
        L[(size_t)j * cb + j] = std::sqrt(d);
        for (int i = j + 1; i < cb; ++i) {
            double v = G[(size_t)i * cb + j];
            for (int k = 0; k < j; ++k) v -= L[(size_t)i * cb + k] * L[(size_t)j * cb + k];
            L[(size_t)i * cb + j] = v / L[(size_t)j * cb + j];
        }
    }
    for (int u : rows) {
        double* T = &vals[(size_t)u * br * cb];
        for (int r = 0; r < br; ++r) {
            double* t = T + (size_t)r * cb;
            for (int j = 0; j < cb; ++j) {
                if (!kept[j]) {
                    t[j] = 0.0;
                    continue;
                }
                double v = t[j];
                for (int k = 0; k < j; ++k) v -= L[(size_t)j * cb + k] * t[k];
                t[j] = v / L[(size_t)j * cb + j];
            }
        }
    }
    std::copy(L.begin(), L.end(), Lout);
}

mgldg_problem* simplex_problem(mgldg_ctx* ctx, int N, int np, const double* pts, int nt, const int* tris, int P,
                               double tau0, double tauD, int agg_levels, uint64_t agg_seed,
                               std::vector<std::vector<int>>* parts) {
    MG_REQUIRE(N == 2 || N == 3, MGLDG_ERR_ARG, "dimension must be 2 or 3");
    MG_REQUIRE(P >= 1 && P <= (N == 2 ? 4 : 3), MGLDG_ERR_UNSUPPORTED, "P must be 1..4 on triangles, 1..3 on tetrahedra");
    MG_REQUIRE(np >= N + 1 && nt >= 1 && pts && tris, MGLDG_ERR_ARG, "empty mesh");
    MG_REQUIRE(N == 2 || np < (1 << 21), MGLDG_ERR_UNSUPPORTED, "more than 2^21 vertices");
    const int nv = N + 1;
    for (int64_t k = 0; k < (int64_t)nv * nt; ++k)
        MG_REQUIRE(tris[k] >= 0 && tris[k] < np, MGLDG_ERR_ARG, "vertex index out of range");
    static const bool trace = std::getenv("MGLDG_SETUP_TRACE") != nullptr;
    auto t_last = std::chrono::steady_clock::now();
    auto phase = [&](const char* what) {
        if (!trace) return;
        sync(ctx);
        const auto now = std::chrono::steady_clock::now();
        std::fprintf(stderr, "[mgldg build] %-14s %8.1f ms\n", what,
                     std::chrono::duration<double, std::milli>(now - t_last).count());
        t_last = now;
    };
    const SMaster MS(N, P), MF(N - 1, P);
    const int b = MS.b, P1 = MF.b;
    std::vector<SEl> el(nt);
    for (int e = 0; e < nt; ++e) el[e] = make_sel(N, pts, tris + (size_t)nv * e);

    // ---- faces in first-encounter order (mesh.h:209-300): face j of an
    // element has the vertices t[(k+j) % (N+1)], k < N
    struct HF {
        int left, right, v[3];
        double n[3], area;
        int sl[10], sr[10];
    };
    std::vector<HF> faces;
    faces.reserve((size_t)nt * (N == 2 ? 2 : 3));
    std::unordered_map<uint64_t, int> f2f;
    f2f.reserve((size_t)nt * 4);
    for (int e = 0; e < nt; ++e)
        for (int j = 0; j < nv; ++j) {
            int f[3];
            for (int k = 0; k < N; ++k) f[k] = tris[(size_t)nv * e + (k + j) % nv];
            std::sort(f, f + N);
            const uint64_t key = N == 2 ? (((uint64_t)f[0] << 32) | (uint32_t)f[1])
                                        : (((uint64_t)f[0] << 42) | ((uint64_t)f[1] << 21) | (uint64_t)f[2]);
            auto it = f2f.find(key);
            if (it == f2f.end()) {
                HF h{};
                h.left = e;
                h.right = -1;
                for (int k = 0; k < N; ++k) h.v[k] = f[k];
                f2f.emplace(key, (int)faces.size());
                faces.push_back(h);
            } else {
                MG_REQUIRE(faces[it->second].right < 0, MGLDG_ERR_ARG, "a face is shared by more than two elements");
                faces[it->second].right = e;
            }
        }
    auto local = [&](int e, int v) {
        for (int i = 0; i < nv; ++i)
            if (tris[(size_t)nv * e + i] == v) return i;
        return -1;
    };
    auto P_ = [&](int v, int d) { return pts[(size_t)N * v + d]; };
    int nb = 0;
    for (HF& f : faces) {
        double e1[3] = {0, 0, 0}, e2[3] = {0, 0, 0}, nrm[3] = {0, 0, 0};
        for (int d = 0; d < N; ++d) e1[d] = P_(f.v[1], d) - P_(f.v[0], d);
        if (N == 2) {
            nrm[0] = e1[1];
            nrm[1] = -e1[0];
            f.area = std::sqrt(e1[0] * e1[0] + e1[1] * e1[1]);
        } else {
            for (int d = 0; d < 3; ++d) e2[d] = P_(f.v[2], d) - P_(f.v[0], d);
            nrm[0] = e1[1] * e2[2] - e1[2] * e2[1];
            nrm[1] = -(e1[0] * e2[2] - e1[2] * e2[0]);
            nrm[2] = e1[0] * e2[1] - e1[1] * e2[0];
            // Simplex<2,3>::volume = sqrt(det(J^T J)) / 2 (geometry.h:66-79)
            double g00 = 0, g01 = 0, g11 = 0;
            for (int d = 0; d < 3; ++d) {
                g00 += e1[d] * e1[d];
                g01 += e1[d] * e2[d];
                g11 += e2[d] * e2[d];
            }
            f.area = std::sqrt(g00 * g11 - g01 * g01) / 2;
        }
        double len = 0;
        for (int d = 0; d < N; ++d) len += nrm[d] * nrm[d];
        len = std::sqrt(len);
        for (int d = 0; d < N; ++d) nrm[d] /= len;
        int a = -1;
        for (int i = 0; i < nv; ++i) {
            const int v = tris[(size_t)nv * f.left + i];
            bool on = false;
            for (int k = 0; k < N; ++k) on = on || (v == f.v[k]);
            if (!on) a = v;
        }
        double dot = 0;
        for (int d = 0; d < N; ++d) dot += nrm[d] * (P_(a, d) - P_(f.v[0], d));
        if (dot > 0)
            for (int d = 0; d < N; ++d) nrm[d] = -nrm[d];
        for (int d = 0; d < N; ++d) f.n[d] = nrm[d];
        if (f.right < 0) {
            ++nb;
            continue;
        }
        // slicing: face node with multi-index j (barycentrics (P-1-|j|, j) on
        // the sorted face vertices) is the element node sum_k lambda_k corner_k
        for (int side = 0; side < 2; ++side) {
            const int e = side ? f.right : f.left;
            int loc[3];
            for (int k = 0; k < N; ++k) loc[k] = local(e, f.v[k]);
            for (int q = 0; q < P1; ++q) {
                int node = 0;
                if (P > 1) {
                    int lam[3];
                    lam[0] = P - 1;
                    for (int k = 1; k < N; ++k) {
                        lam[k] = MF.idx[q][k - 1];
                        lam[0] -= lam[k];
                    }
                    int m[3] = {0, 0, 0};
                    for (int k = 0; k < N; ++k)
                        if (loc[k] > 0) m[loc[k] - 1] += lam[k];   // corner i is the unit vector e_{i-1}
                    node = MS.index_of(m[0], m[1], m[2]);
                }
                (side ? f.sr : f.sl)[q] = node;
            }
        }
    }
    const int nf = (int)faces.size();
    const int nfi = nf - nb;
    phase("faces");

    // ---- contributions: elements (M, G_d), interior faces (2N + 4),
    // boundary faces (N + 1)
    std::vector<int> interior, boundary;
    for (int k = 0; k < nf; ++k) (faces[k].right >= 0 ? interior : boundary).push_back(k);
    std::vector<int> slot(nf);
    for (int q = 0; q < nfi; ++q) slot[interior[q]] = q;
    for (int q = 0; q < nb; ++q) slot[boundary[q]] = q;
    const size_t bsz = (size_t)b * b;
    const int nkf = 2 * N + 4, nkb = N + 1;
    const int64_t c_elem = 0, c_face = (int64_t)(1 + N) * nt, c_bnd = c_face + (int64_t)nkf * nfi;
    const int64_t ncontrib = c_bnd + (int64_t)nkb * nb;
    MG_REQUIRE(ncontrib < (int64_t)1 << 31, MGLDG_ERR_UNSUPPORTED, "mesh too large for the contribution index");

    // boundary blocks on the host (quadrature, mesh.h:284-300)
    std::vector<double> qx, qw;
    face_rule(N, qx, qw);
    const int nq = (int)qw.size();
    std::vector<double> bvals((size_t)nkb * nb * bsz);
    parallel_ranges(nb, 64, [&](int64_t q0, int64_t q1) {
        std::vector<double> phl((size_t)nq * b), Lm((size_t)b * nq), LL(bsz), Minv(bsz);
        for (int64_t q = q0; q < q1; ++q) {
            const HF& f = faces[boundary[q]];
            const SEl& s = el[f.left];
            for (int k = 0; k < nq; ++k) {
                double phys[3];
                for (int d = 0; d < N; ++d) {
                    double acc = 0;
                    for (int j = 1; j < N; ++j) acc += (P_(f.v[j], d) - P_(f.v[0], d)) * qx[(size_t)k * (N - 1) + j - 1];
                    phys[d] = P_(f.v[0], d) + acc;
                }
                double rel[3], xl[3];
                for (int d = 0; d < N; ++d) rel[d] = phys[d] - s.p[0][d];
                for (int i = 0; i < N; ++i) {
                    double acc = 0;
                    for (int d = 0; d < N; ++d) acc += s.Jinv[i][d] * rel[d];
                    xl[i] = acc;
                }
                MS.eval(xl, &phl[(size_t)k * b]);
            }
            for (int a = 0; a < b; ++a)
                for (int k = 0; k < nq; ++k) Lm[(size_t)a * nq + k] = phl[(size_t)k * b + a] * (qw[k] * f.area);
            for (int a = 0; a < b; ++a)
                for (int c = 0; c < b; ++c) {
                    double sum = 0;
                    for (int k = 0; k < nq; ++k) sum += Lm[(size_t)a * nq + k] * phl[(size_t)k * b + c];
                    LL[(size_t)a * b + c] = sum;
                }
            const double jac = MS.volume / s.vol;
            for (size_t k = 0; k < bsz; ++k) Minv[k] = MS.invmass[k] * jac;
            for (int d = 0; d < N; ++d) {
                double* G = &bvals[((size_t)nkb * q + d) * bsz];
                const double sc = -f.n[d];
                for (int r = 0; r < b; ++r)
                    for (int c = 0; c < b; ++c) {
                        double sum = 0;
                        for (int k = 0; k < b; ++k) sum += (sc * Minv[(size_t)r * b + k]) * LL[(size_t)k * b + c];
                        G[(size_t)r * b + c] = sum;
                    }
            }
            double* T = &bvals[((size_t)nkb * q + N) * bsz];
            for (size_t k = 0; k < bsz; ++k) T[k] = tauD * LL[k];
        }
    });

    phase("boundary");
    // per stored block, its contributions in the reference's order
    struct Tr {
        int row, col;
        int64_t seq, contrib;
    };
    std::vector<Tr> tm, tg[3], tt;
    int64_t seq = 0;
    for (int e = 0; e < nt; ++e) tm.push_back({e, e, seq++, c_elem + e});
    for (int d = 0; d < N; ++d)
        for (int e = 0; e < nt; ++e) tg[d].push_back({e, e, seq++, c_elem + (int64_t)(1 + d) * nt + e});
    for (int k = 0; k < nf; ++k) {
        const HF& f = faces[k];
        if (f.right >= 0) {
            const int64_t base = c_face + (int64_t)nkf * slot[k];
            for (int d = 0; d < N; ++d) {
                tg[d].push_back({f.right, f.right, seq++, base + 2 * d});
                tg[d].push_back({f.right, f.left, seq++, base + 2 * d + 1});
            }
            tt.push_back({f.right, f.right, seq++, base + 2 * N});
            tt.push_back({f.left, f.left, seq++, base + 2 * N + 1});
            tt.push_back({f.right, f.left, seq++, base + 2 * N + 2});
            tt.push_back({f.left, f.right, seq++, base + 2 * N + 3});
        } else {
            const int64_t base = c_bnd + (int64_t)nkb * slot[k];
            for (int d = 0; d < N; ++d) tg[d].push_back({f.left, f.left, seq++, base + d});
            tt.push_back({f.left, f.left, seq++, base + N});
        }
    }
    auto assemble = [&](std::vector<Tr>& v) {
        std::sort(v.begin(), v.end(), [](const Tr& a, const Tr& c) {
            if (a.row != c.row) return a.row < c.row;
            if (a.col != c.col) return a.col < c.col;
            return a.seq < c.seq;
        });
        Assembly As;
        As.row_ptr.assign(nt + 1, 0);
        size_t k = 0;
        std::vector<int> cs;
        for (int r = 0; r < nt; ++r) {
            while (k < v.size() && v[k].row == r) {
                const int col = v[k].col;
                cs.clear();
                while (k < v.size() && v[k].row == r && v[k].col == col) cs.push_back((int)v[k++].contrib);
                As.add_block_v(col, cs);
            }
            As.row_ptr[r + 1] = (int)As.col_idx.size();
        }
        return As;
    };
    Assembly AM, AT;
    std::vector<Assembly> AG(N);
    parallel_for(N + 2, 1, [&](int64_t w) {
        if (w == 0) AM = assemble(tm);
        else if (w <= N) AG[w - 1] = assemble(tg[w - 1]);
        else AT = assemble(tt);
    });

    phase("lists");
    // ---- GPU: contributions, then the operators ----
    mgldg_problem* pr = new mgldg_problem();
    pr->ctx = ctx;
    pr->P = P;
    pr->b = b;
    pr->ne = nt;
    pr->n = 0;
    pr->simplex = true;
    pr->sdim = N;
    pr->nfaces = nf;
    pr->nbfaces = nb;
    double *d_contrib = nullptr, *d_geom = nullptr, *d_ref = nullptr;
    FaceDev* d_faces = nullptr;
    mgldg_bsr* M = nullptr;
    std::vector<mgldg_bsr*> Gs;
    mgldg_bsr* Tm = nullptr;
    try {
        std::vector<double> geom((size_t)nt * kGeom, 0.0);
        for (int e = 0; e < nt; ++e) {
            double* g = &geom[(size_t)e * kGeom];
            for (int d = 0; d < N; ++d) g[d] = el[e].p[0][d];
            for (int d = 0; d < 3; ++d)
                for (int i = 0; i < 3; ++i) {
                    g[3 + d * 3 + i] = el[e].J[d][i];
                    g[12 + d * 3 + i] = el[e].Jinv[d][i];
                }
            g[21] = el[e].vol;
        }
        std::vector<FaceDev> fd(nfi);
        for (int q = 0; q < nfi; ++q) {
            const HF& f = faces[interior[q]];
            FaceDev& D = fd[q];
            D.left = f.left;
            D.right = f.right;
            for (int d = 0; d < 3; ++d) D.n[d] = d < N ? f.n[d] : 0.0;
            D.jac = f.area / MF.volume;   // Face::mass (mesh.h:100-104)
            D.volR = el[f.right].vol;
            for (int a = 0; a < 10; ++a) {
                D.sl[a] = a < P1 ? f.sl[a] : -1;
                D.sr[a] = a < P1 ? f.sr[a] : -1;
            }
        }
        // reference tables: Mref | D_0..D_{N-1} | Minv | Mface
        std::vector<double> ref;
        ref.insert(ref.end(), MS.mass.begin(), MS.mass.end());
        for (int d = 0; d < N; ++d) ref.insert(ref.end(), MS.diff[d].begin(), MS.diff[d].end());
        ref.insert(ref.end(), MS.invmass.begin(), MS.invmass.end());
        ref.insert(ref.end(), MF.mass.begin(), MF.mass.end());
        d_geom = dalloc<double>(geom.size());
        d_ref = dalloc<double>(ref.size());
        d_faces = dalloc<FaceDev>(std::max(1, nfi));
        d_contrib = dalloc<double>((size_t)ncontrib * bsz);
        upload(ctx, d_geom, geom.data(), geom.size());
        upload(ctx, d_ref, ref.data(), ref.size());
        if (nfi) upload(ctx, d_faces, fd.data(), fd.size());
        if (nb) upload(ctx, d_contrib + (size_t)c_bnd * bsz, bvals.data(), bvals.size());
        const double* dM = d_ref;
        const double* dD = d_ref + bsz;
        const double* dMinv = d_ref + (size_t)(1 + N) * bsz;
        const double* dMf = d_ref + (size_t)(2 + N) * bsz;
        {
            const int64_t tot = (int64_t)nt * bsz;
            const int g = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, ctx->sm_count * 32));
            Launch L(ctx, MGLDG_K_SETUP);
            k_simplex_elem<<<g, 256, 0, ctx->stream>>>(nt, N, b, d_geom, dM, dD, MS.volume, d_contrib);
        }
        check_launch();
        if (nfi) {
            const int64_t tot = (int64_t)nfi * nkf * bsz;
            const int g = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, ctx->sm_count * 32));
            Launch L(ctx, MGLDG_K_SETUP);
            k_simplex_face<<<g, 256, 0, ctx->stream>>>(nfi, N, b, P1, d_faces, dMf, dMinv, MS.volume, tau0,
                                                       d_contrib + (size_t)c_face * bsz);
        }
        check_launch();
        phase("gpu blocks");
        M = realize(ctx, AM, nt, b, d_contrib);
        for (int d = 0; d < N; ++d) Gs.push_back(realize(ctx, AG[d], nt, b, d_contrib));
        Tm = realize(ctx, AT, nt, b, d_contrib);
        pr->ops = new mgldg_ops();
        pr->ops->ctx = ctx;
        pr->ops->ndim = N;
        pr->ops->M = M; M = nullptr;
        for (int d = 0; d < N; ++d) {
            pr->ops->G[d] = Gs[d];
            Gs[d] = nullptr;
        }
        pr->ops->T = Tm; Tm = nullptr;
        phase("realize");
        construct_laplacian(ctx, pr->ops);
        phase("laplacian");
        // geometry for right-hand sides and dumps
        pr->sgeom = geom;
        pr->snodes = MS.nodes;
        pr->d_geom = d_geom; d_geom = nullptr;
        pr->d_nodes = dalloc<double>(MS.nodes.size());
        upload(ctx, pr->d_nodes, MS.nodes.data(), MS.nodes.size());
        pr->d_Mref = dalloc<double>(bsz);
        upload(ctx, pr->d_Mref, MS.mass.data(), bsz);
        pr->svref = MS.volume;

        // ---- agglomeration hierarchy (interpolationhierarchy.h:89-210) ----
        Graph adj(nt);
        for (const HF& f : faces)
            if (f.right >= 0) {
                adj[f.left].push_back({f.right, f.area});
                adj[f.right].push_back({f.left, f.area});
            }
        for (auto& a : adj) std::sort(a.begin(), a.end());
        std::vector<SBox> box(nt), fbox;
        for (int e = 0; e < nt; ++e)
            for (int d = 0; d < N; ++d) {
                box[e].lo[d] = box[e].hi[d] = el[e].p[0][d];
                for (int j = 1; j < nv; ++j) {
                    box[e].lo[d] = std::min(box[e].lo[d], el[e].p[j][d]);
                    box[e].hi[d] = std::max(box[e].hi[d], el[e].p[j][d]);
                }
            }
        const Ref2 CR(P);
        const int cb = N == 2 ? P * P : P * P * P;
        // tensor Lagrange basis of the box at x (Cartesian LagrangePoly<P>,
        // last index fastest)
        auto lagrangeN = [&](const double* x, double* out) {
            double l[3][8];
            for (int d = 0; d < N; ++d) CR.lagrange1(x[d], l[d]);
            int k = 0;
            for (int i0 = 0; i0 < P; ++i0)
                for (int i1 = 0; i1 < P; ++i1)
                    for (int i2 = 0; i2 < (N == 3 ? P : 1); ++i2) {
                        double v = 1;
                        v *= l[0][i0];
                        v *= l[1][i1];
                        if (N == 3) v *= l[2][i2];
                        out[k++] = v;
                    }
        };
        int nfine = nt;
        std::vector<double> Lprev;   // per finer aggregate: its basis factor L
        for (int lev = 0; lev < agg_levels && nfine > 1; ++lev) {
            int nc = 0;
            std::vector<int> agg = greedy_agglomerate(nfine, adj, agg_seed + (uint64_t)lev, N, &nc);
            if (nc >= nfine) break;
            phase("  agglomerate");
            const std::vector<SBox>& src = lev == 0 ? box : fbox;
            std::vector<SBox> cbox(nc);
            std::vector<char> seen(nc, 0);
            std::vector<int> cnt(nc, 0);
            for (int u = 0; u < nfine; ++u) {
                const int a = agg[u];
                cnt[a]++;
                if (!seen[a]) {
                    cbox[a] = src[u];
                    seen[a] = 1;
                    continue;
                }
                for (int d = 0; d < N; ++d) {
                    cbox[a].lo[d] = std::min(cbox[a].lo[d], src[u].lo[d]);
                    cbox[a].hi[d] = std::max(cbox[a].hi[d], src[u].hi[d]);
                }
            }
            const int br = lev == 0 ? b : cb;
            std::vector<double> vals((size_t)nfine * br * cb, 0.0);
            parallel_for(nfine, 1024, [&](int64_t u) {
                const int a = agg[u];
                const SBox& B = cbox[a];
                double w[3];
                for (int d = 0; d < N; ++d) w[d] = B.hi[d] - B.lo[d];
                double* E = &vals[(size_t)u * br * cb];
                if (lev == 0) {
                    // the fine simplex mapped into the box, the box's tensor
                    // basis at its nodes
                    double rp[4][3];
                    for (int j = 0; j < nv; ++j)
                        for (int d = 0; d < N; ++d) rp[j][d] = (el[u].p[j][d] - B.lo[d]) / w[d];
                    for (int i = 0; i < b; ++i) {
                        double x[3];
                        for (int d = 0; d < N; ++d) {
                            double acc = (rp[1][d] - rp[0][d]) * MS.nodes[(size_t)N * i];
                            for (int j = 1; j < N; ++j) acc += (rp[j + 1][d] - rp[0][d]) * MS.nodes[(size_t)N * i + j];
                            x[d] = rp[0][d] + acc;
                        }
                        lagrangeN(x, E + (size_t)i * cb);
                    }
                } else if (cnt[a] == 1) {
                    for (int i = 0; i < cb; ++i) E[(size_t)i * cb + i] = 1.0;
                } else {
                    const SBox& F = src[u];
                    double rlo[3], rhi[3];
                    for (int d = 0; d < N; ++d) {
                        rlo[d] = (F.lo[d] - B.lo[d]) / w[d];
                        rhi[d] = (F.hi[d] - B.lo[d]) / w[d];
                    }
                    int row = 0;
                    for (int i0 = 0; i0 < P; ++i0)
                        for (int i1 = 0; i1 < P; ++i1)
                            for (int i2 = 0; i2 < (N == 3 ? P : 1); ++i2) {
                                const int id[3] = {i0, i1, i2};
                                double x[3];
                                for (int d = 0; d < N; ++d) x[d] = rlo[d] + (rhi[d] - rlo[d]) * CR.nodes[id[d]];
                                lagrangeN(x, E + (size_t)(row++) * cb);
                            }
                }
            });
            // per aggregate, make the coarse basis orthonormal in the fine
            // mass inner product: T_a <- T_a L_a^-T with L_a L_a^T =
            // sum_{u in a} T_u^T M_u T_u (M_u the element mass on level 0;
            // on coarser levels the previous coarse masses, the identity)
            {
                // rows first: the finer level's own basis change, T_u <- L_u^T T_u
                if (lev > 0)
                    parallel_ranges(nfine, 256, [&](int64_t u0, int64_t u1) {
                        std::vector<double> tmp((size_t)br * cb);
                        for (int64_t u = u0; u < u1; ++u) {
                            double* T = &vals[(size_t)u * br * cb];
                            const double* Lu = &Lprev[(size_t)u * cb * cb];
                            for (int r = 0; r < br; ++r)
                                for (int c = 0; c < cb; ++c) {
                                    double sum = 0;
                                    for (int k = r; k < br; ++k) sum += Lu[(size_t)k * cb + r] * T[(size_t)k * cb + c];
                                    tmp[(size_t)r * cb + c] = sum;
                                }
                            std::copy(tmp.begin(), tmp.end(), T);
                        }
                    });
                phase("  basis");
                std::vector<std::vector<int>> members(nc);
                for (int u = 0; u < nfine; ++u) members[agg[u]].push_back(u);
                std::vector<double> Lnext((size_t)nc * cb * cb);
                parallel_for(nc, 64, [&](int64_t a) {
                    orthonormalize(members[a], vals, br, cb, lev == 0 ? &el : nullptr, MS.mass, MS.volume,
                                   &Lnext[(size_t)a * cb * cb]);
                });
                Lprev.swap(Lnext);
            }
            phase("  orthonormal");
            pr->T.push_back(host_bsr(ctx, nfine, nc, br, cb, agg, vals));
            phase("  upload");
            if (parts) parts->push_back(agg);
            adj = coarse_graph(adj, agg, nc);
            fbox = cbox;
            nfine = nc;
        }
        pr->nlevels = (int)pr->T.size() + 1;
        sync(ctx);
    } catch (...) {
        dfree(d_contrib);
        dfree(d_geom);
        dfree(d_ref);
        dfree(d_faces);
        delete M;
        for (auto* g : Gs) delete g;
        delete Tm;
        delete pr;
        throw;
    }
    dfree(d_contrib);
    dfree(d_ref);
    dfree(d_faces);
    return pr;
}

void simplex_rhs_dev(mgldg_ctx* ctx, const mgldg_problem* pr, uint64_t seed, double* b) {
    const GaussDevS g = gaussian_ball(seed, pr->sdim);
    const int grid = std::max(1, std::min(pr->ne, ctx->sm_count * 32));
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_rhs_simplex<<<grid, 64, pr->b * sizeof(double), ctx->stream>>>(pr->ne, pr->sdim, pr->b, pr->d_geom,
                                                                         pr->d_nodes, pr->d_Mref, pr->svref, g, b);
    }
    check_launch();
}

// Disk mesher (no reference counterpart; the reference reads distmesh
// output): concentric rings of radius k/K (K = ceil(1/h)), ring k with
// max(6k, round(2 pi k)) equally spaced points starting at angle 0, and the
// strip between rings k-1 and k triangulated by advancing whichever ring's
// next point has the smaller angle.  Counter-clockwise triangles.
// Elements sorted (stably) by the Morton key of their centroid: 2^(63/N)
// cells per axis over the centroids' bounding box, bits interleaved with x
// highest.  The element order is the order of block Gauss-Seidel, whose
// sweep is a chain of dependencies through neighbours that come earlier;
// orders that close a loop (a ring around the disk) make that chain as long
// as the mesh, a space-filling order keeps it near the mesh's diameter.
static void morton_order(int N, const double* p, int nt, int* t) {
    const int nv = N + 1, bits = 63 / N;
    std::vector<double> c((size_t)nt * N, 0.0);
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int e = 0; e < nt; ++e)
        for (int d = 0; d < N; ++d) {
            double s = 0;
            for (int v = 0; v < nv; ++v) s += p[(size_t)N * t[(size_t)nv * e + v] + d];
            s /= nv;
            c[(size_t)N * e + d] = s;
            lo[d] = std::min(lo[d], s);
            hi[d] = std::max(hi[d], s);
        }
    const double cells = std::ldexp(1.0, bits);
    std::vector<std::pair<uint64_t, int>> key(nt);
    for (int e = 0; e < nt; ++e) {
        uint64_t q[3] = {0, 0, 0};
        for (int d = 0; d < N; ++d) {
            const double w = hi[d] - lo[d];
            const double f = w > 0 ? (c[(size_t)N * e + d] - lo[d]) / w : 0.0;
            q[d] = (uint64_t)std::min(cells - 1, std::max(0.0, std::floor(f * cells)));
        }
        uint64_t k = 0;
        for (int b = bits - 1; b >= 0; --b)
            for (int d = 0; d < N; ++d) k = (k << 1) | ((q[d] >> b) & 1u);
        key[e] = {k, e};
    }
    std::stable_sort(key.begin(), key.end(),
                     [](const std::pair<uint64_t, int>& a, const std::pair<uint64_t, int>& b) { return a.first < b.first; });
    std::vector<int> old(t, t + (size_t)nv * nt);
    for (int e = 0; e < nt; ++e)
        for (int v = 0; v < nv; ++v) t[(size_t)nv * e + v] = old[(size_t)nv * key[e].second + v];
}

static void disk_mesh(double h, std::vector<double>& p, std::vector<int>& t) {
    MG_REQUIRE(h > 0 && h <= 1, MGLDG_ERR_ARG, "mesh size must be in (0, 1]");
    const int K = (int)std::ceil(1.0 / h - 1e-12);
    MG_REQUIRE(K <= 4096, MGLDG_ERR_ARG, "mesh size too small");
    const double PI = 3.14159265358979323846;
    std::vector<int> start(K + 1), count(K + 1);
    p.clear();
    t.clear();
    p.push_back(0.0);
    p.push_back(0.0);
    start[0] = 0;
    count[0] = 1;
    for (int k = 1; k <= K; ++k) {
        const int n = std::max(6 * k, (int)std::lround(2 * PI * k));
        start[k] = (int)p.size() / 2;
        count[k] = n;
        const double r = (double)k / K;
        for (int j = 0; j < n; ++j) {
            const double a = 2 * PI * j / n;
            p.push_back(r * std::cos(a));
            p.push_back(r * std::sin(a));
        }
    }
    for (int j = 0; j < count[1]; ++j) {
        t.push_back(0);
        t.push_back(start[1] + j);
        t.push_back(start[1] + (j + 1) % count[1]);
    }
    for (int k = 2; k <= K; ++k) {
        const int ni = count[k - 1], no = count[k];
        int i = 0, o = 0;
        while (i < ni || o < no) {
            // angles of the next points (as fractions of a turn)
            const double ai = (double)(i + 1) / ni, ao = (double)(o + 1) / no;
            const int ci = start[k - 1] + i % ni, co = start[k] + o % no;
            if (o < no && (i >= ni || ao <= ai)) {
                t.push_back(ci);
                t.push_back(co);
                t.push_back(start[k] + (o + 1) % no);
                ++o;
            } else {
                t.push_back(ci);
                t.push_back(co);
                t.push_back(start[k - 1] + (i + 1) % ni);
                ++i;
            }
        }
    }
    morton_order(2, p.data(), (int)t.size() / 3, t.data());
}

// Ball mesher (no reference counterpart), a cubed sphere: a core cube
// [-a,a]^3 (a = 0.45) of m^3 hexahedra and, over each of its six faces, nr
// radial layers of hexahedra whose vertices blend the core-surface point q
// into q/|q| (layer l: (1 - l/nr) q + (l/nr) q/|q|).  Hexahedra are about 2h
// across (m = ceil(a/h), nr = ceil((1-a)/(2h))).  Every hexahedron is cut
// into 24 tetrahedra: each face into four triangles about its centre (the
// mean of its corners, shared with the neighbour; projected onto the sphere
// on the boundary), each triangle joined to the cell centre.  The cut of a
// face depends only on the face, so the mesh is conforming, and no
// tetrahedron has four vertices on the sphere (a cube grid mapped onto the
// ball has such slivers along the cube's edges, flatter as h shrinks).
// Positively oriented tetrahedra in the Morton order of their centroids.
static void ball_mesh(double h, std::vector<double>& p, std::vector<int>& t) {
    MG_REQUIRE(h > 0 && h <= 2, MGLDG_ERR_ARG, "mesh size must be in (0, 2]");
    const double a = 0.45;
    const int m = std::max(1, (int)std::ceil(a / h - 1e-12));
    const int nr = std::max(1, (int)std::ceil((1 - a) / (2 * h) - 1e-12));
    MG_REQUIRE(m <= 256 && nr <= 256, MGLDG_ERR_ARG, "mesh size too small");
    p.clear();
    t.clear();
    const int m1 = m + 1;
    auto cid = [&](int i, int j, int k) { return (i * m1 + j) * m1 + k; };
    for (int i = 0; i < m1; ++i)
        for (int j = 0; j < m1; ++j)
            for (int k = 0; k < m1; ++k) {
                p.push_back(-a + 2 * a * i / m);
                p.push_back(-a + 2 * a * j / m);
                p.push_back(-a + 2 * a * k / m);
            }
    // shell vertex of core-surface vertex c at layer l (l = 0: c itself)
    std::vector<int> sid((size_t)m1 * m1 * m1 * nr, -1);
    auto shell = [&](int c, int l) {
        if (l == 0) return c;
        int& v = sid[(size_t)c * nr + l - 1];
        if (v < 0) {
            const double q[3] = {p[3 * c], p[3 * c + 1], p[3 * c + 2]};
            const double r = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
            const double s = (double)l / nr;
            v = (int)p.size() / 3;
            for (int d = 0; d < 3; ++d) p.push_back(l == nr ? q[d] / r : (1 - s) * q[d] + s * q[d] / r);
        }
        return v;
    };
    // hexahedra, corners indexed x + 2y + 4z in a local frame
    std::vector<std::array<int, 8>> hex;
    for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j)
            for (int k = 0; k < m; ++k) {
                std::array<int, 8> hx;
                for (int c = 0; c < 8; ++c) hx[c] = cid(i + (c & 1), j + ((c >> 1) & 1), k + ((c >> 2) & 1));
                hex.push_back(hx);
            }
    for (int d = 0; d < 3; ++d)
        for (int side = 0; side < 2; ++side) {
            const int d1 = (d + 1) % 3, d2 = (d + 2) % 3;
            for (int u = 0; u < m; ++u)
                for (int v = 0; v < m; ++v)
                    for (int l = 0; l < nr; ++l) {
                        std::array<int, 8> hx;
                        for (int c = 0; c < 8; ++c) {
                            int ix[3];
                            ix[d] = side ? m : 0;
                            ix[d1] = u + (c & 1);
                            ix[d2] = v + ((c >> 1) & 1);
                            hx[c] = shell(cid(ix[0], ix[1], ix[2]), l + ((c >> 2) & 1));
                        }
                        hex.push_back(hx);
                    }
        }
    // the 24-tetrahedron cut
    static const int face[6][4] = {{0, 2, 6, 4}, {1, 3, 7, 5}, {0, 1, 5, 4}, {2, 3, 7, 6}, {0, 1, 3, 2}, {4, 5, 7, 6}};
    std::map<std::array<int, 4>, int> fcen;
    std::map<std::array<int, 4>, int> fuse;
    for (const auto& hx : hex)
        for (const auto& f : face) {
            std::array<int, 4> key = {hx[f[0]], hx[f[1]], hx[f[2]], hx[f[3]]};
            std::sort(key.begin(), key.end());
            fuse[key]++;
        }
    auto push_tet = [&](int v0, int v1, int v2, int v3) {
        double e[3][3];
        const int w[3] = {v1, v2, v3};
        for (int s2 = 0; s2 < 3; ++s2)
            for (int q = 0; q < 3; ++q) e[s2][q] = p[3 * w[s2] + q] - p[3 * v0 + q];
        const double det = e[0][0] * (e[1][1] * e[2][2] - e[1][2] * e[2][1]) -
                           e[0][1] * (e[1][0] * e[2][2] - e[1][2] * e[2][0]) +
                           e[0][2] * (e[1][0] * e[2][1] - e[1][1] * e[2][0]);
        if (det < 0) std::swap(v2, v3);
        t.push_back(v0);
        t.push_back(v1);
        t.push_back(v2);
        t.push_back(v3);
    };
    for (const auto& hx : hex) {
        double cc[3] = {0, 0, 0};
        for (int c = 0; c < 8; ++c)
            for (int q = 0; q < 3; ++q) cc[q] += p[3 * hx[c] + q] / 8;
        const int cv = (int)p.size() / 3;
        for (int q = 0; q < 3; ++q) p.push_back(cc[q]);
        for (const auto& f : face) {
            std::array<int, 4> key = {hx[f[0]], hx[f[1]], hx[f[2]], hx[f[3]]};
            std::sort(key.begin(), key.end());
            auto it = fcen.find(key);
            int fv;
            if (it != fcen.end()) {
                fv = it->second;
            } else {
                double fc[3] = {0, 0, 0};
                for (int c = 0; c < 4; ++c)
                    for (int q = 0; q < 3; ++q) fc[q] += p[3 * hx[f[c]] + q] / 4;
                if (fuse[key] == 1) {
                    // a face of one hexahedron only: on the sphere
                    const double r = std::sqrt(fc[0] * fc[0] + fc[1] * fc[1] + fc[2] * fc[2]);
                    for (int q = 0; q < 3; ++q) fc[q] /= r;
                }
                fv = (int)p.size() / 3;
                for (int q = 0; q < 3; ++q) p.push_back(fc[q]);
                fcen.emplace(key, fv);
            }
            for (int c = 0; c < 4; ++c) push_tet(hx[f[c]], hx[f[(c + 1) % 4]], fv, cv);
        }
    }
    morton_order(3, p.data(), (int)t.size() / 4, t.data());
}

}  // namespace mg

// ================================================================== C ABI ==
extern "C" int mgldg_disk_mesh(double h, int* np, int* nt, double* p, int* t) {
    if (!np || !nt) return MGLDG_ERR_ARG;
    try {
        std::vector<double> pv;
        std::vector<int> tv;
        disk_mesh(h, pv, tv);
        *np = (int)pv.size() / 2;
        *nt = (int)tv.size() / 3;
        if (p) std::copy(pv.begin(), pv.end(), p);
        if (t) std::copy(tv.begin(), tv.end(), t);
    } catch (const Error& e) {
        return e.code;
    } catch (const std::bad_alloc&) {
        return MGLDG_ERR_NOMEM;
    }
    return MGLDG_OK;
}

// Wireframe(file) (wireframe.h:24-67): "np nt", a header line, np lines of
// coordinates, an empty line, nt lines of 1-based vertex indices
// Wireframe<N>(file) (wireframe.h:24-67) for N = 2 (triangles) or 3
// (tetrahedra): "np nt", one more header line, np lines of N coordinates,
// an empty line, nt lines of N+1 one-based vertex indices.
extern "C" int mgldg_mesh_read_nd(const char* path, int N, int* np, int* nt, double* p, int* t) {
    if (!path || !np || !nt || (N != 2 && N != 3)) return MGLDG_ERR_ARG;
    std::ifstream ifs(path);
    if (!ifs.is_open()) return MGLDG_ERR_ARG;
    std::string line;
    int n_p = 0, n_t = 0;
    if (!std::getline(ifs, line)) return MGLDG_ERR_ARG;
    {
        std::istringstream ss(line);
        if (!(ss >> n_p >> n_t) || n_p < 0 || n_t < 0) return MGLDG_ERR_ARG;
    }
    std::getline(ifs, line);
    int ip = 0, it = 0;
    while (std::getline(ifs, line) && !line.empty()) {
        std::istringstream ss(line);
        double v[3] = {0, 0, 0};
        int k = 0;
        double x;
        while (ss >> x) {
            if (k < 3) v[k] = x;
            ++k;
        }
        if (k != N || ip >= n_p) return MGLDG_ERR_ARG;
        if (p)
            for (int d = 0; d < N; ++d) p[(size_t)N * ip + d] = v[d];
        ++ip;
    }
    while (std::getline(ifs, line) && !line.empty()) {
        std::istringstream ss(line);
        int v[4] = {0, 0, 0, 0};
        int k = 0;
        int x;
        while (ss >> x) {
            if (k < 4) v[k] = x;
            ++k;
        }
        if (k != N + 1 || it >= n_t) return MGLDG_ERR_ARG;
        for (int j = 0; j <= N; ++j)
            if (v[j] < 1 || v[j] > n_p) return MGLDG_ERR_ARG;
        if (t)
            for (int j = 0; j <= N; ++j) t[(size_t)(N + 1) * it + j] = v[j] - 1;
        ++it;
    }
    if (ip != n_p || it != n_t) return MGLDG_ERR_SHAPE;
    *np = n_p;
    *nt = n_t;
    return MGLDG_OK;
}

extern "C" int mgldg_mesh_read(const char* path, int* np, int* nt, double* p, int* t) {
    return mgldg_mesh_read_nd(path, 2, np, nt, p, t);
}

extern "C" int mgldg_simplex_problem_create_nd(mgldg_ctx* ctx, int N, int np, const double* p, int nt, const int* t,
                                               int P, double tau0, double tauD, int agg_levels, uint64_t agg_seed,
                                               mgldg_problem** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(out != nullptr && agg_levels >= 0, MGLDG_ERR_ARG, "bad arguments");
    *out = nullptr;
    std::vector<std::vector<int>> parts;
    mgldg_problem* pr = simplex_problem(ctx, N, np, p, nt, t, P, tau0, tauD, agg_levels, agg_seed, &parts);
    pr->partitions = std::move(parts);
    *out = pr;
    MG_API_END
}

extern "C" int mgldg_simplex_problem_create(mgldg_ctx* ctx, int np, const double* p, int nt, const int* t, int P,
                                            double tau0, double tauD, int agg_levels, uint64_t agg_seed,
                                            mgldg_problem** out) {
    return mgldg_simplex_problem_create_nd(ctx, 2, np, p, nt, t, P, tau0, tauD, agg_levels, agg_seed, out);
}

extern "C" int mgldg_problem_partition(const mgldg_problem* pr, int l, int* n, int* agg) {
    if (!pr || !n || l < 0 || l >= (int)pr->partitions.size()) return MGLDG_ERR_ARG;
    const std::vector<int>& a = pr->partitions[l];
    *n = (int)a.size();
    if (agg) std::copy(a.begin(), a.end(), agg);
    return MGLDG_OK;
}

extern "C" int mgldg_simplex_master_nd(int N, int P, double* mass, double* diff, double* nodes) {
    if (N < 1 || N > 3 || P < 1 || P > 6 || !mass || !nodes) return MGLDG_ERR_ARG;
    try {
        const SMaster m(N, P);
        std::copy(m.mass.begin(), m.mass.end(), mass);
        if (diff)
            for (int d = 0; d < N; ++d) std::copy(m.diff[d].begin(), m.diff[d].end(), diff + (size_t)d * m.b * m.b);
        std::copy(m.nodes.begin(), m.nodes.end(), nodes);
    } catch (const Error& e) {
        return e.code;
    }
    return MGLDG_OK;
}

extern "C" int mgldg_simplex_master(int N, int P, double* mass, double* diff0, double* diff1, double* nodes) {
    if ((N != 1 && N != 2) || P < 1 || P > 6 || !mass || !nodes) return MGLDG_ERR_ARG;
    try {
        const SMaster m(N, P);
        std::copy(m.mass.begin(), m.mass.end(), mass);
        if (diff0) std::copy(m.diff[0].begin(), m.diff[0].end(), diff0);
        if (diff1 && N == 2) std::copy(m.diff[1].begin(), m.diff[1].end(), diff1);
        std::copy(m.nodes.begin(), m.nodes.end(), nodes);
    } catch (const Error& e) {
        return e.code;
    }
    return MGLDG_OK;
}

extern "C" int mgldg_mesh_morton_order(int N, int np, const double* p, int nt, int* t) {
    if ((N != 2 && N != 3) || np < 1 || nt < 0 || !p || (nt > 0 && !t)) return MGLDG_ERR_ARG;
    for (int64_t k = 0; k < (int64_t)(N + 1) * nt; ++k)
        if (t[k] < 0 || t[k] >= np) return MGLDG_ERR_ARG;
    try {
        morton_order(N, p, nt, t);
    } catch (const std::bad_alloc&) {
        return MGLDG_ERR_NOMEM;
    }
    return MGLDG_OK;
}

extern "C" int mgldg_ball_mesh(double h, int* np, int* nt, double* p, int* t) {
    if (!np || !nt) return MGLDG_ERR_ARG;
    try {
        std::vector<double> pv;
        std::vector<int> tv;
        ball_mesh(h, pv, tv);
        *np = (int)pv.size() / 3;
        *nt = (int)tv.size() / 4;
        if (p) std::copy(pv.begin(), pv.end(), p);
        if (t) std::copy(tv.begin(), tv.end(), t);
    } catch (const Error& e) {
        return e.code;
    } catch (const std::bad_alloc&) {
        return MGLDG_ERR_NOMEM;
    }
    return MGLDG_OK;
}

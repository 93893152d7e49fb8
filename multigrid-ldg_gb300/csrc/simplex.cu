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
#include <cmath>
#include <cstdio>
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

// Master<N,P> for N = 1, 2: equispaced nodes in SimplexRange order (last
// index fastest, index sum < P), nodal basis phi_i = sum_m C(m,i) x^a y^b
struct SMaster {
    int N = 0, P = 0, b = 0;
    double volume = 0;
    std::vector<std::array<int, 2>> idx;     // node multi-indices
    std::vector<std::array<int, 2>> mono;    // monomial exponents
    std::vector<LD> C;                       // b x b, C[m*b + i]
    std::vector<double> nodes;               // b x N
    std::vector<double> mass, invmass, diff[2];
    SMaster(int N_, int P_) : N(N_), P(P_) {
        for (int i0 = 0; i0 < P; ++i0)
            for (int i1 = 0; i1 < (N == 2 ? P - i0 : 1); ++i1) idx.push_back({i0, N == 2 ? i1 : 0});
        b = (int)idx.size();
        for (int d = 0; d < P; ++d)
            for (int a = d; a >= 0; --a)
                if (N == 2) mono.push_back({a, d - a});
                else if (a == d) mono.push_back({a, 0});
        volume = (double)(1 / lfact(N));
        std::vector<LD> xn((size_t)b * 2, 0);
        for (int q = 0; q < b; ++q)
            for (int d = 0; d < N; ++d)
                xn[(size_t)q * 2 + d] = (P == 1) ? (LD)1 / 3 : (LD)idx[q][d] / (P - 1);
        for (int q = 0; q < b; ++q)
            for (int d = 0; d < N; ++d) nodes.push_back((double)xn[(size_t)q * 2 + d]);
        // V(q, m) = mono_m(x_q); C = V^-1
        C.assign((size_t)b * b, 0);
        for (int q = 0; q < b; ++q)
            for (int m = 0; m < b; ++m) C[(size_t)q * b + m] = mono_val(m, &xn[(size_t)q * 2]);
        ld_inverse(C, b);
        // mass: exact monomial integrals over the master simplex
        auto integral = [&](int a0, int a1) -> LD {
            if (N == 1) return (LD)1 / (a0 + 1);
            return lfact(a0) * lfact(a1) / lfact(a0 + a1 + 2);
        };
        std::vector<LD> Mm((size_t)b * b);
        for (int m = 0; m < b; ++m)
            for (int n = 0; n < b; ++n) Mm[(size_t)m * b + n] = integral(mono[m][0] + mono[n][0], mono[m][1] + mono[n][1]);
        std::vector<LD> Ml((size_t)b * b, 0);
        for (int i = 0; i < b; ++i)
            for (int j = 0; j < b; ++j) {
                LD s = 0;
                for (int m = 0; m < b; ++m)
                    for (int n = 0; n < b; ++n) s += C[(size_t)m * b + i] * Mm[(size_t)m * b + n] * C[(size_t)n * b + j];
                Ml[(size_t)i * b + j] = s;
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
                    LD s = 0;
                    for (int m = 0; m < b; ++m) s += C[(size_t)m * b + i] * dmono_val(m, d, &xn[(size_t)q * 2]);
                    diff[d][(size_t)q * b + i] = (double)s;
                }
        }
    }
    LD mono_val(int m, const LD* x) const {
        LD v = 1;
        for (int k = 0; k < mono[m][0]; ++k) v *= x[0];
        if (N == 2)
            for (int k = 0; k < mono[m][1]; ++k) v *= x[1];
        return v;
    }
    LD dmono_val(int m, int d, const LD* x) const {
        const int e = mono[m][d];
        if (e == 0) return 0;
        LD v = e;
        for (int k = 0; k < e - 1; ++k) v *= x[d];
        if (N == 2) {
            const int o = 1 - d;
            for (int k = 0; k < mono[m][o]; ++k) v *= x[o];
        }
        return v;
    }
    // nodal basis at x (double in, double out)
    void eval(const double* x, double* out) const {
        const LD xl[2] = {x[0], N == 2 ? x[1] : 0};
        for (int i = 0; i < b; ++i) {
            LD s = 0;
            for (int m = 0; m < b; ++m) s += C[(size_t)m * b + i] * mono_val(m, xl);
            out[i] = (double)s;
        }
    }
    int index_of(int i0, int i1) const {
        for (int k = 0; k < b; ++k)
            if (idx[k][0] == i0 && idx[k][1] == i1) return k;
        return -1;
    }
};

// ------------------------------------------------------------ GPU kernels
// per element e (geom: p0 x, p0 y, J00, J01, J10, J11, Jinv00, Jinv01,
// Jinv10, Jinv11, vol): M_e = Mref vol / vref; G_d(e,e) = sum_j Jinv(j,d) D_j
__global__ void k_simplex_elem(int ne, int b, const double* __restrict__ geom, const double* __restrict__ Mref,
                               const double* __restrict__ D0, const double* __restrict__ D1, double vref,
                               double* __restrict__ out) {
    const int bsz = b * b;
    const int64_t total = (int64_t)ne * bsz;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int e = (int)(t / bsz), k = (int)(t - (int64_t)e * bsz);
        const double* g = geom + (size_t)e * 11;
        out[(size_t)e * bsz + k] = Mref[k] * (g[10] / vref);
        for (int d = 0; d < 2; ++d) {
            double v = g[6 + d] * D0[k];   // Jinv(0, d) D0
            v += g[8 + d] * D1[k];         // + Jinv(1, d) D1
            out[((size_t)(1 + d) * ne + e) * bsz + k] = v;
        }
    }
}

struct FaceDev {
    int left, right;
    double n0, n1, area, volR;
    int sl[6], sr[6];   // element node of face node a, left / right
};

// per interior face, eight blocks: G_d(R,R) = (n_d MinvR) RR, G_d(R,L) =
// (-n_d MinvR) RL (d = 0, 1), then T(R,R) = tau RR, T(L,L) = tau LL,
// T(R,L) = -tau RL, T(L,R) = -tau RL^T, with RR = S_r^T (M1 area) S_r etc.
__global__ void k_simplex_face(int nf, int b, int P1, const FaceDev* __restrict__ faces,
                               const double* __restrict__ M1, const double* __restrict__ Minv, double vref,
                               double tau0, double* __restrict__ out) {
    const int bsz = b * b;
    const int64_t total = (int64_t)nf * 8 * bsz;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int f = (int)(t / (8 * bsz));
        const int rem = (int)(t - (int64_t)f * 8 * bsz);
        const int kind = rem / bsz, k = rem - kind * bsz;
        const int r = k / b, c = k - r * b;
        const FaceDev& F = faces[f];
        double v = 0;
        if (kind < 4) {
            // (s n_d MinvR)(S_r^T fm S_x), column c must be a face node of the
            // trial side x (right for RR, left for RL)
            const int d = kind >> 1;
            const bool rl = kind & 1;
            const double nd = d == 0 ? F.n0 : F.n1;
            const double s = rl ? -nd : nd;
            const int* sx = rl ? F.sl : F.sr;
            int cc = -1;
            for (int a = 0; a < P1; ++a)
                if (sx[a] == c) cc = a;
            if (cc >= 0) {
                // sum over the element nodes k = sr[a] in ascending order
                int ord[6];
                for (int a = 0; a < P1; ++a) ord[a] = a;
                for (int i = 1; i < P1; ++i)
                    for (int j = i; j > 0 && F.sr[ord[j]] < F.sr[ord[j - 1]]; --j) {
                        int tmp = ord[j]; ord[j] = ord[j - 1]; ord[j - 1] = tmp;
                    }
                const double jac = vref / F.volR;
                for (int q = 0; q < P1; ++q) {
                    const int a = ord[q];
                    const double minv = s * (Minv[r * b + F.sr[a]] * jac);
                    v += minv * (M1[a * P1 + cc] * F.area);
                }
            }
        } else {
            const int kk = kind - 4;
            const int* srow = (kk == 1) ? F.sl : (kk == 3 ? F.sl : F.sr);
            const int* scol = (kk == 0) ? F.sr : (kk == 1 ? F.sl : (kk == 2 ? F.sl : F.sr));
            int ra = -1, cb = -1;
            for (int a = 0; a < P1; ++a) {
                if (srow[a] == r) ra = a;
                if (scol[a] == c) cb = a;
            }
            if (ra >= 0 && cb >= 0) {
                // T(L,R) = -tau RL^T: entry (r, c) = -tau fm(c-face-node, r-face-node)
                const double m = (kk == 3) ? M1[cb * P1 + ra] * F.area : M1[ra * P1 + cb] * F.area;
                const double tau = (kk <= 1) ? tau0 : -tau0;
                v = tau * m;
            }
        }
        out[(size_t)f * 8 * bsz + (size_t)kind * bsz + k] = v;
    }
}

// b_e = M_e f at the element's nodes, f the disk Gaussian sum
struct GaussDevS {
    double cx[8], cy[8], w[8], a[8];
    int constant_one;
};
__global__ void k_rhs_simplex(int ne, int b, const double* __restrict__ geom, const double* __restrict__ nodes,
                              const double* __restrict__ Mref, double vref, GaussDevS g, double* __restrict__ out) {
    extern __shared__ double sf[];
    for (int e = blockIdx.x; e < ne; e += gridDim.x) {
        const double* gm = geom + (size_t)e * 11;
        for (int q = threadIdx.x; q < b; q += blockDim.x) {
            const double x = gm[0] + (gm[2] * nodes[2 * q] + gm[3] * nodes[2 * q + 1]);
            const double y = gm[1] + (gm[4] * nodes[2 * q] + gm[5] * nodes[2 * q + 1]);
            double s = 0;
            if (g.constant_one) {
                s = 1.0;
            } else {
                for (int k = 0; k < 8; ++k) {
                    const double dx = x - g.cx[k], dy = y - g.cy[k];
                    s += g.a[k] * exp(-(dx * dx + dy * dy) / (2.0 * g.w[k] * g.w[k]));
                }
            }
            sf[q] = s;
        }
        __syncthreads();
        const double jac = gm[10] / vref;
        for (int r = threadIdx.x; r < b; r += blockDim.x) {
            double s = 0;
            for (int c = 0; c < b; ++c) s += (Mref[r * b + c] * jac) * sf[c];
            out[(size_t)e * b + r] = s;
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------ host parts
struct STri {
    double p[3][2];
    double J[2][2], Jinv[2][2], vol;
};

static STri make_stri(const double* pts, const int* t) {
    STri s;
    for (int j = 0; j < 3; ++j)
        for (int d = 0; d < 2; ++d) s.p[j][d] = pts[2 * t[j] + d];
    for (int d = 0; d < 2; ++d)
        for (int i = 0; i < 2; ++i) s.J[d][i] = s.p[i + 1][d] - s.p[0][d];
    const double det = s.J[0][0] * s.J[1][1] - s.J[0][1] * s.J[1][0];
    MG_REQUIRE(det != 0 && std::isfinite(det), MGLDG_ERR_ARG, "degenerate triangle");
    s.Jinv[0][0] = s.J[1][1] / det;
    s.Jinv[0][1] = -s.J[0][1] / det;
    s.Jinv[1][0] = -s.J[1][0] / det;
    s.Jinv[1][1] = s.J[0][0] / det;
    s.vol = std::fabs(det) / 2;
    return s;
}

// disk Gaussian sum: centres uniform on the unit disk (rejection from
// [-1,1]^2), widths U[0.05,0.2], amplitudes N(0,1) (Box-Muller, cosine)
static GaussDevS gaussian_disk(uint64_t seed) {
    GaussDevS p{};
    if (seed == 0) {
        p.constant_one = 1;
        return p;
    }
    std::mt19937_64 g(seed);
    auto uni = [&]() { return (double)(g() >> 11) * 0x1.0p-53; };
    for (int k = 0; k < 8; ++k) {
        double x, y;
        do {
            x = 2 * uni() - 1;
            y = 2 * uni() - 1;
        } while (x * x + y * y >= 1);
        p.cx[k] = x;
        p.cy[k] = y;
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
// index); an unassigned node starts an aggregate and takes up to three
// unassigned neighbours, heaviest shared face first (ties: lower index); an
// aggregate of fewer than three elements then joins the neighbouring
// aggregate it shares the most face weight with (ties: lower aggregate;
// two triangles' nodes need not determine the nine Q2 modes of their box).  Aggregates keep their creation
// order.
static std::vector<int> greedy_agglomerate(int n, const Graph& adj, uint64_t seed, int* ncoarse) {
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
        cand.clear();
        for (auto& e : adj[u])
            if (agg[e.first] < 0) cand.push_back(e);
        std::sort(cand.begin(), cand.end(), [](const std::pair<int, double>& x, const std::pair<int, double>& y) {
            if (x.second != y.second) return x.second > y.second;
            return x.first < y.first;
        });
        for (size_t k = 0; k < cand.size() && k < 3; ++k) {
            agg[cand[k].first] = a;
            size[a]++;
        }
    }
    // aggregates of fewer than three elements join the neighbouring
    // aggregate they share the most face weight with (ties: lower aggregate)
    std::vector<std::vector<int>> members(size.size());
    for (int u = 0; u < n; ++u) members[agg[u]].push_back(u);
    for (int a = 0; a < (int)size.size(); ++a) {
        if (size[a] == 0 || size[a] >= 3) continue;
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

}  // namespace mg

namespace mg {

struct SBox {
    double lo[2], hi[2];
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

mgldg_problem* simplex_problem(mgldg_ctx* ctx, int np, const double* pts, int nt, const int* tris, int P, double tau0,
                               double tauD, int agg_levels, uint64_t agg_seed, std::vector<std::vector<int>>* parts) {
    MG_REQUIRE(P >= 1 && P <= 4, MGLDG_ERR_UNSUPPORTED, "P must be 1..4 on triangles");
    MG_REQUIRE(np >= 3 && nt >= 1 && pts && tris, MGLDG_ERR_ARG, "empty mesh");
    for (int k = 0; k < 3 * nt; ++k)
        MG_REQUIRE(tris[k] >= 0 && tris[k] < np, MGLDG_ERR_ARG, "vertex index out of range");
    const SMaster M2(2, P), M1(1, P);
    const int b = M2.b, P1 = M1.b;
    std::vector<STri> el(nt);
    for (int e = 0; e < nt; ++e) el[e] = make_stri(pts, tris + 3 * e);

    // ---- faces in first-encounter order (mesh.h:209-300) ----
    struct HF {
        int left, right, v0, v1;
        double n[2], area;
        int sl[6], sr[6];
    };
    std::vector<HF> faces;
    faces.reserve((size_t)nt * 2);
    std::unordered_map<uint64_t, int> f2f;
    f2f.reserve((size_t)nt * 4);
    for (int e = 0; e < nt; ++e)
        for (int j = 0; j < 3; ++j) {
            const int a = tris[3 * e + j], c = tris[3 * e + (j + 1) % 3];
            const uint64_t key = ((uint64_t)std::min(a, c) << 32) | (uint32_t)std::max(a, c);
            auto it = f2f.find(key);
            if (it == f2f.end()) {
                HF f{};
                f.left = e;
                f.right = -1;
                f.v0 = std::min(a, c);
                f.v1 = std::max(a, c);
                f2f.emplace(key, (int)faces.size());
                faces.push_back(f);
            } else {
                MG_REQUIRE(faces[it->second].right < 0, MGLDG_ERR_ARG, "an edge is shared by more than two triangles");
                faces[it->second].right = e;
            }
        }
    // local corner of a vertex in an element: reference coordinates
    // t0 -> (0,0), t1 -> (1,0), t2 -> (0,1)
    auto local = [&](int e, int v) {
        for (int i = 0; i < 3; ++i)
            if (tris[3 * e + i] == v) return i;
        return -1;
    };
    const int corner[3][2] = {{0, 0}, {1, 0}, {0, 1}};
    int nb = 0;
    for (HF& f : faces) {
        const double* p0 = pts + 2 * f.v0;
        const double* p1 = pts + 2 * f.v1;
        const double dx = p1[0] - p0[0], dy = p1[1] - p0[1];
        f.area = std::sqrt(dx * dx + dy * dy);
        double nrm[2] = {dy, -dx};
        const double len = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1]);
        nrm[0] /= len;
        nrm[1] /= len;
        int a = -1;
        for (int i = 0; i < 3; ++i) {
            const int v = tris[3 * f.left + i];
            if (v != f.v0 && v != f.v1) a = v;
        }
        const double in[2] = {pts[2 * a] - p0[0], pts[2 * a + 1] - p0[1]};
        if (nrm[0] * in[0] + nrm[1] * in[1] > 0) {
            nrm[0] = -nrm[0];
            nrm[1] = -nrm[1];
        }
        f.n[0] = nrm[0];
        f.n[1] = nrm[1];
        if (f.right < 0) {
            ++nb;
            continue;
        }
        // slicing: face node a at t = a/(P-1) from v0 to v1 is the element
        // node (1-t) corner(v0) + t corner(v1)
        for (int side = 0; side < 2; ++side) {
            const int e = side ? f.right : f.left;
            const int la = local(e, f.v0), lb = local(e, f.v1);
            for (int q = 0; q < P1; ++q) {
                int node;
                if (P == 1) {
                    node = 0;
                } else {
                    const int i0 = corner[la][0] * (P - 1 - q) + corner[lb][0] * q;
                    const int i1 = corner[la][1] * (P - 1 - q) + corner[lb][1] * q;
                    node = M2.index_of(i0, i1);
                }
                (side ? f.sr : f.sl)[q] = node;
            }
        }
    }
    const int nf = (int)faces.size();
    const int nfi = nf - nb;

    // ---- contributions: elements (M, G0, G1), interior faces (8), boundary (3)
    std::vector<int> interior, boundary;
    for (int k = 0; k < nf; ++k) (faces[k].right >= 0 ? interior : boundary).push_back(k);
    std::vector<int> slot(nf);
    for (int q = 0; q < nfi; ++q) slot[interior[q]] = q;
    for (int q = 0; q < nb; ++q) slot[boundary[q]] = q;
    const size_t bsz = (size_t)b * b;
    const int64_t c_elem = 0, c_face = (int64_t)3 * nt, c_bnd = c_face + (int64_t)8 * nfi;
    const int64_t ncontrib = c_bnd + (int64_t)3 * nb;

    // boundary blocks on the host (quadrature, mesh.h:312-351)
    std::vector<double> bvals((size_t)3 * nb * bsz);
    {
        std::vector<double> phl((size_t)MGLDG_QF * b), Lm((size_t)b * MGLDG_QF), LL(bsz), Minv(bsz);
        for (int q = 0; q < nb; ++q) {
            const HF& f = faces[boundary[q]];
            const STri& s = el[f.left];
            const double* p0 = pts + 2 * f.v0;
            const double* p1 = pts + 2 * f.v1;
            for (int k = 0; k < MGLDG_QF; ++k) {
                const double phys[2] = {p0[0] + (p1[0] - p0[0]) * kQuadNodes[k], p0[1] + (p1[1] - p0[1]) * kQuadNodes[k]};
                const double rel[2] = {phys[0] - s.p[0][0], phys[1] - s.p[0][1]};
                const double xl[2] = {s.Jinv[0][0] * rel[0] + s.Jinv[0][1] * rel[1],
                                      s.Jinv[1][0] * rel[0] + s.Jinv[1][1] * rel[1]};
                M2.eval(xl, &phl[(size_t)k * b]);
            }
            for (int a = 0; a < b; ++a)
                for (int k = 0; k < MGLDG_QF; ++k)
                    Lm[(size_t)a * MGLDG_QF + k] = phl[(size_t)k * b + a] * (kQuadWeights[k] * f.area);
            for (int a = 0; a < b; ++a)
                for (int c = 0; c < b; ++c) {
                    double sum = 0;
                    for (int k = 0; k < MGLDG_QF; ++k) sum += Lm[(size_t)a * MGLDG_QF + k] * phl[(size_t)k * b + c];
                    LL[(size_t)a * b + c] = sum;
                }
            const double jac = M2.volume / s.vol;
            for (size_t k = 0; k < bsz; ++k) Minv[k] = M2.invmass[k] * jac;
            for (int d = 0; d < 2; ++d) {
                double* G = &bvals[((size_t)3 * q + d) * bsz];
                const double sc = -f.n[d];
                for (int r = 0; r < b; ++r)
                    for (int c = 0; c < b; ++c) {
                        double sum = 0;
                        for (int k = 0; k < b; ++k) sum += (sc * Minv[(size_t)r * b + k]) * LL[(size_t)k * b + c];
                        G[(size_t)r * b + c] = sum;
                    }
            }
            double* T = &bvals[((size_t)3 * q + 2) * bsz];
            for (size_t k = 0; k < bsz; ++k) T[k] = tauD * LL[k];
        }
    }

    // per stored block, its contributions in the reference's order
    struct Tr {
        int row, col;
        int64_t seq, contrib;
    };
    std::vector<Tr> tm, tg[2], tt;
    int64_t seq = 0;
    for (int e = 0; e < nt; ++e) tm.push_back({e, e, seq++, c_elem + e});
    for (int d = 0; d < 2; ++d)
        for (int e = 0; e < nt; ++e) tg[d].push_back({e, e, seq++, c_elem + (int64_t)(1 + d) * nt + e});
    for (int k = 0; k < nf; ++k) {
        const HF& f = faces[k];
        if (f.right >= 0) {
            const int64_t base = c_face + (int64_t)8 * slot[k];
            for (int d = 0; d < 2; ++d) {
                tg[d].push_back({f.right, f.right, seq++, base + 2 * d});
                tg[d].push_back({f.right, f.left, seq++, base + 2 * d + 1});
            }
            tt.push_back({f.right, f.right, seq++, base + 4});
            tt.push_back({f.left, f.left, seq++, base + 5});
            tt.push_back({f.right, f.left, seq++, base + 6});
            tt.push_back({f.left, f.right, seq++, base + 7});
        } else {
            const int64_t base = c_bnd + (int64_t)3 * slot[k];
            for (int d = 0; d < 2; ++d) tg[d].push_back({f.left, f.left, seq++, base + d});
            tt.push_back({f.left, f.left, seq++, base + 2});
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
    MG_REQUIRE(ncontrib < (int64_t)1 << 31, MGLDG_ERR_UNSUPPORTED, "mesh too large for the contribution index");
    const Assembly AM = assemble(tm), AG0 = assemble(tg[0]), AG1 = assemble(tg[1]), AT = assemble(tt);

    // ---- GPU: contributions, then the operators ----
    mgldg_problem* pr = new mgldg_problem();
    pr->ctx = ctx;
    pr->P = P;
    pr->b = b;
    pr->ne = nt;
    pr->n = 0;
    pr->simplex = true;
    pr->nfaces = nf;
    pr->nbfaces = nb;
    double *d_contrib = nullptr, *d_geom = nullptr, *d_ref = nullptr;
    FaceDev* d_faces = nullptr;
    mgldg_bsr *M = nullptr, *G0 = nullptr, *G1 = nullptr, *Tm = nullptr;
    try {
        std::vector<double> geom((size_t)nt * 11);
        for (int e = 0; e < nt; ++e) {
            double* g = &geom[(size_t)e * 11];
            g[0] = el[e].p[0][0];
            g[1] = el[e].p[0][1];
            g[2] = el[e].J[0][0]; g[3] = el[e].J[0][1]; g[4] = el[e].J[1][0]; g[5] = el[e].J[1][1];
            g[6] = el[e].Jinv[0][0]; g[7] = el[e].Jinv[0][1]; g[8] = el[e].Jinv[1][0]; g[9] = el[e].Jinv[1][1];
            g[10] = el[e].vol;
        }
        std::vector<FaceDev> fd(nfi);
        for (int q = 0; q < nfi; ++q) {
            const HF& f = faces[interior[q]];
            FaceDev& D = fd[q];
            D.left = f.left;
            D.right = f.right;
            D.n0 = f.n[0];
            D.n1 = f.n[1];
            D.area = f.area;
            D.volR = el[f.right].vol;
            for (int a = 0; a < 6; ++a) {
                D.sl[a] = a < P1 ? f.sl[a] : -1;
                D.sr[a] = a < P1 ? f.sr[a] : -1;
            }
        }
        // reference tables: Mref | D0 | D1 | Minv | M1 | nodes
        std::vector<double> ref;
        ref.insert(ref.end(), M2.mass.begin(), M2.mass.end());
        ref.insert(ref.end(), M2.diff[0].begin(), M2.diff[0].end());
        ref.insert(ref.end(), M2.diff[1].begin(), M2.diff[1].end());
        ref.insert(ref.end(), M2.invmass.begin(), M2.invmass.end());
        ref.insert(ref.end(), M1.mass.begin(), M1.mass.end());
        ref.insert(ref.end(), M2.nodes.begin(), M2.nodes.end());
        d_geom = dalloc<double>(geom.size());
        d_ref = dalloc<double>(ref.size());
        d_faces = dalloc<FaceDev>(std::max(1, nfi));
        d_contrib = dalloc<double>((size_t)ncontrib * bsz);
        upload(ctx, d_geom, geom.data(), geom.size());
        upload(ctx, d_ref, ref.data(), ref.size());
        if (nfi) upload(ctx, d_faces, fd.data(), fd.size());
        if (nb) upload(ctx, d_contrib + (size_t)c_bnd * bsz, bvals.data(), bvals.size());
        const double* dM = d_ref;
        const double* dD0 = d_ref + bsz;
        const double* dD1 = d_ref + 2 * bsz;
        const double* dMinv = d_ref + 3 * bsz;
        const double* dM1 = d_ref + 4 * bsz;
        {
            const int64_t tot = (int64_t)nt * bsz;
            const int g = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, ctx->sm_count * 32));
            Launch L(ctx, MGLDG_K_SETUP);
            k_simplex_elem<<<g, 256, 0, ctx->stream>>>(nt, b, d_geom, dM, dD0, dD1, M2.volume, d_contrib);
        }
        check_launch();
        if (nfi) {
            const int64_t tot = (int64_t)nfi * 8 * bsz;
            const int g = (int)std::max<int64_t>(1, std::min<int64_t>((tot + 255) / 256, ctx->sm_count * 32));
            Launch L(ctx, MGLDG_K_SETUP);
            k_simplex_face<<<g, 256, 0, ctx->stream>>>(nfi, b, P1, d_faces, dM1, dMinv, M2.volume, tau0,
                                                       d_contrib + (size_t)c_face * bsz);
        }
        check_launch();
        M = realize(ctx, AM, nt, b, d_contrib);
        G0 = realize(ctx, AG0, nt, b, d_contrib);
        G1 = realize(ctx, AG1, nt, b, d_contrib);
        Tm = realize(ctx, AT, nt, b, d_contrib);
        pr->ops = new mgldg_ops();
        pr->ops->ctx = ctx;
        pr->ops->ndim = 2;
        pr->ops->M = M; M = nullptr;
        pr->ops->G[0] = G0; G0 = nullptr;
        pr->ops->G[1] = G1; G1 = nullptr;
        pr->ops->T = Tm; Tm = nullptr;
        construct_laplacian(ctx, pr->ops);
        // geometry for right-hand sides and dumps
        pr->sgeom = geom;
        pr->snodes = M2.nodes;
        pr->d_geom = d_geom; d_geom = nullptr;
        pr->d_nodes = dalloc<double>(M2.nodes.size());
        upload(ctx, pr->d_nodes, M2.nodes.data(), M2.nodes.size());
        pr->d_Mref = dalloc<double>(bsz);
        upload(ctx, pr->d_Mref, M2.mass.data(), bsz);
        pr->svref = M2.volume;

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
            for (int d = 0; d < 2; ++d) {
                box[e].lo[d] = box[e].hi[d] = el[e].p[0][d];
                for (int j = 1; j < 3; ++j) {
                    box[e].lo[d] = std::min(box[e].lo[d], el[e].p[j][d]);
                    box[e].hi[d] = std::max(box[e].hi[d], el[e].p[j][d]);
                }
            }
        const Ref2 CR(P);
        const int cb = P * P;
        int nfine = nt;
        for (int lev = 0; lev < agg_levels && nfine > 1; ++lev) {
            int nc = 0;
            std::vector<int> agg = greedy_agglomerate(nfine, adj, agg_seed + (uint64_t)lev, &nc);
            if (nc >= nfine) break;
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
                for (int d = 0; d < 2; ++d) {
                    cbox[a].lo[d] = std::min(cbox[a].lo[d], src[u].lo[d]);
                    cbox[a].hi[d] = std::max(cbox[a].hi[d], src[u].hi[d]);
                }
            }
            const int br = lev == 0 ? b : cb;
            std::vector<double> vals((size_t)nfine * br * cb);
            for (int u = 0; u < nfine; ++u) {
                const int a = agg[u];
                const SBox& B = cbox[a];
                const double w[2] = {B.hi[0] - B.lo[0], B.hi[1] - B.lo[1]};
                double* E = &vals[(size_t)u * br * cb];
                if (lev == 0) {
                    double rp[3][2];
                    for (int j = 0; j < 3; ++j)
                        for (int d = 0; d < 2; ++d) rp[j][d] = (el[u].p[j][d] - B.lo[d]) / w[d];
                    for (int i = 0; i < b; ++i) {
                        double x[2];
                        for (int d = 0; d < 2; ++d)
                            x[d] = rp[0][d] + ((rp[1][d] - rp[0][d]) * M2.nodes[2 * i] +
                                               (rp[2][d] - rp[0][d]) * M2.nodes[2 * i + 1]);
                        CR.lagrange2(x, E + (size_t)i * cb);
                    }
                } else if (cnt[a] == 1) {
                    for (int i = 0; i < cb; ++i) E[(size_t)i * cb + i] = 1.0;
                } else {
                    const SBox& F = src[u];
                    double rlo[2], rhi[2];
                    for (int d = 0; d < 2; ++d) {
                        rlo[d] = (F.lo[d] - B.lo[d]) / w[d];
                        rhi[d] = (F.hi[d] - B.lo[d]) / w[d];
                    }
                    for (int i0 = 0; i0 < P; ++i0)
                        for (int i1 = 0; i1 < P; ++i1) {
                            const double x[2] = {rlo[0] + (rhi[0] - rlo[0]) * CR.nodes[i0],
                                                 rlo[1] + (rhi[1] - rlo[1]) * CR.nodes[i1]};
                            CR.lagrange2(x, E + (size_t)(i0 * P + i1) * cb);
                        }
                }
            }
            pr->T.push_back(host_bsr(ctx, nfine, nc, br, cb, agg, vals));
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
        delete M; delete G0; delete G1; delete Tm;
        delete pr;
        throw;
    }
    dfree(d_contrib);
    dfree(d_ref);
    dfree(d_faces);
    return pr;
}

void simplex_rhs_dev(mgldg_ctx* ctx, const mgldg_problem* pr, uint64_t seed, double* b) {
    const GaussDevS g = gaussian_disk(seed);
    const int grid = std::max(1, std::min(pr->ne, ctx->sm_count * 32));
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_rhs_simplex<<<grid, 64, pr->b * sizeof(double), ctx->stream>>>(pr->ne, pr->b, pr->d_geom, pr->d_nodes,
                                                                         pr->d_Mref, pr->svref, g, b);
    }
    check_launch();
}

// Disk mesher (no reference counterpart; the reference reads distmesh
// output): concentric rings of radius k/K (K = ceil(1/h)), ring k with
// max(6k, round(2 pi k)) equally spaced points starting at angle 0, and the
// strip between rings k-1 and k triangulated by advancing whichever ring's
// next point has the smaller angle.  Counter-clockwise triangles.
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
extern "C" int mgldg_mesh_read(const char* path, int* np, int* nt, double* p, int* t) {
    if (!path || !np || !nt) return MGLDG_ERR_ARG;
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
        double v[2];
        int k = 0;
        double x;
        while (ss >> x) {
            if (k < 2) v[k] = x;
            ++k;
        }
        if (k != 2 || ip >= n_p) return MGLDG_ERR_ARG;
        if (p) {
            p[2 * ip] = v[0];
            p[2 * ip + 1] = v[1];
        }
        ++ip;
    }
    while (std::getline(ifs, line) && !line.empty()) {
        std::istringstream ss(line);
        int v[3];
        int k = 0;
        int x;
        while (ss >> x) {
            if (k < 3) v[k] = x;
            ++k;
        }
        if (k != 3 || it >= n_t) return MGLDG_ERR_ARG;
        for (int j = 0; j < 3; ++j)
            if (v[j] < 1 || v[j] > n_p) return MGLDG_ERR_ARG;
        if (t)
            for (int j = 0; j < 3; ++j) t[3 * it + j] = v[j] - 1;
        ++it;
    }
    if (ip != n_p || it != n_t) return MGLDG_ERR_SHAPE;
    *np = n_p;
    *nt = n_t;
    return MGLDG_OK;
}

extern "C" int mgldg_simplex_problem_create(mgldg_ctx* ctx, int np, const double* p, int nt, const int* t, int P,
                                            double tau0, double tauD, int agg_levels, uint64_t agg_seed,
                                            mgldg_problem** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(out != nullptr && agg_levels >= 0, MGLDG_ERR_ARG, "bad arguments");
    *out = nullptr;
    std::vector<std::vector<int>> parts;
    mgldg_problem* pr = simplex_problem(ctx, np, p, nt, t, P, tau0, tauD, agg_levels, agg_seed, &parts);
    pr->partitions = std::move(parts);
    *out = pr;
    MG_API_END
}

extern "C" int mgldg_problem_partition(const mgldg_problem* pr, int l, int* n, int* agg) {
    if (!pr || !n || l < 0 || l >= (int)pr->partitions.size()) return MGLDG_ERR_ARG;
    const std::vector<int>& a = pr->partitions[l];
    *n = (int)a.size();
    if (agg) std::copy(a.begin(), a.end(), agg);
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

// quadtree.cu -- adaptive quadtrees on [0,1]^2 and their LDG problems.
//
// Reference: Quadtree<2>(h) (src/cartesian/mesh/quadtree.tpp:10-40, layers
// and leaves quadtree.h:164-186, neighbour search quadtree.tpp:44-114), Mesh
// faces (mesh.h:186-264) with canonical and non-canonical faces
// (mesh.h:21-79) and their lifting matrices (mesh.h:282-352),
// LDGPoisson::discretize (ldgpoisson.tpp:27-100) and the h-interpolation
// hierarchy over the tree's layers (interpolationhierarchy.h:30-82).
//
// Cells are kept as integers (level, ix, iy): the cell is
// [ix, ix+1] x [iy, iy+1] * 2^-level, so every coordinate the reference
// computes by halving is exact here as well.  Neighbours are found through a
// hash of (level, ix, iy) instead of the reference's walk from the root; the
// lists come out in the same depth-first order.  The LDG blocks are sums of
// a few distinct contributions (per element size, face geometry and kind);
// the host computes each distinct block once with the reference's
// arithmetic, lists per stored block the contributions in the reference's
// order, and the GPU sums them (k_sum_blocks), as for uniform grids.
//
// Extensions (no reference counterpart): optional 2:1 face balance (a leaf
// is split while a face-neighbour leaf is two or more levels finer; only
// forced splits, so the result is the unique coarsest balanced refinement)
// and optional per-face penalties tau0/min(h_L, h_R), tauD/h_L.  Boundary
// conditions are homogeneous Dirichlet.
#include <algorithm>
#include <cmath>
#include <map>
#include <random>
#include <unordered_map>

#include "api.cuh"
#include "ldg_build.cuh"

using namespace mg;

struct mgldg_quadtree {
    struct Node {
        int level;
        uint32_t ix, iy;
        int parent;
        int child[4];
        int height;
    };
    std::vector<Node> nodes;
    std::unordered_map<uint64_t, int> at;
    int numLevels = 1;
    int strategy = MGLDG_COARSEN_EQUAL;
};

namespace mg {

using QT = mgldg_quadtree;
constexpr int kMaxTreeLevel = 24;

static uint64_t qkey(int L, uint32_t ix, uint32_t iy) {
    return ((uint64_t)L << 56) | ((uint64_t)ix << 28) | (uint64_t)iy;
}
static bool qleaf(const QT& t, int id) { return t.nodes[id].child[0] < 0; }
static double qwidth(int L) { return std::ldexp(1.0, -L); }

static int qt_add(QT& t, int L, uint32_t ix, uint32_t iy, int parent) {
    QT::Node n;
    n.level = L;
    n.ix = ix;
    n.iy = iy;
    n.parent = parent;
    n.child[0] = n.child[1] = n.child[2] = n.child[3] = -1;
    n.height = 0;
    const int id = (int)t.nodes.size();
    t.nodes.push_back(n);
    t.at[qkey(L, ix, iy)] = id;
    return id;
}

// children in the order b0*2 + b1, bit i set = upper half in dimension i
// (quadtree.tpp:18-31)
static void qt_split(QT& t, int id) {
    const int L = t.nodes[id].level;
    MG_REQUIRE(L < kMaxTreeLevel, MGLDG_ERR_ARG, "quadtree deeper than 24 levels");
    const uint32_t ix = t.nodes[id].ix, iy = t.nodes[id].iy;
    for (int b0 = 0; b0 < 2; ++b0)
        for (int b1 = 0; b1 < 2; ++b1) {
            const int c = qt_add(t, L + 1, 2 * ix + b0, 2 * iy + b1, id);
            t.nodes[id].child[b0 * 2 + b1] = c;
        }
}

static void qt_finish(QT& t) {
    t.numLevels = 1;
    // children are created after their parents
    for (int id = (int)t.nodes.size() - 1; id >= 0; --id) {
        QT::Node& n = t.nodes[id];
        n.height = 0;
        if (n.child[0] >= 0)
            for (int k = 0; k < 4; ++k) n.height = std::max(n.height, t.nodes[n.child[k]].height + 1);
        t.numLevels = std::max(t.numLevels, n.level + 1);
    }
}

// Quadtree<2>(h): split while the width exceeds h(centre) (quadtree.tpp:10-40)
static void qt_build(QT& t, mgldg_h_fn h, void* user) {
    qt_add(t, 0, 0, 0, -1);
    std::vector<int> stack{0};
    while (!stack.empty()) {
        const int id = stack.back();
        stack.pop_back();
        const QT::Node n = t.nodes[id];
        const double w = qwidth(n.level);
        const double mid[2] = {n.ix * w + w / 2, n.iy * w + w / 2};
        const double hv = h(mid, user);
        if (w > hv) {
            qt_split(t, id);
            for (int k = 3; k >= 0; --k) stack.push_back(t.nodes[id].child[k]);
        }
    }
}

// the face-neighbour node at the same level, or -1 (outside or absent)
static int same_level_neighbor(const QT& t, int id, int dim, int dir) {
    const QT::Node& n = t.nodes[id];
    int64_t c[2] = {n.ix, n.iy};
    c[dim] += dir;
    if (c[dim] < 0 || c[dim] >= ((int64_t)1 << n.level)) return -1;
    auto it = t.at.find(qkey(n.level, (uint32_t)c[0], (uint32_t)c[1]));
    return it == t.at.end() ? -1 : it->second;
}

// 2:1 face balance (extension)
static void qt_balance(QT& t) {
    bool changed = true;
    while (changed) {
        changed = false;
        std::vector<int> leaves;
        for (int id = 0; id < (int)t.nodes.size(); ++id)
            if (qleaf(t, id)) leaves.push_back(id);
        for (int id : leaves) {
            bool need = false;
            for (int dim = 0; dim < 2 && !need; ++dim)
                for (int dir = -1; dir <= 1 && !need; dir += 2) {
                    const int m = same_level_neighbor(t, id, dim, dir);
                    if (m < 0 || qleaf(t, m)) continue;
                    // m's children that touch this cell: bit `dim` = 0 if m is
                    // on the upper side, 1 if on the lower side
                    const int side = dir > 0 ? 0 : 1;
                    for (int k = 0; k < 4; ++k) {
                        const int bit = dim == 0 ? (k >> 1) : (k & 1);
                        if (bit == side && !qleaf(t, t.nodes[m].child[k])) need = true;
                    }
                }
            if (need) {
                qt_split(t, id);
                changed = true;
            }
        }
    }
}

// QuadTree::isLeaf (quadtree.h:164-173)
static bool qt_is_leaf(const QT& t, int id, int c) {
    const QT::Node& n = t.nodes[id];
    if (t.strategy == MGLDG_COARSEN_RAPID)
        return n.height == c || (n.height < c && n.parent >= 0 && t.nodes[n.parent].height > c);
    const int cl = t.numLevels - 1 - c;
    return n.level == cl || (n.level < cl && n.height == 0);
}

// QuadTree::layer (quadtree.h:176-186): depth-first, children in order
static std::vector<int> qt_layer(const QT& t, int c) {
    std::vector<int> out, stack{0};
    while (!stack.empty()) {
        const int id = stack.back();
        stack.pop_back();
        if (qt_is_leaf(t, id, c)) {
            out.push_back(id);
            continue;
        }
        if (qleaf(t, id)) continue;
        for (int k = 3; k >= 0; --k) stack.push_back(t.nodes[id].child[k]);
    }
    return out;
}

// leaves of the subtree of id that touch its `side` face in dimension dim,
// depth first
static void face_leaves(const QT& t, int id, int dim, int side, std::vector<int>& out) {
    if (qleaf(t, id)) {
        out.push_back(id);
        return;
    }
    for (int k = 0; k < 4; ++k) {
        const int bit = dim == 0 ? (k >> 1) : (k & 1);
        if (bit == side) face_leaves(t, t.nodes[id].child[k], dim, side, out);
    }
}

// QuadTree::neighbors(gid, dim, dir, 0) on the leaf layer (quadtree.tpp:44-114)
static void qt_neighbors(const QT& t, int id, int dim, int dir, std::vector<int>& out) {
    out.clear();
    const QT::Node& n = t.nodes[id];
    int64_t c[2] = {n.ix, n.iy};
    c[dim] += dir;
    if (c[dim] < 0 || c[dim] >= ((int64_t)1 << n.level)) return;
    for (int L = n.level; L >= 0; --L) {
        auto it = t.at.find(qkey(L, (uint32_t)c[0], (uint32_t)c[1]));
        if (it != t.at.end()) {
            if (L == n.level) face_leaves(t, it->second, dim, dir > 0 ? 0 : 1, out);
            else out.push_back(it->second);   // a coarser leaf
            return;
        }
        c[0] >>= 1;
        c[1] >>= 1;
    }
}

// ---------------------------------------------------------------- assembly
struct Triple {
    int row, col, seq, contrib;
};

struct FaceMats {
    Blk LL, RR, RL;
};

struct Builder {
    const Ref2& R;
    int P, b;
    double tau0, tauD;
    bool per_face;
    std::vector<Blk> table;
    std::map<std::vector<double>, int> index;
    std::map<std::vector<double>, FaceMats> faces;
    Blk mass_ref, invmass_ref;
    Builder(const Ref2& R_, double t0, double tD, bool pf)
        : R(R_), P(R_.P), b(R_.b), tau0(t0), tauD(tD), per_face(pf) {
        mass_ref = R.tensor(R.mass1);
        invmass_ref = R.tensor(R.invmass1);
    }
    template <class F>
    int get(const std::vector<double>& key, F make) {
        auto it = index.find(key);
        if (it != index.end()) return it->second;
        table.push_back(make());
        const int id = (int)table.size() - 1;
        index.emplace(key, id);
        return id;
    }
    Blk invmass(int L) const {
        const double w = qwidth(L);
        double vol = 1;
        vol *= w;
        vol *= w;
        return bscale(1 / vol, invmass_ref);
    }
    // slicing form of a canonical interior face (mesh.h:285-310)
    FaceMats canonical(int dim, int L) const {
        const double area = qwidth(L);
        FaceMats f{Blk((size_t)b * b, 0.0), Blk((size_t)b * b, 0.0), Blk((size_t)b * b, 0.0)};
        int jl[8], jr[8];
        for (int a = 0; a < P; ++a) {
            int jt[2];
            jt[1 - dim] = a;
            jt[dim] = P - 1;
            jl[a] = jt[0] * P + jt[1];
            jt[dim] = 0;
            jr[a] = jt[0] * P + jt[1];
        }
        for (int a = 0; a < P; ++a)
            for (int c = 0; c < P; ++c) {
                const double m = R.mass1[a * P + c] * area;
                f.LL[(size_t)jl[a] * b + jl[c]] = m;
                f.RR[(size_t)jr[a] * b + jr[c]] = m;
                f.RL[(size_t)jr[a] * b + jl[c]] = m;
            }
        return f;
    }
    // quadrature form (mesh.h:312-351): tl/tr are the tangential reference
    // coordinates of the quadrature points on the left / right element,
    // ldim/rdim the normal coordinate of each side
    FaceMats quad(int dim, double area, double al, double bl, double ar, double br, double lnorm,
                  double rnorm) const {
        std::vector<double> phl((size_t)MGLDG_QF * b), phr((size_t)MGLDG_QF * b), w(MGLDG_QF);
        for (int q = 0; q < MGLDG_QF; ++q) {
            const double x = kQuadNodes[q];
            double ql[2], qr[2];
            ql[1 - dim] = al + (bl - al) * x;
            qr[1 - dim] = ar + (br - ar) * x;
            ql[dim] = lnorm;
            qr[dim] = rnorm;
            R.lagrange2(ql, &phl[(size_t)q * b]);
            R.lagrange2(qr, &phr[(size_t)q * b]);
            w[q] = 1;
            w[q] *= kQuadWeights[q];
        }
        for (int q = 0; q < MGLDG_QF; ++q) w[q] *= area;
        FaceMats f{Blk((size_t)b * b), Blk((size_t)b * b), Blk((size_t)b * b)};
        for (int a = 0; a < b; ++a)
            for (int c = 0; c < b; ++c) {
                double sll = 0, srr = 0, srl = 0;
                for (int q = 0; q < MGLDG_QF; ++q) {
                    const double lw = phl[(size_t)q * b + a] * w[q];
                    const double rw = phr[(size_t)q * b + a] * w[q];
                    sll += lw * phl[(size_t)q * b + c];
                    srr += rw * phr[(size_t)q * b + c];
                    srl += rw * phl[(size_t)q * b + c];
                }
                f.LL[(size_t)a * b + c] = sll;
                f.RR[(size_t)a * b + c] = srr;
                f.RL[(size_t)a * b + c] = srl;
            }
        return f;
    }
    template <class F>
    const FaceMats& face(const std::vector<double>& key, F make) {
        auto it = faces.find(key);
        if (it != faces.end()) return it->second;
        return faces.emplace(key, make()).first->second;
    }
};

}  // namespace mg

namespace mg {

static mgldg_problem* quadtree_problem(mgldg_ctx* ctx, const QT& t, int P, double tau0, double tauD,
                                       bool per_face) {
    MG_REQUIRE(P >= 1 && P <= 5, MGLDG_ERR_UNSUPPORTED, "P must be 1..5 (block size <= 25)");
    const Ref2 R(P);
    const int b = R.b;
    Builder B(R, tau0, tauD, per_face);

    // elements: the leaf layer in depth-first order (mesh.h:197-207)
    const std::vector<int> elems = qt_layer(t, 0);
    const int ne = (int)elems.size();
    std::unordered_map<int, int> g2l;
    g2l.reserve(elems.size() * 2);
    for (int l = 0; l < ne; ++l) g2l[elems[l]] = l;
    auto lev = [&](int lid) { return t.nodes[elems[lid]].level; };

    std::vector<Triple> tm, tg[2], tt;
    int seq = 0;
    // construct_mass_matrix and construct_broken_gradient (ldgpoisson.tpp:27-60)
    for (int e = 0; e < ne; ++e) {
        const int L = lev(e);
        const int c = B.get({0, (double)L}, [&] {
            const double w = qwidth(L);
            double vol = 1;
            vol *= w;
            vol *= w;
            return bscale(vol, B.mass_ref);
        });
        tm.push_back({e, e, seq++, c});
    }
    for (int d = 0; d < 2; ++d)
        for (int e = 0; e < ne; ++e) {
            const int L = lev(e);
            const int c = B.get({1, (double)d, (double)L}, [&] { return bscale(1.0 / qwidth(L), R.diff(d)); });
            tg[d].push_back({e, e, seq++, c});
        }

    // faces in the reference's order (mesh.h:210-261) and their lifting
    // and penalty terms (ldgpoisson.tpp:63-100)
    int nfaces = 0, nb = 0;
    std::vector<int> nbrs;
    for (int lid = 0; lid < ne; ++lid) {
        const int gid = elems[lid];
        for (int dim = 0; dim < 2; ++dim) {
            for (int dir = -1; dir <= 1; dir += 2) {
                qt_neighbors(t, gid, dim, dir, nbrs);
                if (nbrs.empty()) {
                    // boundary face, outward normal dir, quadrature form with
                    // the canonical nodes on the element's side
                    ++nfaces;
                    ++nb;
                    const int L = lev(lid);
                    const double nrm = dir;
                    const FaceMats& F = B.face({10, (double)dim, (double)dir, (double)L}, [&] {
                        const double side = nrm > 0 ? 1.0 : 0.0;
                        return B.quad(dim, qwidth(L), 0.0, 1.0, 0.0, 1.0, side, 1.0 - side);
                    });
                    const double tD = per_face ? tauD / qwidth(L) : tauD;
                    const int cg = B.get({20, (double)dim, nrm, (double)L},
                                         [&] { return bmul(bscale(-nrm, B.invmass(L)), F.LL, b); });
                    const int ct = B.get({21, (double)dim, nrm, (double)L, tD}, [&] { return bscale(tD, F.LL); });
                    tg[dim].push_back({lid, lid, seq++, cg});
                    tt.push_back({lid, lid, seq++, ct});
                    continue;
                }
                for (int ngid : nbrs) {
                    const int nlid = g2l.at(ngid);
                    if (!(lid < nlid)) continue;
                    ++nfaces;
                    const int left = dir < 0 ? nlid : lid, right = dir > 0 ? nlid : lid;
                    const QT::Node& nl = t.nodes[elems[left]];
                    const QT::Node& nr = t.nodes[elems[right]];
                    const int Ll = nl.level, Lr = nr.level;
                    const double wl = qwidth(Ll), wr = qwidth(Lr);
                    const int tg_ = 1 - dim;
                    const double lol = (tg_ == 0 ? nl.ix : nl.iy) * wl, lor = (tg_ == 0 ? nr.ix : nr.iy) * wr;
                    const double flo = std::max(lol, lor), fhi = std::min(lol + wl, lor + wr);
                    const double area = fhi - flo;
                    const bool canonical = Ll == Lr;
                    std::vector<double> fkey;
                    const FaceMats* Fp;
                    if (canonical) {
                        fkey = {11, (double)dim, (double)Ll};
                        Fp = &B.face(fkey, [&] { return B.canonical(dim, Ll); });
                    } else {
                        const double al = (flo - lol) / wl, bl = (fhi - lol) / wl;
                        const double ar = (flo - lor) / wr, br = (fhi - lor) / wr;
                        fkey = {12, (double)dim, (double)Ll, (double)Lr, al, bl, ar, br};
                        Fp = &B.face(fkey, [&] { return B.quad(dim, area, al, bl, ar, br, 1.0, 0.0); });
                    }
                    const FaceMats& F = *Fp;
                    const double tau = per_face ? tau0 / std::min(wl, wr) : tau0;
                    auto key = [&](double kind, std::initializer_list<double> extra) {
                        std::vector<double> k = fkey;
                        k.push_back(kind);
                        k.insert(k.end(), extra);
                        return k;
                    };
                    const int cgrr = B.get(key(30, {}), [&] { return bmul(bscale(1.0, B.invmass(Lr)), F.RR, b); });
                    const int cgrl = B.get(key(31, {}), [&] { return bmul(bscale(-1.0, B.invmass(Lr)), F.RL, b); });
                    const int ctrr = B.get(key(32, {tau}), [&] { return bscale(tau, F.RR); });
                    const int ctll = B.get(key(33, {tau}), [&] { return bscale(tau, F.LL); });
                    const int ctrl = B.get(key(34, {tau}), [&] { return bscale(-tau, F.RL); });
                    const int ctlr = B.get(key(35, {tau}), [&] { return bscale(-tau, btrans(F.RL, b)); });
                    tg[dim].push_back({right, right, seq++, cgrr});
                    tg[dim].push_back({right, left, seq++, cgrl});
                    tt.push_back({right, right, seq++, ctrr});
                    tt.push_back({left, left, seq++, ctll});
                    tt.push_back({right, left, seq++, ctrl});
                    tt.push_back({left, right, seq++, ctlr});
                }
            }
        }
    }

    // per stored block, its contributions in order
    auto assemble = [&](std::vector<Triple>& v) {
        std::sort(v.begin(), v.end(), [](const Triple& a, const Triple& c) {
            if (a.row != c.row) return a.row < c.row;
            if (a.col != c.col) return a.col < c.col;
            return a.seq < c.seq;
        });
        Assembly As;
        As.row_ptr.assign(ne + 1, 0);
        size_t k = 0;
        for (int r = 0; r < ne; ++r) {
            while (k < v.size() && v[k].row == r) {
                const int col = v[k].col;
                std::vector<int> cs;
                while (k < v.size() && v[k].row == r && v[k].col == col) cs.push_back(v[k++].contrib);
                As.add_block_v(col, cs);
            }
            As.row_ptr[r + 1] = (int)As.col_idx.size();
        }
        return As;
    };
    const Assembly AM = assemble(tm), AG0 = assemble(tg[0]), AG1 = assemble(tg[1]), AT = assemble(tt);

    mgldg_problem* pr = new mgldg_problem();
    pr->ctx = ctx;
    pr->P = P;
    pr->b = b;
    pr->ne = ne;
    pr->n = 0;
    pr->nfaces = nfaces;
    pr->nbfaces = nb;
    pr->nlevels = t.numLevels;
    double* d_table = nullptr;
    mgldg_bsr *M = nullptr, *G0 = nullptr, *G1 = nullptr, *Tm = nullptr;
    try {
        std::vector<double> flat;
        for (auto& blk : B.table) flat.insert(flat.end(), blk.begin(), blk.end());
        d_table = dalloc<double>(std::max<size_t>(1, flat.size()));
        upload(ctx, d_table, flat.data(), flat.size());
        M = realize(ctx, AM, ne, b, d_table);
        G0 = realize(ctx, AG0, ne, b, d_table);
        G1 = realize(ctx, AG1, ne, b, d_table);
        Tm = realize(ctx, AT, ne, b, d_table);
        pr->ops = new mgldg_ops();
        pr->ops->ctx = ctx;
        pr->ops->ndim = 2;
        pr->ops->M = M; M = nullptr;
        pr->ops->G[0] = G0; G0 = nullptr;
        pr->ops->G[1] = G1; G1 = nullptr;
        pr->ops->T = Tm; Tm = nullptr;
        construct_laplacian(ctx, pr->ops);
        pr->ex.resize(ne);
        pr->ey.resize(ne);
        pr->ew.resize(ne);
        for (int e = 0; e < ne; ++e) {
            const QT::Node& n = t.nodes[elems[e]];
            const double w = qwidth(n.level);
            pr->ex[e] = n.ix * w;
            pr->ey[e] = n.iy * w;
            pr->ew[e] = w;
        }
        problem_upload_geometry(ctx, pr);

        // h-interpolation hierarchy over the layers (interpolationhierarchy.h:30-82):
        // a fine element that is also on the coarse layer gets the identity,
        // any other one its parent's basis at its own nodes (child position
        // k = b0*2 + b1 -> lower corner (b0/2, b1/2))
        std::vector<double> E5((size_t)5 * b * b, 0.0);
        for (int cpos = 0; cpos < 4; ++cpos) {
            const double lo[2] = {0.5 * (cpos >> 1), 0.5 * (cpos & 1)};
            for (int i0 = 0; i0 < P; ++i0)
                for (int i1 = 0; i1 < P; ++i1) {
                    double node[2];
                    const int idx[2] = {i0, i1};
                    for (int d = 0; d < 2; ++d) node[d] = lo[d] + 0.5 * R.nodes[idx[d]];
                    R.lagrange2(node, &E5[(size_t)cpos * b * b + (size_t)(i0 * P + i1) * b]);
                }
        }
        for (int a = 0; a < b; ++a) E5[(size_t)4 * b * b + (size_t)a * b + a] = 1.0;
        std::vector<int> fine = elems;
        for (int l = 0; l + 1 < t.numLevels; ++l) {
            const std::vector<int> coarse = qt_layer(t, l + 1);
            std::unordered_map<int, int> cmap;
            cmap.reserve(coarse.size() * 2);
            for (int k = 0; k < (int)coarse.size(); ++k) cmap[coarse[k]] = k;
            std::vector<int> col(fine.size()), blk(fine.size());
            for (size_t k = 0; k < fine.size(); ++k) {
                const int g = fine[k];
                if (qt_is_leaf(t, g, l + 1)) {
                    col[k] = cmap.at(g);
                    blk[k] = 4;
                } else {
                    const int p = t.nodes[g].parent;
                    col[k] = cmap.at(p);
                    int pos = 0;
                    while (t.nodes[p].child[pos] != g) ++pos;
                    blk[k] = pos;
                }
            }
            pr->T.push_back(table_operator(ctx, (int)fine.size(), (int)coarse.size(), b, b, col, blk, E5));
            fine = coarse;
        }
        sync(ctx);
    } catch (...) {
        dfree(d_table);
        delete M; delete G0; delete G1; delete Tm;
        delete pr;
        throw;
    }
    dfree(d_table);
    return pr;
}

}  // namespace mg

// ================================================================== C ABI ==
extern "C" double mgldg_h_points(const double* x, void* user) {
    const mgldg_points_rule* r = (const mgldg_points_rule*)user;
    double d = 1e300;
    for (int k = 0; k < r->npoints; ++k) {
        const double dx = x[0] - r->points[2 * k], dy = x[1] - r->points[2 * k + 1];
        d = std::min(d, std::sqrt(dx * dx + dy * dy));
    }
    const double lo = std::ldexp(1.0, -(r->base_level + r->extra_levels)), hi = std::ldexp(1.0, -r->base_level);
    return std::min(hi, std::max(lo, d / (r->radius * std::ldexp(1.0, r->base_level))));
}

extern "C" int mgldg_seeded_points(uint64_t seed, int n, double* xy) {
    if (n < 0 || (n > 0 && !xy)) return MGLDG_ERR_ARG;
    std::mt19937_64 g(seed);
    for (int k = 0; k < 2 * n; ++k) xy[k] = (double)(g() >> 11) * 0x1.0p-53;
    return MGLDG_OK;
}

extern "C" int mgldg_quadtree_create(mgldg_h_fn h, void* user, int balance, int strategy, mgldg_quadtree** out) {
    if (!h || !out) return MGLDG_ERR_ARG;
    if (strategy != MGLDG_COARSEN_EQUAL && strategy != MGLDG_COARSEN_RAPID) return MGLDG_ERR_ARG;
    *out = nullptr;
    QT* t = nullptr;
    try {
        t = new QT();
        t->strategy = strategy;
        qt_build(*t, h, user);
        if (balance) qt_balance(*t);
        qt_finish(*t);
    } catch (const Error& e) {
        delete t;
        return e.code;
    } catch (const std::bad_alloc&) {
        delete t;
        return MGLDG_ERR_NOMEM;
    }
    *out = t;
    return MGLDG_OK;
}

extern "C" int mgldg_quadtree_destroy(mgldg_quadtree* qt) {
    delete qt;
    return MGLDG_OK;
}

extern "C" int mgldg_quadtree_info(const mgldg_quadtree* qt, int* nnodes, int* nlevels, int* nleaves) {
    if (!qt) return MGLDG_ERR_ARG;
    if (nnodes) *nnodes = (int)qt->nodes.size();
    if (nlevels) *nlevels = qt->numLevels;
    if (nleaves) {
        int c = 0;
        for (int id = 0; id < (int)qt->nodes.size(); ++id) c += qleaf(*qt, id) ? 1 : 0;
        *nleaves = c;
    }
    return MGLDG_OK;
}

extern "C" int mgldg_quadtree_layer(const mgldg_quadtree* qt, int l, int* n, int* level, int* ix, int* iy) {
    if (!qt || !n || l < 0 || l >= qt->numLevels) return MGLDG_ERR_ARG;
    const std::vector<int> ids = qt_layer(*qt, l);
    *n = (int)ids.size();
    if (level || ix || iy) {
        for (size_t k = 0; k < ids.size(); ++k) {
            const QT::Node& nd = qt->nodes[ids[k]];
            if (level) level[k] = nd.level;
            if (ix) ix[k] = (int)nd.ix;
            if (iy) iy[k] = (int)nd.iy;
        }
    }
    return MGLDG_OK;
}

extern "C" int mgldg_quadtree_problem_create(mgldg_ctx* ctx, const mgldg_quadtree* qt, int P, double tau0,
                                             double tauD, int tau_per_face, mgldg_problem** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(qt && out, MGLDG_ERR_ARG, "null argument");
    *out = nullptr;
    *out = quadtree_problem(ctx, *qt, P, tau0, tauD, tau_per_face != 0);
    MG_API_END
}

extern "C" int mgldg_problem_mesh_info(const mgldg_problem* pr, int* nfaces, int* nbfaces, int* nlevels) {
    if (!pr) return MGLDG_ERR_ARG;
    if (nfaces) *nfaces = pr->nfaces;
    if (nbfaces) *nbfaces = pr->nbfaces;
    if (nlevels) *nlevels = pr->nlevels;
    return MGLDG_OK;
}

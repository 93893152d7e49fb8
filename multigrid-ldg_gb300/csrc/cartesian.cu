// cartesian.cu -- the callers on either side of the solver path for a
// uniform Cartesian quadtree: mesh topology, LDG operator assembly on the
// GPU, the h-interpolation hierarchy and the Gaussian-sum right-hand side.
//
// Reference: Quadtree / Mesh (src/cartesian/mesh/quadtree.tpp:10-127,
// mesh.h:186-352), LDGPoisson::discretize (src/cartesian/dg/ldgpoisson.tpp:
// 14-100), computeRHS (:167-176) and InterpolationHierarchy
// (src/cartesian/multigrid/interpolationhierarchy.h:30-82).
//
// Elements are numbered in the reference's depth-first quadtree order, which
// on a uniform 2^L x 2^L tree is the Morton order with the x bit above the y
// bit at every level.  All blocks of the LDG operators on a uniform mesh are
// sums of a few distinct contributions (mass, broken gradient, lifting and
// penalty terms per face orientation); the host builds that short table with
// the reference's arithmetic, and for every stored block the ordered list of
// contributions in the reference's face order.  The GPU then writes every
// block (the bulk of the work: bytes), one thread per block entry.
#include <algorithm>
#include <cmath>
#include <random>

#include "api.cuh"
#include "ldg_build.cuh"

using namespace mg;

namespace mg {

// 8 Gaussians: centres U[0,1]^2, widths U[0.05,0.2], amplitudes N(0,1);
// mt19937_64, 53-bit uniforms, Box-Muller with the cosine branch
Gauss8 gaussian_params(uint64_t seed) {
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

static uint32_t morton_encode(uint32_t ix, uint32_t iy) {
    uint32_t e = 0;
    for (int bit = 0; bit < 16; ++bit) {
        e |= ((ix >> bit) & 1u) << (2 * bit + 1);
        e |= ((iy >> bit) & 1u) << (2 * bit);
    }
    return e;
}
static void morton_decode(uint32_t e, uint32_t& ix, uint32_t& iy) {
    ix = iy = 0;
    for (int bit = 0; bit < 16; ++bit) {
        ix |= ((e >> (2 * bit + 1)) & 1u) << bit;
        iy |= ((e >> (2 * bit)) & 1u) << bit;
    }
}

// out block o = sum of table[tidx[t]], t in [tptr[o], tptr[o+1]) in order
__global__ void k_sum_blocks(int64_t nout, int bsz, const int64_t* __restrict__ tptr, const int* __restrict__ tidx,
                             const double* __restrict__ table, double* __restrict__ out) {
    for (int64_t t = (int64_t)blockIdx.x * 256 + threadIdx.x; t < nout * bsz; t += (int64_t)gridDim.x * 256) {
        const int64_t o = t / bsz;
        const int e = (int)(t - o * bsz);
        double v = 0.0;
        const int64_t t0 = tptr[o], t1 = tptr[o + 1];
        if (t1 > t0) v = table[(size_t)tidx[t0] * bsz + e];
        for (int64_t q = t0 + 1; q < t1; ++q) v += table[(size_t)tidx[q] * bsz + e];
        out[t] = v;
    }
}

// b_e = M_e f_e with f the Gaussian sum at the element's Gauss-Lobatto nodes
// and M_e = |e| M_ref (Element::mass, mesh.h:143-147)
struct GaussDev {
    double cx[8], cy[8], w[8], a[8];
};
__global__ void k_rhs_gaussian(int ne, int P, const double* __restrict__ geom, GaussDev g,
                               const double* __restrict__ nodes, const double* __restrict__ Mref,
                               double* __restrict__ out) {
    extern __shared__ double sf[];
    const int b = P * P;
    for (int e = blockIdx.x; e < ne; e += gridDim.x) {
        const double lox = geom[e], loy = geom[ne + e], h = geom[2 * ne + e];
        const double vol = h * h;
        for (int q = threadIdx.x; q < b; q += blockDim.x) {
            const int i0 = q / P, i1 = q - i0 * P;
            const double x = lox + h * nodes[i0], y = loy + h * nodes[i1];
            double s = 0;
            for (int k = 0; k < 8; ++k) {
                const double dx = x - g.cx[k], dy = y - g.cy[k];
                s += g.a[k] * exp(-(dx * dx + dy * dy) / (2.0 * g.w[k] * g.w[k]));
            }
            sf[q] = s;
        }
        __syncthreads();
        for (int r = threadIdx.x; r < b; r += blockDim.x) {
            double s = 0;
            for (int c = 0; c < b; ++c) s += (vol * Mref[r * b + c]) * sf[c];
            out[(size_t)e * b + r] = s;
        }
        __syncthreads();
    }
}

}  // namespace mg

namespace mg {

mgldg_bsr* realize(mgldg_ctx* ctx, const Assembly& As, int ne, int b, const double* d_table) {
    mgldg_bsr* A = bsr_new(ctx, ne, ne, b, b, As.row_ptr, As.col_idx);
    int64_t* dptr = nullptr;
    int* didx = nullptr;
    try {
        dptr = dalloc<int64_t>(As.tptr.size());
        didx = dalloc<int>(std::max<size_t>(1, As.tidx.size()));
        upload(ctx, dptr, As.tptr.data(), As.tptr.size());
        upload(ctx, didx, As.tidx.data(), As.tidx.size());
        const int64_t nout = (int64_t)As.col_idx.size();
        const int bsz = b * b;
        int g = (int)std::min<int64_t>((nout * bsz + 255) / 256, ctx->sm_count * 64);
        {
            Launch L(ctx, MGLDG_K_SETUP);
            k_sum_blocks<<<std::max(1, g), 256, 0, ctx->stream>>>(nout, bsz, dptr, didx, d_table, A->val);
        }
        check_launch();
        sync(ctx);
    } catch (...) {
        dfree(dptr);
        dfree(didx);
        delete A;
        throw;
    }
    dfree(dptr);
    dfree(didx);
    return A;
}

// A block-CSR operator with one block per row, given column per row and a
// table of distinct blocks (br x bc) indexed per row.
mgldg_bsr* table_operator(mgldg_ctx* ctx, int nbr, int nbc, int br, int bc, const std::vector<int>& col,
                                 const std::vector<int>& blk, const std::vector<double>& table) {
    mgldg_bsr* T = new mgldg_bsr();
    try {
        std::vector<int> rp(nbr + 1);
        for (int k = 0; k <= nbr; ++k) rp[k] = k;
        T->ctx = ctx;
        T->nbr = nbr; T->nbc = nbc; T->br = br; T->bc = bc;
        T->nnzb = nbr;
        T->nuniq = (int64_t)(table.size() / ((size_t)br * bc));
        T->h_row_ptr = rp;
        T->h_col_idx = col;
        T->h_blk = blk;
        T->row_ptr = dalloc<int>(nbr + 1);
        T->col_idx = dalloc<int>(nbr + 4);
        T->blk = dalloc<int>(std::max(1, nbr));
        T->val = dalloc<double>(table.size());
        upload(ctx, T->row_ptr, rp.data(), rp.size());
        upload(ctx, T->col_idx, col.data(), col.size());
        upload(ctx, T->blk, blk.data(), blk.size());
        upload(ctx, T->val, table.data(), table.size());
    } catch (...) {
        delete T;
        throw;
    }
    return T;
}

// h-interpolation from the (nf/2)^2 to the nf^2 uniform mesh at degree P
// (interpolationhierarchy.h:53-79): fine element k of the Morton order lies
// in parent k>>2 at child position k&3 = (x bit, y bit); its block evaluates
// the parent's Lagrange basis at the child's nodes.  Four distinct blocks.
static mgldg_bsr* h_interp(mgldg_ctx* ctx, int nf, int P) {
    MG_REQUIRE(P >= 1 && P <= MGLDG_PMAX && nf >= 2 && (nf & (nf - 1)) == 0, MGLDG_ERR_ARG,
               "h-interpolation needs P in 1..6 and a power-of-two n >= 2");
    const Ref2 R(P);
    const int b = R.b;
    std::vector<double> E4((size_t)4 * b * b);
    for (int cpos = 0; cpos < 4; ++cpos) {
        const double lo[2] = {0.5 * (cpos >> 1), 0.5 * (cpos & 1)};
        for (int i0 = 0; i0 < P; ++i0)
            for (int i1 = 0; i1 < P; ++i1) {
                double node[2];
                int idx[2] = {i0, i1};
                for (int d = 0; d < 2; ++d) node[d] = lo[d] + 0.5 * R.nodes[idx[d]];
                R.lagrange2(node, &E4[(size_t)cpos * b * b + (size_t)(i0 * P + i1) * b]);
            }
    }
    const int nef = nf * nf;
    std::vector<int> col(nef), blk(nef);
    for (int k = 0; k < nef; ++k) {
        col[k] = k >> 2;
        blk[k] = k & 3;
    }
    return table_operator(ctx, nef, nef / 4, b, b, col, blk, E4);
}

// p-interpolation from degree Pc to degree Pf on the same ne elements
// (interpolationhierarchy.h:109-129): every block evaluates the Pc Lagrange
// basis at the Pf nodes of the master element.  One distinct block.
static mgldg_bsr* p_interp(mgldg_ctx* ctx, int ne, int Pf, int Pc) {
    MG_REQUIRE(Pf >= 1 && Pf <= MGLDG_PMAX && Pc >= 1 && Pc <= MGLDG_PMAX && ne >= 1, MGLDG_ERR_ARG,
               "p-interpolation needs degrees in 1..6 and at least one element");
    const Ref2 Rf(Pf), Rc(Pc);
    std::vector<double> E((size_t)Rf.b * Rc.b);
    for (int i0 = 0; i0 < Pf; ++i0)
        for (int i1 = 0; i1 < Pf; ++i1) {
            const double node[2] = {Rf.nodes[i0], Rf.nodes[i1]};
            Rc.lagrange2(node, &E[(size_t)(i0 * Pf + i1) * Rc.b]);
        }
    std::vector<int> col(ne), blk(ne, 0);
    for (int k = 0; k < ne; ++k) col[k] = k;
    return table_operator(ctx, ne, ne, Rf.b, Rc.b, col, blk, E);
}

static mgldg_problem* cartesian_create(mgldg_ctx* ctx, int P, int n, double tau0, double tauD) {
    MG_REQUIRE(P >= 1 && P <= 5, MGLDG_ERR_UNSUPPORTED, "P must be 1..5 (block size <= 25)");
    MG_REQUIRE(n >= 1 && n <= 32768 && (n & (n - 1)) == 0, MGLDG_ERR_ARG, "n must be a power of two");
    const Ref2 R(P);
    const int b = R.b;
    const int ne = n * n;
    const double h = 1.0 / n;
    const double area = h, vol = h * h;

    // ---- distinct contributions (the reference's per-face arithmetic) ----
    Blk Mblk = bscale(vol, R.tensor(R.mass1));
    Blk Minv = bscale(1 / vol, R.tensor(R.invmass1));
    std::vector<Blk> table;
    auto add = [&](Blk&& B) { table.push_back(std::move(B)); return (int)table.size() - 1; };
    const int cM = add(Blk(Mblk));
    int cDg[2], cGRR[2], cGRL[2], cGB[2][2], cTRR[2], cTLL[2], cTRL[2], cTLR[2], cTB[2][2];
    for (int d = 0; d < 2; ++d) {
        double jac = 1.0 / h;
        cDg[d] = add(bscale(jac, R.diff(d)));
        // canonical interior face in dimension d (mesh.h:285-310)
        Blk LL((size_t)b * b, 0.0), RR((size_t)b * b, 0.0), RL((size_t)b * b, 0.0);
        int jl[8], jr[8];
        for (int a = 0; a < P; ++a) {
            int jt[2];
            jt[1 - d] = a;
            jt[d] = P - 1;
            jl[a] = jt[0] * P + jt[1];
            jt[d] = 0;
            jr[a] = jt[0] * P + jt[1];
        }
        for (int a = 0; a < P; ++a)
            for (int c = 0; c < P; ++c) {
                double m = R.mass1[a * P + c] * area;
                LL[(size_t)jl[a] * b + jl[c]] = m;
                RR[(size_t)jr[a] * b + jr[c]] = m;
                RL[(size_t)jr[a] * b + jl[c]] = m;
            }
        cGRR[d] = add(bmul(bscale(1.0, Minv), RR, b));
        cGRL[d] = add(bmul(bscale(-1.0, Minv), RL, b));
        cTRR[d] = add(bscale(tau0, RR));
        cTLL[d] = add(bscale(tau0, LL));
        cTRL[d] = add(bscale(-tau0, RL));
        cTLR[d] = add(bscale(-tau0, btrans(RL, b)));
        // boundary faces of dimension d, side s (0: lower, normal -1; 1:
        // upper, normal +1): 10-point Gauss rule (mesh.h:312-351)
        for (int sd = 0; sd < 2; ++sd) {
            const double nrm = sd ? 1.0 : -1.0;
            std::vector<double> phi((size_t)MGLDG_QF * b), w(MGLDG_QF);
            for (int q = 0; q < MGLDG_QF; ++q) {
                double ql[2];
                ql[1 - d] = kQuadNodes[q];
                ql[d] = (nrm > 0) ? 1 : 0;
                R.lagrange2(ql, &phi[(size_t)q * b]);
                w[q] = 1;
                w[q] *= kQuadWeights[q];
            }
            for (int q = 0; q < MGLDG_QF; ++q) w[q] *= area;
            Blk Lm((size_t)b * MGLDG_QF);
            for (int a = 0; a < b; ++a)
                for (int q = 0; q < MGLDG_QF; ++q) Lm[(size_t)a * MGLDG_QF + q] = phi[(size_t)q * b + a] * w[q];
            Blk LLb((size_t)b * b);
            for (int a = 0; a < b; ++a)
                for (int c = 0; c < b; ++c) {
                    double s = 0;
                    for (int q = 0; q < MGLDG_QF; ++q) s += Lm[(size_t)a * MGLDG_QF + q] * phi[(size_t)q * b + c];
                    LLb[(size_t)a * b + c] = s;
                }
            cGB[d][sd] = add(bmul(bscale(-nrm, Minv), LLb, b));
            cTB[d][sd] = add(bscale(tauD, LLb));
        }
    }

    // ---- per-block contribution lists in the reference's face order ----
    Assembly AM, AG[2], AT;
    AM.row_ptr.push_back(0);
    AG[0].row_ptr.push_back(0);
    AG[1].row_ptr.push_back(0);
    AT.row_ptr.push_back(0);
    for (int e = 0; e < ne; ++e) {
        uint32_t ix, iy;
        morton_decode((uint32_t)e, ix, iy);
        const uint32_t c[2] = {ix, iy};
        int left[2], right[2];
        for (int d = 0; d < 2; ++d) {
            uint32_t lx = ix, ly = iy, rx = ix, ry = iy;
            if (d == 0) { lx = ix - 1; rx = ix + 1; } else { ly = iy - 1; ry = iy + 1; }
            left[d] = (c[d] > 0) ? (int)morton_encode(lx, ly) : -1;
            right[d] = (c[d] + 1 < (uint32_t)n) ? (int)morton_encode(rx, ry) : -1;
        }
        // mass
        AM.add_block(e, {cM});
        AM.row_ptr.push_back((int)AM.col_idx.size());
        // gradients: G_d(e,left) and G_d(e,e)
        for (int d = 0; d < 2; ++d) {
            std::vector<int> diag{cDg[d]};
            if (left[d] >= 0) diag.push_back(cGRR[d]);
            if (left[d] < 0) diag.push_back(cGB[d][0]);
            if (right[d] < 0) diag.push_back(cGB[d][1]);
            if (left[d] >= 0) AG[d].add_block(left[d], {cGRL[d]});   // left < e in Morton order
            AG[d].add_block_v(e, diag);
            AG[d].row_ptr.push_back((int)AG[d].col_idx.size());
        }
        // penalty: faces where e is the right element come first, in the
        // order of their left elements; then e's own faces in (dim, dir)
        std::vector<int> tdiag;
        {
            int l0 = left[0], l1 = left[1];
            if (l0 >= 0 && l1 >= 0) {
                if (l0 < l1) { tdiag.push_back(cTRR[0]); tdiag.push_back(cTRR[1]); }
                else { tdiag.push_back(cTRR[1]); tdiag.push_back(cTRR[0]); }
            } else if (l0 >= 0) {
                tdiag.push_back(cTRR[0]);
            } else if (l1 >= 0) {
                tdiag.push_back(cTRR[1]);
            }
            for (int d = 0; d < 2; ++d) {
                if (left[d] < 0) tdiag.push_back(cTB[d][0]);
                if (right[d] < 0) tdiag.push_back(cTB[d][1]);
                else tdiag.push_back(cTLL[d]);
            }
        }
        struct Ent { int col; std::vector<int> c; };
        std::vector<Ent> row;
        for (int d = 0; d < 2; ++d) {
            if (left[d] >= 0) row.push_back({left[d], {cTRL[d]}});
            if (right[d] >= 0) row.push_back({right[d], {cTLR[d]}});
        }
        row.push_back({e, tdiag});
        std::sort(row.begin(), row.end(), [](const Ent& a, const Ent& b2) { return a.col < b2.col; });
        for (auto& en : row) AT.add_block_v(en.col, en.c);
        AT.row_ptr.push_back((int)AT.col_idx.size());
    }

    mgldg_problem* pr = new mgldg_problem();
    pr->ctx = ctx;
    pr->P = P; pr->b = b; pr->n = n; pr->ne = ne; pr->h = h;
    double* d_table = nullptr;
    mgldg_bsr *M = nullptr, *G0 = nullptr, *G1 = nullptr, *Tm = nullptr;
    try {
        std::vector<double> flat;
        for (auto& B : table) flat.insert(flat.end(), B.begin(), B.end());
        d_table = dalloc<double>(flat.size());
        upload(ctx, d_table, flat.data(), flat.size());
        M = realize(ctx, AM, ne, b, d_table);
        G0 = realize(ctx, AG[0], ne, b, d_table);
        G1 = realize(ctx, AG[1], ne, b, d_table);
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
        pr->ew.assign(ne, h);
        for (int e = 0; e < ne; ++e) {
            uint32_t ix, iy;
            morton_decode((uint32_t)e, ix, iy);
            pr->ex[e] = ix * h;
            pr->ey[e] = iy * h;
        }
        pr->nlevels = 1;
        for (int m = n; m > 1; m >>= 1) ++pr->nlevels;
        pr->nbfaces = 4 * n;
        pr->nfaces = 2 * n * (n - 1) + pr->nbfaces;
        problem_upload_geometry(ctx, pr);

        // ---- h-interpolation hierarchy (interpolationhierarchy.h:30-82) ----
        for (int nf = n; nf > 1; nf >>= 1) pr->T.push_back(h_interp(ctx, nf, P));
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

static void rhs_gaussian_dev(mgldg_ctx* ctx, mgldg_problem* pr, uint64_t seed, double* b) {
    if (pr->simplex) {
        simplex_rhs_dev(ctx, pr, seed, b);
        return;
    }
    Gauss8 g = gaussian_params(seed);
    GaussDev gd;
    std::memcpy(gd.cx, g.cx, sizeof g.cx);
    std::memcpy(gd.cy, g.cy, sizeof g.cy);
    std::memcpy(gd.w, g.w, sizeof g.w);
    std::memcpy(gd.a, g.a, sizeof g.a);
    int grid = std::max(1, std::min(pr->ne, ctx->sm_count * 32));
    {
        Launch L(ctx, MGLDG_K_SETUP);
        k_rhs_gaussian<<<grid, 128, pr->b * sizeof(double), ctx->stream>>>(pr->ne, pr->P, pr->d_geom, gd,
                                                                           pr->d_nodes, pr->d_Mref, b);
    }
    check_launch();
}

}  // namespace mg

// ================================================================== C ABI ==
extern "C" int mgldg_cartesian_create(mgldg_ctx* ctx, int P, int n, double tau0, double tauD, mgldg_problem** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(out != nullptr, MGLDG_ERR_ARG, "null output");
    *out = nullptr;
    *out = cartesian_create(ctx, P, n, tau0, tauD);
    MG_API_END
}

extern "C" int mgldg_problem_destroy(mgldg_problem* pr) {
    if (!pr) return MGLDG_OK;
    if (pr->ctx) cudaSetDevice(pr->ctx->device);
    delete pr;
    return MGLDG_OK;
}

namespace mg {
void problem_boxes(const mgldg_problem* pr, int* P, int* ne, const double** ex, const double** ey,
                   const double** ew) {
    *P = pr->P;
    *ne = pr->ne;
    *ex = pr->ex.data();
    *ey = pr->ey.data();
    *ew = pr->ew.data();
}

int problem_node_coords(const mgldg_problem* pr, std::vector<double>& xy) {
    const int b = pr->b, P = pr->P;
    const int dim = pr->simplex ? pr->sdim : 2;
    xy.assign((size_t)pr->ne * b * dim, 0.0);
    for (int e = 0; e < pr->ne; ++e) {
        double* o = &xy[(size_t)e * b * dim];
        if (pr->simplex) {
            // Master::dgnodes: p0 + J node (master.h:40-45)
            const double* g = &pr->sgeom[(size_t)e * 22];
            for (int i = 0; i < b; ++i)
                for (int d = 0; d < dim; ++d) {
                    double acc = g[3 + d * 3] * pr->snodes[(size_t)dim * i];
                    for (int j = 1; j < dim; ++j) acc += g[3 + d * 3 + j] * pr->snodes[(size_t)dim * i + j];
                    o[(size_t)dim * i + d] = g[d] + acc;
                }
        } else {
            const double h = pr->ew[e];
            for (int i0 = 0; i0 < P; ++i0)
                for (int i1 = 0; i1 < P; ++i1) {
                    o[2 * (i0 * P + i1)] = pr->ex[e] + h * kNodes[P - 1][i0];
                    o[2 * (i0 * P + i1) + 1] = pr->ey[e] + h * kNodes[P - 1][i1];
                }
        }
    }
    return dim;
}

void problem_upload_geometry(mgldg_ctx* ctx, mgldg_problem* pr) {
    const Ref2 R(pr->P);
    const int ne = pr->ne, b = pr->b;
    std::vector<double> g((size_t)3 * ne);
    std::copy(pr->ex.begin(), pr->ex.end(), g.begin());
    std::copy(pr->ey.begin(), pr->ey.end(), g.begin() + ne);
    std::copy(pr->ew.begin(), pr->ew.end(), g.begin() + 2 * (size_t)ne);
    pr->d_geom = dalloc<double>(std::max<size_t>(1, g.size()));
    upload(ctx, pr->d_geom, g.data(), g.size());
    pr->d_nodes = dalloc<double>(pr->P);
    upload(ctx, pr->d_nodes, R.nodes, pr->P);
    const Blk Mref = R.tensor(R.mass1);
    pr->d_Mref = dalloc<double>((size_t)b * b);
    upload(ctx, pr->d_Mref, Mref.data(), Mref.size());
}
}  // namespace mg

extern "C" int mgldg_problem_info(const mgldg_problem* pr, int* ne, int* npl, int64_t* ndof, int* nT) {
    if (!pr) return MGLDG_ERR_ARG;
    if (ne) *ne = pr->ne;
    if (npl) *npl = pr->b;
    if (ndof) *ndof = (int64_t)pr->ne * pr->b;
    if (nT) *nT = (int)pr->T.size();
    return MGLDG_OK;
}

extern "C" int mgldg_problem_ops(mgldg_problem* pr, mgldg_ops** ops) {
    if (!pr || !ops) return MGLDG_ERR_ARG;
    *ops = pr->ops;
    return MGLDG_OK;
}

extern "C" int mgldg_problem_interp(mgldg_problem* pr, int l, const mgldg_bsr** T) {
    if (!pr || !T || l < 0 || l >= (int)pr->T.size()) return MGLDG_ERR_ARG;
    *T = pr->T[l];
    return MGLDG_OK;
}

extern "C" int mgldg_problem_rhs_gaussian_dev(mgldg_ctx* ctx, mgldg_problem* pr, uint64_t seed, double* b) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(pr && b, MGLDG_ERR_ARG, "null argument");
    rhs_gaussian_dev(ctx, pr, seed, b);
    MG_API_END
}

extern "C" int mgldg_problem_rhs_gaussian(mgldg_ctx* ctx, mgldg_problem* pr, uint64_t seed, double* b) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(pr && b, MGLDG_ERR_ARG, "null argument");
    const int64_t n = (int64_t)pr->ne * pr->b;
    double* d = dalloc<double>(n);
    try {
        rhs_gaussian_dev(ctx, pr, seed, d);
        download(ctx, b, d, n);
        sync(ctx);
    } catch (...) {
        dfree(d);
        throw;
    }
    dfree(d);
    MG_API_END
}

extern "C" int mgldg_cartesian_h_interp(mgldg_ctx* ctx, int n_fine, int P, mgldg_bsr** T) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(T != nullptr, MGLDG_ERR_ARG, "null output");
    *T = nullptr;
    *T = h_interp(ctx, n_fine, P);
    sync(ctx);
    MG_API_END
}

extern "C" int mgldg_cartesian_p_interp(mgldg_ctx* ctx, int ne, int P_fine, int P_coarse, mgldg_bsr** T) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(T != nullptr, MGLDG_ERR_ARG, "null output");
    *T = nullptr;
    *T = p_interp(ctx, ne, P_fine, P_coarse);
    sync(ctx);
    MG_API_END
}

// adjoint.cu -- per-element diffusivity and adjoint gradients.
//
// With a diffusivity kappa_e per element, the LDG operator becomes
//     A(kappa) = T + sum_d G_d^T diag(kappa_e M_e) G_d
// (kappa weights the flux sigma = kappa q, q = G u; kappa = 1 gives the
// reference's construct_laplacian, src/cartesian/dg/ldgpoisson.h:34-52).
// For a loss L(u) with A u = b, the adjoint lambda solves A lambda = dL/du
// (A is symmetric, so the adjoint solve reuses the forward multigrid-PCG),
// dL/db = lambda and
//     dL/dkappa_e = -lambda^T (dA/dkappa_e) u
//                 = -sum_d (G_d lambda)_e^T M_e (G_d u)_e,
// an element-local contraction of two gradient fields with the element mass
// matrix.  The reference has no such path; it is built on its operators.
#include "api.cuh"

#include <algorithm>
#include <vector>

using namespace mg;

namespace mg {

// every block of row i scaled by kappa[i] (a copy of M becomes kappa M)
__global__ void k_scale_rows(int nbr, const int* __restrict__ row_ptr, int bsz, const double* __restrict__ kappa,
                             double* __restrict__ val) {
    for (int i = blockIdx.x; i < nbr; i += gridDim.x) {
        const double s = kappa[i];
        for (int k = row_ptr[i]; k < row_ptr[i + 1]; ++k)
            for (int e = threadIdx.x; e < bsz; e += blockDim.x) val[(size_t)k * bsz + e] *= s;
    }
}

static mgldg_bsr* scaled_rows(mgldg_ctx* ctx, const mgldg_bsr* M, const double* kappa_dev) {
    MG_REQUIRE(!M->blk, MGLDG_ERR_ARG, "mass matrix must store its blocks");
    mgldg_bsr* Mk = bsr_clone(ctx, M);
    try {
        if (M->nbr) {
            Launch L(ctx, MGLDG_K_SETUP);
            k_scale_rows<<<std::min(M->nbr, ctx->sm_count * 32), 128, 0, ctx->stream>>>(M->nbr, Mk->row_ptr,
                                                                                       (int)M->bsz(), kappa_dev, Mk->val);
        }
        check_launch();
    } catch (...) {
        delete Mk;
        throw;
    }
    return Mk;
}

// out[e] (+)= -gl_e^T M_e gu_e, M_e the diagonal block of row e of M; one
// warp per element, lanes over the rows of M_e
__global__ void k_kappa_contract(int ne, int b, const int* __restrict__ diag, const double* __restrict__ Mval,
                                 const double* __restrict__ gu, const double* __restrict__ gl, double* __restrict__ out,
                                 int accumulate) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    for (int e = blockIdx.x * wpb + warp; e < ne; e += gridDim.x * wpb) {
        const double* Me = Mval + (size_t)diag[e] * b * b;
        const double* u = gu + (size_t)e * b;
        const double* l = gl + (size_t)e * b;
        double acc = 0;
        for (int r = lane; r < b; r += 32) {
            double w = 0;
            for (int c = 0; c < b; ++c) w = fma(Me[r * b + c], u[c], w);
            acc = fma(l[r], w, acc);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) out[e] = (accumulate ? out[e] : 0.0) - acc;
    }
}

// r = u - u_obs
__global__ void k_misfit(int64_t n, const double* __restrict__ u, const double* __restrict__ u_obs,
                         double* __restrict__ r) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = u[i] - u_obs[i];
}

// dkappa[e] = -sum_d (G_d lambda)_e^T M_e (G_d u)_e, with two work vectors
static void kappa_gradient(mgldg_ctx* ctx, const mgldg_ops* ops, const double* u, const double* lambda, double* dkappa,
                           double* gu, double* gl) {
    mgldg_bsr* M = ops->M;
    bsr_build_diag(M);
    const int wpb = 8;
    const int grid = std::max(1, std::min((M->nbr + wpb - 1) / wpb, ctx->sm_count * 16));
    for (int d = 0; d < ops->ndim; ++d) {
        spmv<double>(ctx, ops->G[d], 1.0, u, 0.0, nullptr, gu);
        spmv<double>(ctx, ops->G[d], 1.0, lambda, 0.0, nullptr, gl);
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_kappa_contract<<<grid, wpb * 32, 0, ctx->stream>>>(M->nbr, M->br, M->diag, M->val, gu, gl, dkappa,
                                                                 d > 0 ? 1 : 0);
        }
        check_launch();
    }
}

static void require_gradient_ops(const mgldg_ops* ops) {
    MG_REQUIRE(ops && ops->has_MGT(), MGLDG_ERR_ARG, "operators need M, G and T");
    MG_REQUIRE(!ops->M->blk, MGLDG_ERR_ARG, "mass matrix must store its blocks");
    MG_REQUIRE(ops->M->br == ops->M->bc && ops->M->nbr == ops->M->nbc, MGLDG_ERR_SHAPE, "M must be square");
    for (int d = 0; d < ops->ndim; ++d)
        MG_REQUIRE(ops->G[d]->nbr == ops->M->nbr && ops->G[d]->br == ops->M->br, MGLDG_ERR_SHAPE,
                   "G and M block shapes differ");
}

}  // namespace mg

// ================================================================== C ABI ==
extern "C" int mgldg_ops_construct_laplacian_kappa(mgldg_ctx* ctx, mgldg_ops* ops, const double* kappa) {
    MG_API_BEGIN(ctx)
    require_gradient_ops(ops);
    const int ne = ops->M->nbr;
    std::vector<double> k(ne, 1.0);
    if (kappa) k.assign(kappa, kappa + ne);
    for (int e = 0; e < ne; ++e)
        MG_REQUIRE(k[e] > 0 && k[e] < 1e300, MGLDG_ERR_ARG, "kappa must be positive and finite");
    double* dk = nullptr;
    mgldg_bsr* Mk = nullptr;
    try {
        dk = dalloc<double>(std::max(1, ne));
        upload(ctx, dk, k.data(), ne);
        Mk = scaled_rows(ctx, ops->M, dk);
        mgldg_bsr* A = laplacian_of(ctx, Mk, ops->G, ops->ndim, ops->T);
        delete ops->A;
        ops->A = A;
        sync(ctx);
    } catch (...) {
        dfree(dk);
        delete Mk;
        throw;
    }
    dfree(dk);
    delete Mk;
    MG_API_END
}

extern "C" int mgldg_kappa_gradient_dev(mgldg_ctx* ctx, const mgldg_ops* ops, const double* u, const double* lambda,
                                        double* dkappa) {
    MG_API_BEGIN(ctx)
    require_gradient_ops(ops);
    MG_REQUIRE(u && lambda && dkappa, MGLDG_ERR_ARG, "null vector");
    const int64_t n = (int64_t)ops->M->nbr * ops->M->br;
    double *gu = nullptr, *gl = nullptr;
    try {
        gu = dalloc<double>(std::max<int64_t>(1, n));
        gl = dalloc<double>(std::max<int64_t>(1, n));
        kappa_gradient(ctx, ops, u, lambda, dkappa, gu, gl);
        sync(ctx);
    } catch (...) {
        dfree(gu);
        dfree(gl);
        throw;
    }
    dfree(gu);
    dfree(gl);
    MG_API_END
}

extern "C" int mgldg_adjoint_l2_dev(mgldg_ctx* ctx, mgldg_mg* mg, const mgldg_ops* ops, const double* b,
                                    const double* u_obs, double tol, int maxit, double* u, double* lambda,
                                    double* dkappa, double* loss, int* iters) {
    MG_API_BEGIN(ctx)
    require_gradient_ops(ops);
    MG_REQUIRE(ops->A, MGLDG_ERR_ARG, "operators hold no Laplacian");
    MG_REQUIRE(b && u_obs && u && lambda, MGLDG_ERR_ARG, "null vector");
    const mgldg_bsr* A = ops->A;
    const int64_t n = (int64_t)A->nbr * A->br;
    MG_REQUIRE(n == (int64_t)ops->M->nbr * ops->M->br, MGLDG_ERR_SHAPE, "A and M sizes differ");
    int it[2] = {0, 0};
    int rc = mgldg_pcg_dev(ctx, mg, A, b, u, tol, maxit, &it[0], nullptr);
    if (rc != MGLDG_OK) return rc;
    double *r = nullptr, *gu = nullptr, *gl = nullptr, *dsum = nullptr;
    try {
        r = dalloc<double>(std::max<int64_t>(1, n));
        dsum = dalloc<double>(1);
        const int g = std::max(1, (int)std::min<int64_t>((n + 255) / 256, ctx->sm_count * 8));
        {
            Launch L(ctx, MGLDG_K_VECTOR);
            k_misfit<<<g, 256, 0, ctx->stream>>>(n, u, u_obs, r);
        }
        check_launch();
        if (loss) {
            int np = 0;
            dot_partials<double>(ctx, (int)n, r, r, ctx->d_partials, &np);
            finish_sum(ctx, ctx->d_partials, np, dsum);
            double h = 0;
            download(ctx, &h, dsum, 1);
            sync(ctx);
            *loss = 0.5 * h;
        }
        rc = mgldg_pcg_dev(ctx, mg, A, r, lambda, tol, maxit, &it[1], nullptr);
        if (rc == MGLDG_OK && dkappa) {
            gu = dalloc<double>(std::max<int64_t>(1, n));
            gl = dalloc<double>(std::max<int64_t>(1, n));
            kappa_gradient(ctx, ops, u, lambda, dkappa, gu, gl);
            sync(ctx);
        }
    } catch (...) {
        dfree(r); dfree(gu); dfree(gl); dfree(dsum);
        throw;
    }
    dfree(r); dfree(gu); dfree(gl); dfree(dsum);
    if (iters) {
        iters[0] = it[0];
        iters[1] = it[1];
    }
    if (rc != MGLDG_OK) return rc;
    MG_API_END
}

// io.cu -- on-disk formats for diffing operators and solutions against the
// reference's dumps.
//
// Matrix Market: the reference's SparseBlockMatrix::write
// (src/cartesian/util/sparseblockmatrix.tpp:145-164) writes
// "%%MatrixMarket matrix coordinate real general", then "rows cols nnz" with
// nnz = every entry of every stored block, then one "i j value" line per
// entry, 1-based, with max_digits10 (17) significant digits.  The same file
// is written here (blocks in sorted order instead of hash-map order) and
// read back into a BSR handle with a given block shape.
//
// .fun: the reference's Function::write (src/cartesian/dg/function.h:173-190)
// writes "P N ne", then for every element its nodes in tensor order, one
// line "x y value" per node, and an empty line after each element.
#include <cstdio>
#include <map>

#include "api.cuh"
#include "ldg_build.cuh"

using namespace mg;

extern "C" int mgldg_bsr_write_mtx(mgldg_ctx* ctx, const mgldg_bsr* A, const char* path) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(A && path, MGLDG_ERR_ARG, "null argument");
    const size_t bs = A->bsz();
    std::vector<int> rp(A->nbr + 1), ci(std::max<int64_t>(1, A->nnzb));
    std::vector<double> v(std::max<size_t>(1, (size_t)A->nnzb * bs));
    int rc = mgldg_bsr_download(ctx, A, rp.data(), ci.data(), v.data());
    MG_REQUIRE(rc == MGLDG_OK, rc, "download failed: " + ctx->err);
    FILE* f = std::fopen(path, "w");
    MG_REQUIRE(f != nullptr, MGLDG_ERR_ARG, std::string("cannot open ") + path);
    std::fprintf(f, "%%%%MatrixMarket matrix coordinate real general\n");
    std::fprintf(f, "%lld %lld %lld\n", (long long)A->nbr * A->br, (long long)A->nbc * A->bc,
                 (long long)A->nnzb * (long long)bs);
    for (int i = 0; i < A->nbr; ++i)
        for (int k = rp[i]; k < rp[i + 1]; ++k) {
            const long long bi = (long long)i * A->br, bj = (long long)ci[k] * A->bc;
            for (int r = 0; r < A->br; ++r)
                for (int c = 0; c < A->bc; ++c)
                    std::fprintf(f, "%lld %lld %.17g\n", bi + r + 1, bj + c + 1, v[(size_t)k * bs + (size_t)r * A->bc + c]);
        }
    const bool ok = std::fclose(f) == 0;
    MG_REQUIRE(ok, MGLDG_ERR_ARG, std::string("write failed: ") + path);
    MG_API_END
}

extern "C" int mgldg_bsr_read_mtx(mgldg_ctx* ctx, const char* path, int br, int bc, mgldg_bsr** out) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(path && out && br >= 1 && bc >= 1, MGLDG_ERR_ARG, "bad arguments");
    *out = nullptr;
    FILE* f = std::fopen(path, "r");
    MG_REQUIRE(f != nullptr, MGLDG_ERR_ARG, std::string("cannot open ") + path);
    char line[512];
    long long rows = -1, cols = -1, nnz = -1;
    bool header = false;
    std::map<std::pair<int, int>, std::vector<double>> blocks;
    bool bad = false;
    long long seen = 0;
    while (std::fgets(line, sizeof line, f)) {
        if (line[0] == '%') {
            if (!header && std::string(line).find("coordinate real general") == std::string::npos) bad = true;
            header = true;
            continue;
        }
        if (rows < 0) {
            if (std::sscanf(line, "%lld %lld %lld", &rows, &cols, &nnz) != 3) bad = true;
            continue;
        }
        long long i, j;
        double val;
        if (std::sscanf(line, "%lld %lld %lg", &i, &j, &val) != 3) continue;
        if (i < 1 || j < 1 || i > rows || j > cols) { bad = true; break; }
        const int bi = (int)((i - 1) / br), bj = (int)((j - 1) / bc);
        auto& blk = blocks[{bi, bj}];
        if (blk.empty()) blk.assign((size_t)br * bc, 0.0);
        blk[(size_t)((i - 1) % br) * bc + (j - 1) % bc] += val;
        ++seen;
    }
    std::fclose(f);
    MG_REQUIRE(!bad && rows >= 0 && seen == nnz, MGLDG_ERR_ARG, std::string("not a coordinate real general file: ") + path);
    MG_REQUIRE(rows % br == 0 && cols % bc == 0, MGLDG_ERR_SHAPE, "matrix size is not a multiple of the block size");
    const int nbr = (int)(rows / br), nbc = (int)(cols / bc);
    std::vector<int> rp(nbr + 1, 0), ci;
    std::vector<double> v;
    for (auto& kv : blocks) {
        rp[kv.first.first + 1]++;
        ci.push_back(kv.first.second);
        v.insert(v.end(), kv.second.begin(), kv.second.end());
    }
    for (int i = 0; i < nbr; ++i) rp[i + 1] += rp[i];
    if (ci.empty()) { ci.push_back(0); v.assign((size_t)br * bc, 0.0); }
    int rc = mgldg_bsr_create(ctx, nbr, nbc, br, bc, rp.data(), ci.data(), v.data(), out);
    MG_REQUIRE(rc == MGLDG_OK, rc, ctx->err);
    MG_API_END
}

extern "C" int mgldg_problem_write_fun(mgldg_ctx* ctx, const mgldg_problem* pr, const double* u, const char* path) {
    MG_API_BEGIN(ctx)
    MG_REQUIRE(pr && u && path, MGLDG_ERR_ARG, "null argument");
    std::vector<double> xy;
    const int dim = problem_node_coords(pr, xy);
    const int b = pr->b;
    FILE* f = std::fopen(path, "w");
    MG_REQUIRE(f != nullptr, MGLDG_ERR_ARG, std::string("cannot open ") + path);
    std::fprintf(f, "%d %d %d\n", pr->P, dim, pr->ne);
    for (int e = 0; e < pr->ne; ++e) {
        for (int i = 0; i < b; ++i) {
            const size_t k = (size_t)e * b + i;
            for (int d = 0; d < dim; ++d) std::fprintf(f, "%.17g ", xy[(size_t)dim * k + d]);
            std::fprintf(f, "%.17g\n", u[k]);
        }
        std::fprintf(f, "\n");
    }
    const bool ok = std::fclose(f) == 0;
    MG_REQUIRE(ok, MGLDG_ERR_ARG, std::string("write failed: ") + path);
    MG_API_END
}

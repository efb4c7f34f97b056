// api_perm.cu -- DoF permutation between the engine's vertex numbering and
// another numbering of the same vertices (ugcore's DoFDistribution of a
// script's approximation space, whose order follows lib_grid's element lists,
// dof_distribution.cpp:1339-1440).  The engine's kernels need their own
// numbering (lexicographic on structured levels, refinement order on
// unstructured ones), so the ugcore-side glue moves vectors and operators
// across the boundary with these gathers.  No ugcore counterpart.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "gmg.cuh"

using namespace ug4gb;

struct ug4gb_perm {
    ug4gb_ctx *ctx = nullptr;
    int n = 0;
    DevBuf<int> ext_to_eng;   // perm[i] = engine index of external index i
    DevBuf<int> eng_to_ext;   // inverse
    // cached value maps of a permuted matrix: B.val[k] = A.val[map[k]]
    struct MatMap {
        uint64_t key = 0;
        int64_t nnz = 0;
        DevBuf<int> map;
    } mat[2];
};

template <class F>
static int guarded(ug4gb_ctx *ctx, F &&f)
{
    try {
        f();
        return UG4GB_OK;
    } catch (const Error &e) {
        if (ctx) ctx->c.err = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        if (ctx) ctx->c.err = e.what();
        return UG4GB_ERR_INVALID;
    }
}

namespace {

__global__ void k_gather_vec(int n, const int *idx, const double *src, double *dst)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[idx[i]];
}

__global__ void k_perm_row_len(int n, const int *rowmap, const int *rowptr, int *len)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) len[i] = rowptr[rowmap[i] + 1] - rowptr[rowmap[i]];
}

// row i of B from row rowmap[i] of A, columns through colmap; val holds the
// source positions (as doubles, exact) so that the row sort carries them
__global__ void k_perm_fill(int n, const int *rowmap, const int *colmap, const int *rowptr, const int *col,
                            const int *browptr, int *bcol, double *bsrc)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int r = rowmap[i];
    int q = browptr[i];
    for (int a = rowptr[r]; a < rowptr[r + 1]; ++a, ++q) {
        bcol[q] = colmap[col[a]];
        bsrc[q] = (double)a;
    }
}

__global__ void k_src_to_map(int64_t nnz, const double *src, int *map)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) map[k] = (int)src[k];
}

__global__ void k_gather_vals(int64_t nnz, const int *map, const double *a, double *b)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < nnz) b[k] = a[map[k]];
}

__global__ void k_sort_row_pairs(const int *rowptr, int *col, double *val, int nrows)
{
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    int a0 = rowptr[r], a1 = rowptr[r + 1];
    for (int a = a0 + 1; a < a1; ++a) {
        int cc = col[a];
        double vv = val[a];
        int b = a - 1;
        while (b >= a0 && col[b] > cc) {
            col[b + 1] = col[b];
            val[b + 1] = val[b];
            --b;
        }
        col[b + 1] = cc;
        val[b + 1] = vv;
    }
}

void make_perm(ug4gb_perm *p, const std::vector<int> &e2x_host_inv /* ext_to_eng */)
{
    Ctx &c = p->ctx->c;
    const int n = p->n;
    std::vector<int> inv(n, -1);
    for (int i = 0; i < n; ++i) {
        const int e = e2x_host_inv[i];
        UG_REQUIRE(e >= 0 && e < n && inv[e] < 0, UG4GB_ERR_INVALID, "permutation: not a bijection of 0..n-1");
        inv[e] = i;
    }
    p->ext_to_eng.alloc(n > 0 ? n : 1);
    p->eng_to_ext.alloc(n > 0 ? n : 1);
    if (n) {
        copy_in(c, p->ext_to_eng.p, e2x_host_inv.data(), sizeof(int) * (size_t)n);
        copy_in(c, p->eng_to_ext.p, inv.data(), sizeof(int) * (size_t)n);
    }
    UG_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace

extern "C" {

int ug4gb_perm_create(ug4gb_ctx *ctx, int n, const int *engine_of_external, ug4gb_perm **out)
{
    if (!ctx || !out || n < 0 || (n > 0 && !engine_of_external)) return UG4GB_ERR_INVALID;
    *out = nullptr;
    ug4gb_perm *p = new ug4gb_perm;
    p->ctx = ctx;
    p->n = n;
    const int rc = guarded(ctx, [&] {
        std::vector<int> h(n);
        if (n) {
            if (is_device_ptr(engine_of_external)) copy_out(ctx->c, h.data(), engine_of_external, sizeof(int) * (size_t)n);
            else std::memcpy(h.data(), engine_of_external, sizeof(int) * (size_t)n);
        }
        make_perm(p, h);
    });
    if (rc != UG4GB_OK) {
        delete p;
        return rc;
    }
    ug4gb_ctx_retain(ctx);
    *out = p;
    return UG4GB_OK;
}

int ug4gb_perm_from_positions(ug4gb_ctx *ctx, const ug4gb_grid *g, int level, int n, const double *positions,
                              double tol, ug4gb_perm **out)
{
    if (!ctx || !g || !out || !positions || level < 0 || level >= (int)g->lev.size()) return UG4GB_ERR_INVALID;
    if (!(tol > 0.0)) return UG4GB_ERR_INVALID;
    *out = nullptr;
    std::vector<int> e2x;
    const int rc = guarded(ctx, [&] {
        const Level &L = g->lev[level];
        UG_REQUIRE(n == L.nv, UG4GB_ERR_INVALID, "perm_from_positions: the level has another number of vertices");
        std::vector<double> xe((size_t)L.nv * L.dim);
        copy_out(ctx->c, xe.data(), L.coords.p, sizeof(double) * xe.size());
        std::vector<double> xx((size_t)n * L.dim);
        if (is_device_ptr(positions)) copy_out(ctx->c, xx.data(), positions, sizeof(double) * xx.size());
        else std::memcpy(xx.data(), positions, sizeof(double) * xx.size());
        // engine vertices by their position rounded to the tolerance grid;
        // an external position is looked up in its cell and the neighbours
        typedef std::vector<long long> Key;
        std::map<Key, std::vector<int>> cells;
        auto key_of = [&](const double *x, const int *shift) {
            Key k(L.dim);
            for (int d = 0; d < L.dim; ++d) k[d] = (long long)std::floor(x[d] / tol) + (shift ? shift[d] : 0);
            return k;
        };
        for (int v = 0; v < L.nv; ++v) cells[key_of(&xe[(size_t)v * L.dim], nullptr)].push_back(v);
        e2x.assign(n, -1);
        std::vector<char> used(L.nv, 0);
        for (int i = 0; i < n; ++i) {
            const double *x = &xx[(size_t)i * L.dim];
            int found = -1;
            int sh[3];
            const int lim = (L.dim == 3) ? 27 : 9;
            for (int s = 0; s < lim && found < 0; ++s) {
                sh[0] = s % 3 - 1;
                sh[1] = (s / 3) % 3 - 1;
                sh[2] = s / 9 - 1;
                auto it = cells.find(key_of(x, sh));
                if (it == cells.end()) continue;
                for (int v : it->second) {
                    double d2 = 0.0;
                    for (int d = 0; d < L.dim; ++d) {
                        const double t = xe[(size_t)v * L.dim + d] - x[d];
                        d2 += t * t;
                    }
                    if (d2 <= tol * tol && !used[v]) {
                        found = v;
                        break;
                    }
                }
            }
            UG_REQUIRE(found >= 0, UG4GB_ERR_INVALID, "perm_from_positions: a position matches no vertex of the level");
            used[found] = 1;
            e2x[i] = found;
        }
    });
    if (rc != UG4GB_OK) return rc;
    return ug4gb_perm_create(ctx, n, e2x.data(), out);
}

int ug4gb_perm_vector(const ug4gb_perm *p, int to_external, const ug4gb_vector *src, ug4gb_vector *dst)
{
    if (!p || !src || !dst || src == dst || src->n != p->n || dst->n != p->n) return UG4GB_ERR_INVALID;
    return guarded(p->ctx, [&] {
        Ctx &c = p->ctx->c;
        // external x[i] = engine y[perm[i]]; engine y[e] = external x[inv[e]]
        const int *idx = to_external ? p->ext_to_eng.p : p->eng_to_ext.p;
        if (p->n) UG_LAUNCH(c, k_gather_vec, div_up(p->n, 256), 256, 0, p->n, idx, src->d, dst->d);
    });
}

int ug4gb_perm_matrix(ug4gb_perm *p, int to_external, const ug4gb_matrix *A, ug4gb_matrix *B)
{
    if (!p || !A || !B || A == B || A->A.nrows != p->n || A->A.ncols != p->n) return UG4GB_ERR_INVALID;
    return guarded(p->ctx, [&] {
        Ctx &c = p->ctx->c;
        const int n = p->n;
        // B(i, j) = A(rowmap[i], rowmap[j]); columns of A map through colmap
        const int *rowmap = to_external ? p->ext_to_eng.p : p->eng_to_ext.p;
        const int *colmap = to_external ? p->eng_to_ext.p : p->ext_to_eng.p;
        ug4gb_perm::MatMap &mm = p->mat[to_external ? 1 : 0];
        const uint64_t src = A->pattern_key();
        const uint64_t key = src ? (src ^ (to_external ? 0x5a5a000000000000ULL : 0xa5a5000000000000ULL)) : 0;
        if (key && mm.key == src && B->derived_key == key && mm.nnz == A->A.nnz && B->A.nnz == A->A.nnz) {
            if (A->A.nnz)
                UG_LAUNCH(c, k_gather_vals, div_up(A->A.nnz, (int64_t)256), 256, 0, A->A.nnz, mm.map.p, A->A.val.p,
                          B->A.val.p);
        } else {
            Csr &T = B->A;
            T.nrows = T.ncols = n;
            T.nnz = A->A.nnz;
            DevBuf<int> len;
            len.alloc(n + 1);
            UG_CUDA(cudaMemsetAsync(len.p, 0, sizeof(int) * (size_t)(n + 1), c.stream));
            if (n) UG_LAUNCH(c, k_perm_row_len, div_up(n, 256), 256, 0, n, rowmap, A->A.rowptr.p, len.p);
            T.rowptr.alloc(n + 1);
            int64_t nnz = 0;
            exclusive_scan_int(c, len.p, T.rowptr.p, n + 1, &nnz);
            UG_REQUIRE(nnz == A->A.nnz, UG4GB_ERR_INVALID, "perm_matrix: inconsistent row pointers");
            T.col.alloc(nnz > 0 ? nnz : 1);
            T.val.alloc(nnz > 0 ? nnz : 1);
            if (n) {
                UG_LAUNCH(c, k_perm_fill, div_up(n, 256), 256, 0, n, rowmap, colmap, A->A.rowptr.p, A->A.col.p,
                          T.rowptr.p, T.col.p, T.val.p);
                UG_LAUNCH(c, k_sort_row_pairs, div_up(n, 256), 256, 0, T.rowptr.p, T.col.p, T.val.p, n);
            }
            mm.map.alloc(nnz > 0 ? nnz : 1);
            if (nnz) {
                UG_LAUNCH(c, k_src_to_map, div_up(nnz, (int64_t)256), 256, 0, nnz, T.val.p, mm.map.p);
                UG_LAUNCH(c, k_gather_vals, div_up(nnz, (int64_t)256), 256, 0, nnz, mm.map.p, A->A.val.p, T.val.p);
            }
            UG_CUDA(cudaStreamSynchronize(c.stream));
            mm.key = src;
            mm.nnz = nnz;
        }
        B->op_valid = false;
        B->pattern_grid = 0;
        B->pattern_level = -1;
        B->derived_key = key;
    });
}

void ug4gb_perm_destroy(ug4gb_perm *p)
{
    if (!p) return;
    ug4gb_ctx *ctx = p->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    delete p;
    ug4gb_ctx_release(ctx);
}

}  // extern "C"

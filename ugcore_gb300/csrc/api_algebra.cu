// api_algebra.cu -- the rest of the SparseMatrix / Vector interface that
// ugcore's algebra templates call on a matrix_type / vector_type
// (lib_algebra/cpu_algebra/sparsematrix.h:98-330, vector.h:54-230): pattern
// and value resets, copies and scaling, apply_ignore_zero_rows, entry and
// row access from the host, scatter-add of element contributions, max norm.
// These are set-up and glue operations; the solve path does not use them.
#include <cmath>
#include <vector>

#include "gmg.cuh"

using namespace ug4gb;

namespace {

template <class F>
int guarded(ug4gb_ctx *ctx, F &&f)
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

__global__ void k_scale(double *v, int64_t n, double a)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) v[i] *= a;
}

__global__ void k_copy_scaled(const double *src, double *dst, int64_t n, double a)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = a * src[i];
}

// SparseMatrix::apply_ignore_zero_rows (sparsematrix_impl.h:270-288): rows
// without stored entries keep dest; the others get sum_k (beta a_ik) w_k in
// stored order
__global__ void k_apply_ignore_zero_rows(const int *rowptr, const int *col, const double *val, int n, double beta,
                                         const double *w, double *dest)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int a0 = rowptr[r], a1 = rowptr[r + 1];
    if (a0 == a1) return;
    double s = (beta * val[a0]) * w[col[a0]];
    for (int a = a0 + 1; a < a1; ++a) s += (beta * val[a]) * w[col[a]];
    dest[r] = s;
}

// A(r, c) += v for entries of the pattern; err = 1 for an entry outside it
__global__ void k_add_entries(const int *rowptr, const int *col, double *val, int nrows, int ncols, int n,
                              const int *r, const int *c, const double *v, int *err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int row = r[i], cc = c[i];
    if (row < 0 || row >= nrows || cc < 0 || cc >= ncols) {
        atomicExch(err, 1);
        return;
    }
    int lo = rowptr[row], hi = rowptr[row + 1] - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (col[mid] == cc) {
            atomicAdd(val + mid, v[i]);
            return;
        }
        if (col[mid] < cc) lo = mid + 1;
        else hi = mid - 1;
    }
    atomicExch(err, 1);
}

__global__ void k_gather(const double *v, int nv, const int *idx, int n, double *out, int *err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (idx[i] < 0 || idx[i] >= nv) {
        atomicExch(err, 1);
        return;
    }
    out[i] = v[idx[i]];
}

__global__ void k_scatter(double *v, int nv, const int *idx, int n, const double *in, int *err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (idx[i] < 0 || idx[i] >= nv) {
        atomicExch(err, 1);
        return;
    }
    v[idx[i]] = in[i];
}

// max |v_i|: per-block maxima, then one block over them (absolute values
// compare as their bit patterns: no atomics on doubles needed)
__global__ void k_absmax_blocks(const double *v, int64_t n, double *part)
{
    __shared__ double sh[256];
    double m = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        m = fmax(m, fabs(v[i]));
    sh[threadIdx.x] = m;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

void check_err(Ctx &c, const DevBuf<int> &err, const char *what)
{
    int h = 0;
    UG_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    UG_REQUIRE(!h, UG4GB_ERR_INVALID, what);
}

}  // namespace

extern "C" {

int ug4gb_matrix_resize_and_clear(ug4gb_matrix *A, int num_rows, int num_cols)
{
    if (!A || num_rows < 0 || num_cols < 0) return UG4GB_ERR_INVALID;
    return guarded(A->ctx, [&] {
        Ctx &c = A->ctx->c;
        A->A.nrows = num_rows;
        A->A.ncols = num_cols;
        A->A.nnz = 0;
        A->A.rowptr.alloc(num_rows + 1);
        A->A.col.alloc(1);
        A->A.val.alloc(1);
        UG_CUDA(cudaMemsetAsync(A->A.rowptr.p, 0, sizeof(int) * (size_t)(num_rows + 1), c.stream));
        UG_CUDA(cudaStreamSynchronize(c.stream));
        A->op_valid = false;
        A->pattern_grid = 0;
        A->derived_key = 0;
        A->pattern_level = -1;
    });
}

int ug4gb_matrix_clear_retain_structure(ug4gb_matrix *A)
{
    if (!A) return UG4GB_ERR_INVALID;
    return guarded(A->ctx, [&] {
        Ctx &c = A->ctx->c;
        if (A->A.nnz) UG_CUDA(cudaMemsetAsync(A->A.val.p, 0, sizeof(double) * (size_t)A->A.nnz, c.stream));
        UG_CUDA(cudaStreamSynchronize(c.stream));
        A->op_valid = false;
    });
}

int ug4gb_matrix_set_as_copy_of(ug4gb_matrix *A, const ug4gb_matrix *B, double scale)
{
    if (!A || !B) return UG4GB_ERR_INVALID;
    if (A == B) return ug4gb_matrix_scale(A, scale);
    return guarded(A->ctx, [&] {
        Ctx &c = A->ctx->c;
        const Csr &S = B->A;
        A->A.nrows = S.nrows;
        A->A.ncols = S.ncols;
        A->A.nnz = S.nnz;
        A->A.rowptr.alloc(S.nrows + 1);
        A->A.col.alloc(S.nnz > 0 ? S.nnz : 1);
        A->A.val.alloc(S.nnz > 0 ? S.nnz : 1);
        UG_CUDA(cudaMemcpyAsync(A->A.rowptr.p, S.rowptr.p, sizeof(int) * (size_t)(S.nrows + 1),
                                cudaMemcpyDeviceToDevice, c.stream));
        if (S.nnz) {
            UG_CUDA(cudaMemcpyAsync(A->A.col.p, S.col.p, sizeof(int) * (size_t)S.nnz, cudaMemcpyDeviceToDevice,
                                    c.stream));
            UG_LAUNCH(c, k_copy_scaled, div_up(S.nnz, 256), 256, 0, S.val.p, A->A.val.p, S.nnz, scale);
        }
        UG_CUDA(cudaStreamSynchronize(c.stream));
        A->op_valid = false;
        A->pattern_grid = B->pattern_grid;
        A->pattern_level = B->pattern_level;
        A->derived_key = B->derived_key;
    });
}

int ug4gb_matrix_scale(ug4gb_matrix *A, double alpha)
{
    if (!A) return UG4GB_ERR_INVALID;
    return guarded(A->ctx, [&] {
        Ctx &c = A->ctx->c;
        if (A->A.nnz) UG_LAUNCH(c, k_scale, div_up(A->A.nnz, 256), 256, 0, A->A.val.p, A->A.nnz, alpha);
        UG_CUDA(cudaStreamSynchronize(c.stream));
        A->op_valid = false;
    });
}

int ug4gb_matrix_apply_ignore_zero_rows(const ug4gb_matrix *A, ug4gb_vector *dest, double beta,
                                        const ug4gb_vector *w)
{
    if (!A || !dest || !w || dest->n != A->A.nrows || w->n != A->A.ncols || dest == w) return UG4GB_ERR_INVALID;
    return guarded(A->ctx, [&] {
        Ctx &c = A->ctx->c;
        UG_LAUNCH(c, k_apply_ignore_zero_rows, div_up(A->A.nrows, 256), 256, 0, A->A.rowptr.p, A->A.col.p,
                  A->A.val.p, A->A.nrows, beta, w->d, dest->d);
        UG_CUDA(cudaStreamSynchronize(c.stream));
    });
}

int ug4gb_matrix_get_row(const ug4gb_matrix *A, int row, int *cols, double *vals, int capacity)
{
    if (!A || row < 0 || row >= A->A.nrows) return UG4GB_ERR_INVALID;
    int len = 0;
    const int rc = guarded(A->ctx, [&] {
        Ctx &c = A->ctx->c;
        int rp[2];
        copy_out(c, rp, A->A.rowptr.p + row, sizeof(int) * 2);
        len = rp[1] - rp[0];
        const int m = len < capacity ? len : capacity;
        if (m > 0 && cols) copy_out(c, cols, A->A.col.p + rp[0], sizeof(int) * (size_t)m);
        if (m > 0 && vals) copy_out(c, vals, A->A.val.p + rp[0], sizeof(double) * (size_t)m);
    });
    return rc != UG4GB_OK ? rc : len;
}

int ug4gb_matrix_add_entries(ug4gb_matrix *A, int n, const int *rows, const int *cols, const double *vals)
{
    if (!A || n < 0 || (n > 0 && (!rows || !cols || !vals))) return UG4GB_ERR_INVALID;
    if (n == 0) return UG4GB_OK;
    return guarded(A->ctx, [&] {
        Ctx &c = A->ctx->c;
        DevBuf<int> r, cc, err;
        DevBuf<double> v;
        r.alloc(n);
        cc.alloc(n);
        v.alloc(n);
        err.alloc(1);
        copy_in(c, r.p, rows, sizeof(int) * (size_t)n);
        copy_in(c, cc.p, cols, sizeof(int) * (size_t)n);
        copy_in(c, v.p, vals, sizeof(double) * (size_t)n);
        UG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), c.stream));
        UG_LAUNCH(c, k_add_entries, div_up(n, 256), 256, 0, A->A.rowptr.p, A->A.col.p, A->A.val.p, A->A.nrows,
                  A->A.ncols, n, r.p, cc.p, v.p, err.p);
        check_err(c, err, "add_entries: an entry outside the matrix pattern");
        A->op_valid = false;
    });
}

int ug4gb_vector_maxnorm(const ug4gb_vector *v, double *out)
{
    if (!v || !out) return UG4GB_ERR_INVALID;
    return guarded(v->ctx, [&] {
        Ctx &c = v->ctx->c;
        const int nb = 256;
        DevBuf<double> part, res;
        part.alloc(nb);
        res.alloc(1);
        UG_LAUNCH(c, k_absmax_blocks, nb, 256, 0, v->d, (int64_t)v->n, part.p);
        UG_LAUNCH(c, k_absmax_blocks, 1, 256, 0, part.p, (int64_t)nb, res.p);
        copy_out(c, out, res.p, sizeof(double));
    });
}

int ug4gb_vector_get_values(const ug4gb_vector *v, int n, const int *idx, double *vals)
{
    if (!v || n < 0 || (n > 0 && (!idx || !vals))) return UG4GB_ERR_INVALID;
    if (n == 0) return UG4GB_OK;
    return guarded(v->ctx, [&] {
        Ctx &c = v->ctx->c;
        DevBuf<int> id, err;
        DevBuf<double> o;
        id.alloc(n);
        o.alloc(n);
        err.alloc(1);
        copy_in(c, id.p, idx, sizeof(int) * (size_t)n);
        UG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), c.stream));
        UG_LAUNCH(c, k_gather, div_up(n, 256), 256, 0, v->d, v->n, id.p, n, o.p, err.p);
        check_err(c, err, "get_values: index out of range");
        copy_out(c, vals, o.p, sizeof(double) * (size_t)n);
    });
}

int ug4gb_vector_set_values(ug4gb_vector *v, int n, const int *idx, const double *vals)
{
    if (!v || n < 0 || (n > 0 && (!idx || !vals))) return UG4GB_ERR_INVALID;
    if (n == 0) return UG4GB_OK;
    return guarded(v->ctx, [&] {
        Ctx &c = v->ctx->c;
        DevBuf<int> id, err;
        DevBuf<double> in;
        id.alloc(n);
        in.alloc(n);
        err.alloc(1);
        copy_in(c, id.p, idx, sizeof(int) * (size_t)n);
        copy_in(c, in.p, vals, sizeof(double) * (size_t)n);
        UG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), c.stream));
        UG_LAUNCH(c, k_scatter, div_up(n, 256), 256, 0, v->d, v->n, id.p, n, in.p, err.p);
        check_err(c, err, "set_values: index out of range");
    });
}

}  // extern "C"

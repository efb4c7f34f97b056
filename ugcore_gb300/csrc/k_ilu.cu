// k_ilu.cu -- ILU(0) smoother in multicolour order (GPU variant of ugcore's
// ILU, lib_algebra/operator/preconditioner/ilu.h:109-210 factorisation,
// :250-290 solve).
//
// ugcore factorises A = L U on A's pattern in the index order and applies
// the two triangular solves sequentially.  Here the order is colour-major
// (vertex colours: parity on structured levels, greedy on unstructured ones):
// vertices of one colour are never coupled, so the rows of a colour are
// factorised in parallel once the earlier colours are done, and each
// triangular solve is one launch per colour.  It is ILU(0) of the permuted
// operator P A P^T, a different (parallel) preconditioner than ugcore's
// index-order ILU, with the same set-up rule (IKJ, fill restricted to the
// pattern of A) and the same use as a smoother (t = damp (L U)^{-1} d).
//
// Storage: a copy of the level CRS whose rows are re-ordered by (colour,
// column): the strictly lower part (earlier colours) first, then the
// diagonal, then the upper part; L is unit lower (its multipliers stored in
// the lower part), U the diagonal and upper part.  Factorisation in FP64,
// the factors kept in the level precision.
#include "common.cuh"
#include "k_solve.cuh"

namespace ug4gb {

namespace {

constexpr int NTI = 256;

__device__ __forceinline__ long long ekey(const int *color, int n, int j) { return (long long)color[j] * n + j; }

// rows re-ordered by (colour, column); nlow = entries of earlier colours
__global__ void k_ilu_order(const int *rowptr, int *col, double *val, const int *color, int n, int *nlow)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= n) return;
    const int a0 = rowptr[r], a1 = rowptr[r + 1];
    for (int a = a0 + 1; a < a1; ++a) {
        const int cc = col[a];
        const double vv = val[a];
        const long long kk = ekey(color, n, cc);
        int b = a - 1;
        while (b >= a0 && ekey(color, n, col[b]) > kk) {
            col[b + 1] = col[b];
            val[b + 1] = val[b];
            --b;
        }
        col[b + 1] = cc;
        val[b + 1] = vv;
    }
    // position of the diagonal: entries ordered before it (earlier colours)
    int lo = 0;
    const long long kr = ekey(color, n, r);
    for (int a = a0; a < a1; ++a) lo += ekey(color, n, col[a]) < kr;
    nlow[r] = lo;
}

// IKJ ILU(0) of the rows of one colour (all earlier colours are final)
__global__ void k_ilu_factor(const int *rowptr, const int *col, double *val, const int *color, int n,
                             const int *nlow, const int *rows, int nrows, int *err)
{
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrows) return;
    const int i = rows[q];
    const int a0 = rowptr[i], a1 = rowptr[i + 1], al = a0 + nlow[i];
    for (int p = a0; p < al; ++p) {
        const int k = col[p];
        const double ukk = val[rowptr[k] + nlow[k]];
        if (!(ukk != 0.0)) {
            atomicExch(err, 1);
            return;
        }
        const double l = val[p] / ukk;
        val[p] = l;
        // a_ij -= l u_kj for the entries j after k in row i that row k holds
        const int k0 = rowptr[k] + nlow[k] + 1, k1 = rowptr[k + 1];
        for (int s = p + 1; s < a1; ++s) {
            const long long js = ekey(color, n, col[s]);
            int lo = k0, hi = k1 - 1;
            while (lo <= hi) {
                const int mid = (lo + hi) >> 1;
                const long long km = ekey(color, n, col[mid]);
                if (km == js) {
                    val[s] -= l * val[mid];
                    break;
                }
                if (km < js) lo = mid + 1;
                else hi = mid - 1;
            }
        }
    }
    if (!(val[al] != 0.0)) atomicExch(err, 1);
}

template <class V>
__global__ void k_ilu_convert(const double *val, int nnz, V *out)
{
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < nnz) out[a] = (V)val[a];
}

template <class V>
__global__ void k_ilu_uinv(const int *rowptr, const int *nlow, const double *val, int n, V *uinv)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < n) uinv[r] = (V)(1.0 / val[rowptr[r] + nlow[r]]);
}

// y_i = d_i - sum_{lower} l_ij y_j   (rows of one colour)
template <class V>
__global__ void __launch_bounds__(NTI) k_ilu_fwd(const int *__restrict__ rowptr, const int *__restrict__ col,
                                                 const V *__restrict__ val, const int *__restrict__ nlow,
                                                 const int *__restrict__ rows, int nrows, const V *__restrict__ d,
                                                 V *__restrict__ y, const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    const int stride = gridDim.x * NTI;
    for (int q = blockIdx.x * NTI + threadIdx.x; q < nrows; q += stride) {
        const int i = rows[q];
        const int a0 = rowptr[i], al = a0 + nlow[i];
        V s = d[i];
        for (int a = a0; a < al; ++a) s -= val[a] * y[col[a]];
        y[i] = s;
    }
}

// t_i = (y_i - sum_{upper} u_ij t_j) / u_ii   (rows of one colour)
template <class V>
__global__ void __launch_bounds__(NTI) k_ilu_bwd(const int *__restrict__ rowptr, const int *__restrict__ col,
                                                 const V *__restrict__ val, const int *__restrict__ nlow,
                                                 const V *__restrict__ uinv, const int *__restrict__ rows,
                                                 int nrows, const V *__restrict__ y, V *__restrict__ t,
                                                 const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    const int stride = gridDim.x * NTI;
    for (int q = blockIdx.x * NTI + threadIdx.x; q < nrows; q += stride) {
        const int i = rows[q];
        const int a1 = rowptr[i + 1], ad = rowptr[i] + nlow[i];
        V s = y[i];
        for (int a = ad + 1; a < a1; ++a) s -= val[a] * t[col[a]];
        t[i] = s * uinv[i];
    }
}

template <class V>
__global__ void k_ilu_scale(int n, V *t, V damp, const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) t[i] *= damp;
}

int ilu_grid(const Ctx &c, int nrows)
{
    const int need = (int)div_up(nrows > 0 ? nrows : 1, NTI);
    const int cap = c.num_sms * 8;
    return need < cap ? need : cap;
}

}  // namespace

template <class V>
void ilu_setup(Ctx &c, const Csr &A, const int *color, const std::vector<DevBuf<int>> &crow,
               const std::vector<int> &ncrow, IluFactors<V> &F)
{
    const int n = A.nrows;
    F.n = n;
    F.rowptr.alloc(n + 1);
    F.col.alloc(A.nnz > 0 ? A.nnz : 1);
    F.nlow.alloc(n > 0 ? n : 1);
    DevBuf<double> v64;
    v64.alloc(A.nnz > 0 ? A.nnz : 1);
    UG_CUDA(cudaMemcpyAsync(F.rowptr.p, A.rowptr.p, sizeof(int) * (size_t)(n + 1), cudaMemcpyDeviceToDevice, c.stream));
    UG_CUDA(cudaMemcpyAsync(F.col.p, A.col.p, sizeof(int) * (size_t)A.nnz, cudaMemcpyDeviceToDevice, c.stream));
    UG_CUDA(cudaMemcpyAsync(v64.p, A.val.p, sizeof(double) * (size_t)A.nnz, cudaMemcpyDeviceToDevice, c.stream));
    UG_LAUNCH(c, k_ilu_order, div_up(n, 128), 128, 0, F.rowptr.p, F.col.p, v64.p, color, n, F.nlow.p);
    DevBuf<int> err;
    err.alloc(1);
    UG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), c.stream));
    for (size_t q = 0; q < crow.size(); ++q)
        if (ncrow[q] > 0)
            UG_LAUNCH(c, k_ilu_factor, div_up(ncrow[q], 128), 128, 0, F.rowptr.p, F.col.p, v64.p, color, n, F.nlow.p,
                      crow[q].p, ncrow[q], err.p);
    F.val.alloc(A.nnz > 0 ? A.nnz : 1);
    F.uinv.alloc(n > 0 ? n : 1);
    UG_LAUNCH(c, k_ilu_convert<V>, div_up(A.nnz, 256), 256, 0, v64.p, (int)A.nnz, F.val.p);
    UG_LAUNCH(c, k_ilu_uinv<V>, div_up(n, 256), 256, 0, F.rowptr.p, F.nlow.p, v64.p, n, F.uinv.p);
    int h = 0;
    UG_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    UG_REQUIRE(!h, UG4GB_ERR_SINGULAR, "ILU: zero pivot in the multicolour factorisation");
}

template <class V>
void ilu_apply(Ctx &c, const IluFactors<V> &F, const std::vector<DevBuf<int>> &crow, const std::vector<int> &ncrow,
               const V *d, V *y, V *t, double damp, const int *skip)
{
    for (size_t q = 0; q < crow.size(); ++q)
        if (ncrow[q] > 0)
            UG_LAUNCH_PDL(c, k_ilu_fwd<V>, ilu_grid(c, ncrow[q]), NTI, 0, F.rowptr.p, F.col.p, F.val.p, F.nlow.p,
                          crow[q].p, ncrow[q], d, y, skip);
    for (size_t q = crow.size(); q-- > 0;)
        if (ncrow[q] > 0)
            UG_LAUNCH_PDL(c, k_ilu_bwd<V>, ilu_grid(c, ncrow[q]), NTI, 0, F.rowptr.p, F.col.p, F.val.p, F.nlow.p,
                          F.uinv.p, crow[q].p, ncrow[q], y, t, skip);
    if (damp != 1.0) UG_LAUNCH_PDL(c, k_ilu_scale<V>, div_up(F.n, 256), 256, 0, F.n, t, (V)damp, skip);
}

template void ilu_setup<double>(Ctx &, const Csr &, const int *, const std::vector<DevBuf<int>> &,
                                const std::vector<int> &, IluFactors<double> &);
template void ilu_setup<float>(Ctx &, const Csr &, const int *, const std::vector<DevBuf<int>> &,
                               const std::vector<int> &, IluFactors<float> &);
template void ilu_apply<double>(Ctx &, const IluFactors<double> &, const std::vector<DevBuf<int>> &,
                                const std::vector<int> &, const double *, double *, double *, double, const int *);
template void ilu_apply<float>(Ctx &, const IluFactors<float> &, const std::vector<DevBuf<int>> &,
                               const std::vector<int> &, const float *, float *, float *, double, const int *);

}  // namespace ug4gb

// api_gmg.cu -- AssembledMultiGridCycle on the GPU: level setup (operator
// copy / re-assembly, StdTransfer P and R with Dirichlet adjustment, Jacobi
// or multicolour Gauss-Seidel smoother, dense LU base) and the cycle as a
// fixed sequence of fused kernels, replayed from a CUDA graph.
//
// Reference: lib_disc/operator/linear_operator/multi_grid_solver/
// mg_solver_impl.hpp (init :380, init_transfer :1078, init_smoother :1137,
// init_base_solver :1173, apply :176, lmgc :2091, presmooth_and_restriction
// :1687, prolongation_and_postsmooth :1820, base_solve :1969) for a fully
// refined hierarchy, where the last defect update after post-smoothing and
// after the base solve is dead (m_LocalFullRefLevel == top level) except on
// the top level, where it only feeds the returned correction's defect and
// is skipped here because apply() returns the correction alone.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "disc.cuh"
#include "gmg.cuh"

using namespace ug4gb;

namespace ug4gb {

void disc_assemble(ug4gb_disc *d, int level, ug4gb_matrix *A, double *b, const TimeScale *ts);

// ------------------------------------------------------------- helpers ---
// Jacobi factors of a level in FP64 and in the level precision V (one
// launch: the re-initialisation of small levels is bound by launches)
template <class V>
__global__ void k_diag_inv(const int *rowptr, const int *col, const double *val, int n, double damp, int smoother,
                           double *dinv, double *dfac, V *dinv_v, V *dfac_v)
{
    PDL_ENTRY();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double a = 0.0;
    for (int q = rowptr[i]; q < rowptr[i + 1]; ++q)
        if (col[q] == i) a = val[q];
    double di, df;
    if (smoother == UG4GB_SMOOTHER_JACOBI) {
        // Jacobi::preprocess (jacobi.h:196-208): diagInv = 1 / (a_ii * (1/damp))
        double m = a * (1. / damp);
        di = 1. / m;
        df = m;
    } else {
        di = damp / a;
        df = 1.0;
    }
    dinv[i] = di;
    if (dfac) dfac[i] = df;
    if constexpr (sizeof(V) == 4) {
        dinv_v[i] = f64_to_f32(di);
        if (dfac_v) dfac_v[i] = f64_to_f32(df);
    } else {
        dinv_v[i] = (V)di;
        if (dfac_v) dfac_v[i] = (V)df;
    }
}

__global__ void k_scale_vals(double *val, int64_t nnz, double s)
{
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nnz) val[i] *= s;
}

template <class V>
__global__ void k_to_v(const double *in, V *out, int n)
{
    PDL_ENTRY();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        if constexpr (sizeof(V) == 4) out[i] = f64_to_f32(in[i]);
        else out[i] = (V)in[i];
    }
}

// P rows from the parent table; Dirichlet fine rows: values 0, and 1 to a
// vertex parent (DirichletBoundary::adjust_prolongation)
__global__ void k_build_P(const int *npar, const int *par, const unsigned char *bnd, int nf, int *rowptr_len,
                          int *col, double *val, const int *rowptr, int mode)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nf) return;
    int n = npar[i];
    if (mode == 0) {
        rowptr_len[i] = n;
        return;
    }
    double w = (n == 1) ? 1.0 : (n == 2 ? 0.5 : (n == 4 ? 0.25 : 0.125));
    int a0 = rowptr[i];
    for (int j = 0; j < n; ++j) {
        col[a0 + j] = par[8 * (size_t)i + j];
        double v = w;
        if (bnd[i]) v = (n == 1) ? 1.0 : 0.0;
        val[a0 + j] = v;
    }
}

// rows of coarse Dirichlet vertices in R: 0, and 1 at the fine child
// (DirichletBoundary::adjust_restriction)
__global__ void k_adjust_R(const int *npar, const int *par, const unsigned char *bnd, int nf, const int *rowptr,
                           const int *col, double *val)
{
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf || !bnd[f] || npar[f] != 1) return;
    int c = par[8 * (size_t)f];
    for (int a = rowptr[c]; a < rowptr[c + 1]; ++a) val[a] = (col[a] == f) ? 1.0 : 0.0;
}

// transposed operator: Dirichlet rows reset to identity
__global__ void k_dirichlet_identity(const unsigned char *bnd, int n, const int *rowptr, const int *col, double *val)
{
    PDL_ENTRY();
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n || !bnd[v]) return;
    for (int a = rowptr[v]; a < rowptr[v + 1]; ++a) val[a] = (col[a] == v) ? 1.0 : 0.0;
}

// rows of colour c in increasing order (stable compaction by a scan of the flags)
__global__ void k_colour_flag(const int *color, int n, int c, int *flag)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flag[i] = (color[i] == c) ? 1 : 0;
}

__global__ void k_colour_scatter(const int *color, int n, int c, const int *pos, int *rows)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && color[i] == c) rows[pos[i]] = i;
}

template <class V>
__global__ void k_vadd(int n, V *a, const V *b, const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += b[i];
}

template <class V>
__global__ void k_vscale(int n, V *a, V f, const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] *= f;
}

template <class V>
__global__ void k_zero(int n, V *a, const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = (V)0;
}

// dense inverse of the base matrix through a partially pivoted LU, in the
// order of LUDecomp / SolveLU (lib_algebra/small_algebra/no_lapack/lu_decomp.h)
static void dense_lu_inverse(int n, std::vector<double> &M, std::vector<double> &inv)
{
    std::vector<int> piv(n);
    for (int k = 0; k < n; ++k) {
        int big = k;
        for (int j = k + 1; j < n; ++j)
            if (std::fabs(M[(size_t)big * n + k]) < std::fabs(M[(size_t)j * n + k])) big = j;
        if (big != k)
            for (int j = 0; j < n; ++j) std::swap(M[(size_t)k * n + j], M[(size_t)big * n + j]);
        piv[k] = big;
        UG_REQUIRE(std::fabs(M[(size_t)k * n + k]) >= 1e-10, UG4GB_ERR_SINGULAR,
                   "GMG base solver: LU pivot below 1e-10 (singular base matrix)");
        for (int i = k + 1; i < n; ++i) {
            M[(size_t)i * n + k] = M[(size_t)i * n + k] / M[(size_t)k * n + k];
            for (int j = k + 1; j < n; ++j) M[(size_t)i * n + j] -= M[(size_t)i * n + k] * M[(size_t)k * n + j];
        }
    }
    // the n solves with the unit vectors, all columns at once (X row-major,
    // each element with the operations of one solve, in the same order):
    // X = P I, then X(i,:) -= M(i,k) X(k,:) for k < i in increasing k, then
    // X(i,:) -= M(i,k) X(k,:) for k > i in increasing k and X(i,:) /= M(i,i)
    inv.assign((size_t)n * n, 0.0);
    double *X = inv.data();
    for (int i = 0; i < n; ++i) X[(size_t)i * n + i] = 1.0;
    for (int i = 0; i < n; ++i)
        if (i < piv[i])
            for (int c = 0; c < n; ++c) std::swap(X[(size_t)i * n + c], X[(size_t)piv[i] * n + c]);
    for (int i = 0; i < n; ++i) {
        double *xi = X + (size_t)i * n;
        for (int k = 0; k < i; ++k) {
            const double m = M[(size_t)i * n + k];
            const double *xk = X + (size_t)k * n;
            for (int c = 0; c < n; ++c) xi[c] -= m * xk[c];
        }
    }
    for (int i = n - 1; i >= 0; --i) {
        double *xi = X + (size_t)i * n;
        for (int k = i + 1; k < n; ++k) {
            const double m = M[(size_t)i * n + k];
            const double *xk = X + (size_t)k * n;
            for (int c = 0; c < n; ++c) xi[c] -= m * xk[c];
        }
        const double d = M[(size_t)i * n + i];
        for (int c = 0; c < n; ++c) xi[c] = xi[c] / d;
    }
}

// The same factorisation on the device for bases of at most kDeviceLuMax
// unknowns (no host round trip in a re-initialisation): one block, M in
// shared memory, the inverse X built in place in the output array.  Partial
// pivoting as above (the first row of the largest magnitude), row swaps
// applied to X = I as they happen, products and differences rounded
// separately; the forward substitution runs over all columns at once,
// right-looking (subtracting in increasing column order), the backward one
// column by column in the order of SolveLU, so that each element of the
// inverse takes the operations of the host statement above.  *status = 1 on a
// pivot below 1e-10 (the output is then not an inverse).
constexpr int kDeviceLuMax = 160;
constexpr int kLuThreads = 256;

__global__ void __launch_bounds__(kLuThreads) k_base_lu(const int *__restrict__ rowptr, const int *__restrict__ col,
                                                        const double *__restrict__ val, int n,
                                                        double *__restrict__ inv, int *__restrict__ status)
{
    PDL_ENTRY();
    extern __shared__ double lu_sh[];
    __shared__ int big_sh;
    double *M = lu_sh, *X = inv;
    const int tid = threadIdx.x, nt = blockDim.x, nn = n * n;
    for (int i = tid; i < nn; i += nt) {
        M[i] = 0.0;
        X[i] = 0.0;
    }
    __syncthreads();
    for (int r = tid; r < n; r += nt) {
        for (int a = rowptr[r]; a < rowptr[r + 1]; ++a) M[r * n + col[a]] = val[a];
        X[r * n + r] = 1.0;
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (tid < 32) {
            // each lane: the first largest |M[j][k]| of its rows j >= k; then
            // the larger value wins, a tie goes to the smaller row
            double bv = -1.0;
            int bi = n;
            for (int j = k + tid; j < n; j += 32) {
                const double v = fabs(M[j * n + k]);
                if (v > bv) {
                    bv = v;
                    bi = j;
                }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const double ov = __shfl_xor_sync(0xffffffffu, bv, o);
                const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                if (ov > bv || (ov == bv && oi < bi)) {
                    bv = ov;
                    bi = oi;
                }
            }
            if (tid == 0) big_sh = bi < n ? bi : k;
        }
        __syncthreads();
        const int big = big_sh;
        if (big != k)
            for (int j = tid; j < n; j += nt) {
                const double t = M[k * n + j];
                M[k * n + j] = M[big * n + j];
                M[big * n + j] = t;
                const double u = X[k * n + j];
                X[k * n + j] = X[big * n + j];
                X[big * n + j] = u;
            }
        __syncthreads();
        const double p = M[k * n + k];
        if (!(fabs(p) >= 1e-10)) {
            if (tid == 0) *status = 1;
            return;
        }
        for (int i = k + 1 + tid; i < n; i += nt) M[i * n + k] = __ddiv_rn(M[i * n + k], p);
        __syncthreads();
        const int m = n - k - 1;
        for (int t = tid; t < m * m; t += nt) {
            const int i = k + 1 + t / m, j = k + 1 + t % m;
            M[i * n + j] = __dsub_rn(M[i * n + j], __dmul_rn(M[i * n + k], M[k * n + j]));
        }
        __syncthreads();
    }
    for (int k = 0; k < n; ++k) {
        const int m = n - k - 1;
        for (int t = tid; t < m * n; t += nt) {
            const int i = k + 1 + t / n, c = t % n;
            X[i * n + c] = __dsub_rn(X[i * n + c], __dmul_rn(M[i * n + k], X[k * n + c]));
        }
        __syncthreads();
    }
    // backward: one thread per column, each row's sum in increasing column
    // order as SolveLU (the columns are independent: no barrier)
    for (int c = tid; c < n; c += nt)
        for (int i = n - 1; i >= 0; --i) {
            double v = X[i * n + c];
            for (int k = i + 1; k < n; ++k) v = __dsub_rn(v, __dmul_rn(M[i * n + k], X[k * n + c]));
            X[i * n + c] = __ddiv_rn(v, M[i * n + i]);
        }
    if (tid == 0) *status = 0;
}

// ---------------------------------------------------------------- GmgT ---
template <class V>
struct GmgT : GmgBase {
    std::vector<GLevel<V>> lev;
    int base = 0, nu1 = 2, nu2 = 2, cycle = 1, smoother = 0, smoother2 = 0;
    int base_kind = UG4GB_BASE_LU, base_steps = 0;
    double damp = 1.0, damp2 = 1.0;
    DevBuf<double> Ainv;
    DevBuf<int> lu_status;       // device factorisation of the base: 1 = singular
    int *lu_host = nullptr;      // its page-locked copy, read after the next wait
    bool lu_pending = false;
    ~GmgT() override
    {
        if (lu_host) cudaFreeHost(lu_host);
    }
    void check_base() override
    {
        if (!lu_pending) return;
        lu_pending = false;
        UG_REQUIRE(*lu_host == 0, UG4GB_ERR_SINGULAR, "GMG base solver: LU pivot below 1e-10 (singular base matrix)");
    }
    DevBuf<double> z64;          // mixed precision: FP64 copy of the top correction
    uint64_t top_key = 0;        // pattern key of the top operator of the last set-up
    int nbase = 0;
    bool top_converted = false;  // this apply: the FP32 top defect is already in dA of the top level
    // the coarse end of the V-cycle in one launch (k_coarse.cu): levels
    // base .. coarse_top, or none (coarse_top < 0)
    int coarse_top = -1;
    size_t coarse_smem = 0;
    CoarsePlan<V> coarse_host{};
    DevBuf<CoarsePlan<V>> coarse_plan;

    int top() const override { return (int)lev.size() - 1; }
    bool is_fp32() const override { return sizeof(V) == 4; }
    void *sc_top() override { return lev.back().sc.p; }
    const Csr &P(int l) const override { return lev[l].P; }
    const Csr &R(int l) const override { return lev[l].R; }
    const Csr &levelA(int l) const override { return lev[l].A; }
    int base_level() const override { return base; }

    uint64_t signature() const override
    {
        uint64_t h = 1469598103934665603ULL;
        auto mix = [&](const void *p) {
            h ^= (uint64_t)(uintptr_t)p;
            h *= 1099511628211ULL;
        };
        for (const GLevel<V> &L : lev) {
            mix(L.At.dia.val.p); mix(L.At.sell.val.p); mix(L.At.sell.col.p); mix(L.At.sell.sptr.p);
            mix(L.At.sell.swidth.p); mix(L.dinv.p); mix(L.dfac.p); mix(L.sc.p); mix(L.dA.p); mix(L.dB.p);
            mix(L.w.p); mix(L.t.p); mix(L.y.p); mix(L.dinv2.p); mix(L.Ps.dia.val.p); mix(L.Ps.sell.val.p); mix(L.Rs.dia.val.p);
            mix(L.Rs.sell.val.p); mix(L.sweep2.get()); mix(L.vcolor.p);
            for (const DevBuf<int> &q : L.crow) mix(q.p);
            mix(L.ilu.val.p); mix(L.ilu.col.p); mix(L.ilu.rowptr.p); mix(L.ilu.nlow.p); mix(L.ilu.uinv.p);
            h ^= (uint64_t)L.n;
        }
        mix(Ainv.p);
        mix(z64.p);
        mix(coarse_plan.p);
        h ^= (uint64_t)(coarse_top + 2);
        h *= 1099511628211ULL;
        return h;
    }

    // reuse: the same structure as the previous set-up of this level (its
    // pattern, layout, colours): only values are refreshed, in place
    void setup_level(Ctx &c, GLevel<V> &L, const Level &G, int l, double damp, bool is_base, bool reuse)
    {
        int n = L.A.nrows;
        L.n = n;
        L.sc.alloc(n);
        L.dA.alloc(n);
        L.dB.alloc(n);
        if (is_base) return;
        if (!reuse) L.At_lay.known = false;
        L.w.alloc(n);
        L.dinv64.alloc(n);
        L.dfac64.alloc(n);
        L.dinv.alloc(n);
        L.dfac.alloc(n);
        UG_LAUNCH_PDL(c, k_diag_inv<V>, div_up(n, 256), 256, 0, L.A.rowptr.p, L.A.col.p, L.A.val.p, n, damp, smoother,
                  L.dinv64.p, L.dfac64.p, L.dinv.p, L.dfac.p);
        // a Gauss-Seidel post-smoother with its own relaxation
        if (smoother2 != UG4GB_SMOOTHER_JACOBI && smoother2 != UG4GB_SMOOTHER_ILU && damp2 != damp) {
            L.dinv2_64.alloc(n);
            L.dinv2.alloc(n);
            UG_LAUNCH_PDL(c, k_diag_inv<V>, div_up(n, 256), 256, 0, L.A.rowptr.p, L.A.col.p, L.A.val.p, n, damp2,
                      smoother2, L.dinv2_64.p, (double *)nullptr, L.dinv2.p, (V *)nullptr);
        }
        if (smoother == UG4GB_SMOOTHER_JACOBI) {
            op_from_csr_cached<V>(c, L.A, L.At, L.dinv64.p, c.allow_dia, L.At_lay);
        } else {
            op_from_csr_cached<V>(c, L.A, L.At, nullptr, c.allow_dia, L.At_lay);
            L.t.alloc(n);
            // colours with no coupling inside a colour: parity on structured
            // levels (valid for their stencils and for R A P of them); on
            // unstructured levels a greedy colouring of this operator's graph,
            // which a Galerkin operator may widen beyond the grid's elements
            const int *colour = G.structured ? G.color.p : L.vcolor.p;
            int ncol = G.ncolors;
            // a re-init on the same structure keeps the colours and row lists
            const bool have_colours = reuse && !L.crow.empty();
            if (!G.structured && !have_colours) {
                std::vector<int> rp(n + 1), ci((size_t)L.A.nnz), vc(n, -1), seen;
                copy_out(c, rp.data(), L.A.rowptr.p, sizeof(int) * (size_t)(n + 1));
                copy_out(c, ci.data(), L.A.col.p, sizeof(int) * (size_t)L.A.nnz);
                ncol = 0;
                for (int i = 0; i < n; ++i) {
                    seen.clear();
                    for (int a = rp[i]; a < rp[i + 1]; ++a)
                        if (ci[a] != i && vc[ci[a]] >= 0) seen.push_back(vc[ci[a]]);
                    std::sort(seen.begin(), seen.end());
                    int q = 0;
                    for (int x : seen) {
                        if (x == q) ++q;
                        else if (x > q) break;
                    }
                    vc[i] = q;
                    ncol = std::max(ncol, q + 1);
                }
                L.vcolor.alloc(n > 0 ? n : 1);
                copy_in(c, L.vcolor.p, vc.data(), sizeof(int) * (size_t)n);
                colour = L.vcolor.p;
            }
            if (!have_colours) {
            L.crow.resize(ncol);
            L.ncrow.assign(ncol, 0);
            DevBuf<int> flag, pos;
            flag.alloc(n + 1);
            pos.alloc(n + 1);
            for (int q = 0; q < ncol; ++q) {
                L.crow[q].alloc(n);
                UG_CUDA(cudaMemsetAsync(flag.p + n, 0, sizeof(int), c.stream));
                UG_LAUNCH(c, k_colour_flag, div_up(n, 256), 256, 0, colour, n, q, flag.p);
                int64_t cnt = 0;
                exclusive_scan_int(c, flag.p, pos.p, n + 1, &cnt);
                UG_LAUNCH(c, k_colour_scatter, div_up(n, 256), 256, 0, colour, n, q, pos.p, L.crow[q].p);
                L.ncrow[q] = (int)cnt;
            }
            UG_CUDA(cudaStreamSynchronize(c.stream));
            }
            if (smoother == UG4GB_SMOOTHER_ILU || smoother2 == UG4GB_SMOOTHER_ILU) {
                ilu_setup<V>(c, L.A, colour, L.crow, L.ncrow, L.ilu);
                L.y.alloc(n);
            }
        }
        (void)l;
    }

    // solve-format copy of a transfer matrix scaled by a damping factor (the
    // assembled P and R, which export returns, stay undamped as in ugcore)
    void damped_op(Ctx &c, const Csr &T, double damp, OpMat<V> &out)
    {
        if (damp == 1.0) {
            op_from_csr<V>(c, T, out, nullptr, false);
            return;
        }
        Csr S;
        csr_copy(c, T, S);
        if (S.nnz > 0)
            UG_LAUNCH(c, k_scale_vals, (unsigned)div_up(S.nnz, (int64_t)256), 256, 0, S.val.p, S.nnz, damp);
        op_from_csr<V>(c, S, out, nullptr, false);
        UG_CUDA(cudaStreamSynchronize(c.stream));
    }

    void setup_transfers(Ctx &c, GLevel<V> &F, const Level &Gf, const Level &Gc, double dprol, double dres)
    {
        Csr &P = F.P;
        P.nrows = Gf.nv;
        P.ncols = Gc.nv;
        DevBuf<int> len;
        len.alloc(Gf.nv + 1);
        UG_CUDA(cudaMemsetAsync(len.p, 0, len.bytes(), c.stream));
        UG_LAUNCH(c, k_build_P, div_up(Gf.nv, 256), 256, 0, Gf.npar.p, Gf.par.p, Gf.bnd.p, Gf.nv, len.p, (int *)nullptr,
                  (double *)nullptr, (const int *)nullptr, 0);
        P.rowptr.alloc(Gf.nv + 1);
        int64_t nnz = 0;
        exclusive_scan_int(c, len.p, P.rowptr.p, Gf.nv + 1, &nnz);
        P.nnz = nnz;
        P.col.alloc(nnz);
        P.val.alloc(nnz);
        UG_LAUNCH(c, k_build_P, div_up(Gf.nv, 256), 256, 0, Gf.npar.p, Gf.par.p, Gf.bnd.p, Gf.nv, (int *)nullptr, P.col.p,
                  P.val.p, (const int *)P.rowptr.p, 1);
        csr_transpose(c, P, F.R, true);
        UG_LAUNCH(c, k_adjust_R, div_up(Gf.nv, 256), 256, 0, Gf.npar.p, Gf.par.p, Gf.bnd.p, Gf.nv, F.R.rowptr.p,
                  F.R.col.p, F.R.val.p);
        damped_op(c, F.P, dprol, F.Ps);
        damped_op(c, F.R, dres, F.Rs);
        // the structured hierarchy's P and R need no stored matrix (AUTO
        // format); the assembled CSR stays for export and the SELL format
        F.grid_transfer = c.allow_dia && Gf.structured && Gc.structured;
        F.gp = GridPair{Gf.nx, Gf.ny, Gf.nz, Gc.nx, Gc.ny, Gc.nz, Gf.dim, Gf.elem_type == UG4GB_TET ? 1 : 0,
                        dprol, dres};
        UG_CUDA(cudaStreamSynchronize(c.stream));
    }

    void setup_base(Ctx &c)
    {
        if (base_kind != UG4GB_BASE_LU) return;   // the base level smooths (setup_level)
        const Csr &A = lev[base].A;
        int n = A.nrows;
        UG_REQUIRE(n <= 4096, UG4GB_ERR_INVALID, "GMG base level larger than 4096 unknowns (dense LU limit)");
        if (n <= kDeviceLuMax) {
            const size_t smem = (size_t)kDeviceLuMax * kDeviceLuMax * sizeof(double);
            UG_CUDA(cudaFuncSetAttribute(k_base_lu, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            Ainv.alloc((size_t)n * n);
            lu_status.alloc(1);
            UG_LAUNCH_PDL(c, k_base_lu, 1, kLuThreads, (size_t)n * n * sizeof(double), A.rowptr.p, A.col.p, A.val.p,
                      n, Ainv.p, lu_status.p);
            // no wait: the status is read back behind the factorisation and
            // checked after the next apply's or solve's own wait (check_base)
            if (!lu_host) UG_CUDA(cudaMallocHost((void **)&lu_host, sizeof(int)));
            UG_CUDA(cudaMemcpyAsync(lu_host, lu_status.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            lu_pending = true;
            nbase = n;
            return;
        }
        std::vector<int> rp(n + 1), ci(A.nnz);
        std::vector<double> va(A.nnz);
        copy_out(c, rp.data(), A.rowptr.p, sizeof(int) * (n + 1));
        copy_out(c, ci.data(), A.col.p, sizeof(int) * A.nnz);
        copy_out(c, va.data(), A.val.p, sizeof(double) * A.nnz);
        std::vector<double> M((size_t)n * n, 0.0), inv;
        for (int r = 0; r < n; ++r)
            for (int a = rp[r]; a < rp[r + 1]; ++a) M[(size_t)r * n + ci[a]] = va[a];
        dense_lu_inverse(n, M, inv);
        Ainv.alloc((size_t)n * n);
        copy_in(c, Ainv.p, inv.data(), sizeof(double) * inv.size());   // from pageable memory: staged on return
        nbase = n;
    }

    // Which coarse levels the one-block kernel cycles (Ctx::coarse_levels),
    // and its shared-memory layout (CoarsePlan).  Inside the one block every
    // phase is a chain of dependent FMAs on one SM; on GB300 an FP64 chain
    // issues at a small fraction of the FP32 rate, so the block only pays
    // where a phase is shorter than a separate launch (about 1.5 us).
    // Measured on GB300 (c0/c3 quads, c1 hexes, c2 Kuhn tets, c4 upwind
    // hexes): levels whose Jacobi sweep is at most about 4000 FP64 row-
    // operations, rows x (S + 3), an FP32 one counting a quarter, gain
    // (9-point 2D levels up to 17^2 in FP64 and 33^2 in FP32: 8-15% of a
    // solve); a base level of more than 32 rows loses (its dense solve, one
    // warp per row with a five-step warp sum, is FP64 bound on one SM).
    void setup_coarse(Ctx &c)
    {
        coarse_top = -1;
        coarse_smem = 0;
        if (c.coarse_levels == 0 || cycle != 1 || smoother != UG4GB_SMOOTHER_JACOBI ||
            smoother2 != UG4GB_SMOOTHER_JACOBI || base_kind != UG4GB_BASE_LU)
            return;
        constexpr double kSweepWork = 4000.0;
        constexpr int kBaseRows = 32;
        constexpr size_t kSmemMax = 216 * 1024;
        constexpr int kAlign = 16 / (int)sizeof(V);   // elements per 16 bytes
        auto up = [](size_t v, size_t a) { return (v + a - 1) / a * a; };
        if (c.coarse_levels < 0 && nbase > kBaseRows) return;
        CoarsePlan<V> &P = coarse_host;
        P = CoarsePlan<V>{};
        P.vbase = (int)up((size_t)(nbase + 1) * nbase * sizeof(double), 16);
        size_t e = up(2 * (size_t)lev[base].n, kAlign);   // level-precision elements so far
        P.lev[0].n = lev[base].n;
        P.lev[0].vofs = 0;
        int best = -1;
        size_t best_bytes = 0;
        const int last = std::min(top() - 1, base + kCoarseMaxLevels - 1);
        for (int l = base + 1; l <= last; ++l) {
            const GLevel<V> &L = lev[l];
            const GridPair &gp = L.gp;
            if (!L.grid_transfer || L.At.kind != 1 || L.At.nrows != L.n || L.At.ncols != L.n ||
                gp.nx * gp.ny * gp.nz != L.n || gp.cnx * gp.cny * gp.cnz != lev[l - 1].n ||
                !coarse_width_ok(L.At.dia.S) || L.At.dia.S != lev[base + 1].At.dia.S)
                break;
            const Dia<V> &D = L.At.dia;
            CoarseLevel<V> &Q = P.lev[l - base];
            Q.n = L.n;
            Q.val = D.vals();
            Q.dinv = L.dinv.p;
            Q.dfac = L.dfac.p;
            Q.ncols = D.ncols;
            Q.ld = D.ld;
            Q.S = D.S;
            for (int k = 0; k < D.S; ++k) Q.off[k] = D.off.o[k];
            Q.gp = gp;
            Q.aofs = (int)e;
            e = up(e + (size_t)D.S * D.ld, kAlign);
            Q.iofs = (int)e;
            e = up(e + (size_t)L.n, kAlign);
            Q.fofs = (int)e;
            e = up(e + (size_t)L.n, kAlign);
            Q.vofs = (int)e;
            e = up(e + 4 * (size_t)L.n, kAlign);
            const size_t bytes = (size_t)P.vbase + e * sizeof(V);
            if (bytes > kSmemMax) break;
            if (c.coarse_levels > 0) {
                if (l - base > c.coarse_levels) break;
            } else if ((double)L.n * (D.S + 3) * (sizeof(V) == 8 ? 1.0 : 0.25) > kSweepWork) {
                break;
            }
            best = l;
            best_bytes = bytes;
        }
        if (best < 0) return;
        P.m = best - base + 1;
        P.nu1 = nu1;
        P.nu2 = nu2;
        P.nbase = nbase;
        P.Ainv = Ainv.p;
        P.d_in = lev[best].dA.p;
        P.sc_out = lev[best].sc.p;
        coarse_smem = best_bytes;
        coarse_plan.alloc(1);
        copy_in(c, coarse_plan.p, &P, sizeof(P));   // from pageable memory: staged on return
        coarse_prepare<V>(kSmemMax);   // the most any multigrid asks for
        coarse_top = best;
    }

    // ------------------------------------------------------------ cycle --
    // level l; dtop = FP64 defect of the top level (r), first = first visit.
    // In mixed precision the top defect is converted to FP32 once, and the
    // last top-level kernel writes the correction back in FP64 (z64): every
    // float<->double conversion happens once per row, never per nonzero
    // (conversions issue on GB300's slow FP64 pipe).
    // ctype: this visit's cycle type (gamma >= 1, or -1 for the F-cycle:
    // the coarser level once as an F-cycle, then once as a V-cycle;
    // AssembledMultiGridCycle::lmgc, mg_solver_impl.hpp:2091-2134)
    void lmgc(Ctx &c, int l, int ctype, const double *dtop, bool first, const int *skip, const double *r_rho,
              RedArgs *red,
              int rho_kind, bool &rho_done)
    {
        const int T = top();
        GLevel<V> &L = lev[l];
        c.prof_tag = "L" + std::to_string(l);
        const V *top_in = nullptr;
        if (l == T) {
            if constexpr (sizeof(V) == sizeof(double)) {
                top_in = (const V *)dtop;
            } else {
                if (!top_converted) UG_LAUNCH_PDL(c, k_to_v<V>, div_up(L.n, 256), 256, 0, dtop, L.dA.p, L.n);
                top_in = L.dA.p;
            }
        }
        if (l == base) {
            // top == base: a single-level "cycle" is the base solve
            base_correct(c, L, top_in, skip);
            if (z64.p) copy_z<V>(c, L.n, L.sc.p, z64.p, skip);
            return;
        }
        GLevel<V> &C = lev[l - 1];
        const V *cur = (l == T) ? top_in : L.dcur;
        // ---- pre-smoothing
        if (nu1 == 0 && first) UG_LAUNCH_PDL(c, k_zero<V>, div_up(L.n, 256), 256, 0, L.n, L.sc.p, skip);
        for (int k = 0; k < nu1; ++k) {
            V *out = (cur == L.dA.p) ? L.dB.p : L.dA.p;
            int mode = (k == 0) ? (first ? SC_SET_FROM_BASE : SC_ADD_FROM_BASE) : SC_ADD_FROM_BASE;
            // two steps in one pass over the operator where the level allows it
            if (k + 1 < nu1 && L.sweep2 &&
                smooth_pair<V>(c, L.sweep2.get(), L.gp, cur, nullptr, L.dinv.p, L.sc.p, out, mode, SC_ADD_FROM_BASE,
                               skip, nullptr, nullptr, 0, nullptr)) {
                cur = out;
                ++k;
                continue;
            }
            if (smoother == UG4GB_SMOOTHER_JACOBI) {
                smooth_step<V, V, V>(c, L.At, cur, cur, L.dinv.p, L.sc.p, out, mode, skip, nullptr, nullptr, 0);
            } else {
                gs_sweep(c, L, cur, skip, smoother, L.dinv.p, damp);
                residual_update<V, V>(c, L.At, L.t.p, cur, out, L.sc.p, mode == SC_SET_FROM_BASE ? 1 : 0, skip);
            }
            cur = out;
        }
        const V *dpre = cur;
        // ---- restriction
        if (L.grid_transfer) restrict_grid<V>(c, L.gp, dpre, C.dA.p, skip);
        else restrict_apply<V>(c, L.Rs, dpre, C.dA.p, skip);
        C.dcur = C.dA.p;
        // ---- coarse correction
        if (l - 1 == base) {
            c.prof_tag = "L" + std::to_string(l - 1);
            base_correct(c, C, C.dA.p, skip);
        } else if (l - 1 == coarse_top) {
            // V-cycle below: the coarse end in one launch (setup_coarse)
            c.prof_tag = "L" + std::to_string(base) + "-" + std::to_string(l - 1);
            coarse_cycle<V>(c, coarse_plan.p, coarse_host.lev[1].S, coarse_smem, skip);
        } else {
            const int visits = (ctype == -1) ? 2 : ctype;
            for (int i = 0; i < visits; ++i) {
                bool rd = false;
                const int sub = (ctype == -1) ? (i == 0 ? -1 : 1) : ctype;
                lmgc(c, l - 1, sub, nullptr, i == 0, skip, nullptr, nullptr, 0, rd);
            }
        }
        c.prof_tag = "L" + std::to_string(l);
        // ---- prolongation + post-smoothing
        if (L.grid_transfer) prolong_grid<V>(c, L.gp, C.sc.p, L.sc.p, L.dfac.p, nu2 > 0 ? L.w.p : (V *)nullptr, skip);
        else prolong_apply<V>(c, L.Ps, C.sc.p, L.sc.p, L.dfac.p, nu2 > 0 ? L.w.p : (V *)nullptr, skip);
        const V *dbase = dpre;
        bool z_written = false;
        if (smoother2 == UG4GB_SMOOTHER_JACOBI) {
            for (int k = 0; k < nu2; ++k) {
                const V *x = (k == 0) ? L.w.p : dbase;
                // two steps in one pass where the level allows it
                if (k + 1 < nu2 && L.sweep2) {
                    bool need_out = (k + 1 < nu2 - 1) || (l != T && cycle != 1);
                    V *out = need_out ? ((dbase == L.dA.p) ? L.dB.p : L.dA.p) : nullptr;
                    bool last_top = (l == T && k + 1 == nu2 - 1);
                    if (smooth_pair<V>(c, L.sweep2.get(), L.gp, x, k == 0 ? dbase : nullptr, L.dinv.p, L.sc.p, out,
                                       SC_ADD_FROM_NEW, SC_ADD_FROM_NEW, skip, last_top ? r_rho : nullptr,
                                       last_top ? red : nullptr, rho_kind, last_top ? z64.p : nullptr)) {
                        if (last_top) {
                            rho_done = (r_rho != nullptr);
                            z_written = true;
                        }
                        if (out) dbase = out;
                        ++k;
                        continue;
                    }
                }
                // a level below the top is visited again (W, gamma > 2, F cycles):
                // its last defect is the next visit's start
                bool need_out = (k < nu2 - 1) || (l != T && cycle != 1);
                V *out = need_out ? ((dbase == L.dA.p) ? L.dB.p : L.dA.p) : nullptr;
                bool last_top = (l == T && k == nu2 - 1);
                smooth_step<V, V, V>(c, L.At, x, dbase, L.dinv.p, L.sc.p, out, SC_ADD_FROM_NEW, skip,
                                     last_top ? r_rho : nullptr, last_top ? red : nullptr, rho_kind,
                                     last_top ? z64.p : nullptr);
                if (last_top) {
                    rho_done = (r_rho != nullptr);
                    z_written = true;
                }
                if (out) dbase = out;
            }
        } else {
            for (int k = 0; k < nu2; ++k) {
                const V *tprev = (k == 0) ? L.w.p : L.t.p;
                V *out = (dbase == L.dA.p) ? L.dB.p : L.dA.p;
                residual_update<V, V>(c, L.At, tprev, dbase, out, L.sc.p, k == 0 ? 2 : 0, skip);
                gs_sweep(c, L, out, skip, smoother2, L.dinv2.p ? L.dinv2.p : L.dinv.p, damp2);
                dbase = out;
            }
            if (nu2 > 0) UG_LAUNCH_PDL(c, k_vadd<V>, div_up(L.n, 256), 256, 0, L.n, L.sc.p, L.t.p, skip);
        }
        if (l == T && z64.p && !z_written) copy_z<V>(c, L.n, L.sc.p, z64.p, skip);
        L.dcur = const_cast<V *>(dbase);
    }

    // sc = base solver applied to the base level defect d: the dense LU, or
    // base_steps steps of the pre-smoother from sc = 0 (c += B d, d -= A B d;
    // the defect buffers of the level take the updated defects)
    void base_correct(Ctx &c, GLevel<V> &L, const V *d, const int *skip)
    {
        if (base_kind == UG4GB_BASE_LU) {
            base_solve<V>(c, Ainv.p, nbase, d, L.sc.p, skip);
            return;
        }
        const V *cur = d;
        for (int k = 0; k < base_steps; ++k) {
            V *out = (cur == L.dA.p) ? L.dB.p : L.dA.p;
            const int mode = (k == 0) ? SC_SET_FROM_BASE : SC_ADD_FROM_BASE;
            if (smoother == UG4GB_SMOOTHER_JACOBI) {
                smooth_step<V, V, V>(c, L.At, cur, cur, L.dinv.p, L.sc.p, out, mode, skip, nullptr, nullptr, 0);
            } else {
                gs_sweep(c, L, cur, skip, smoother, L.dinv.p, damp);
                residual_update<V, V>(c, L.At, L.t.p, cur, out, L.sc.p, mode == SC_SET_FROM_BASE ? 1 : 0, skip);
            }
            cur = out;
        }
    }

    // t = B d of smoother `kind` (dinv = relax/a_ii; ILU: damp scales the
    // correction): colours in increasing order from t = 0; the symmetric
    // smoother then sweeps the colours in decreasing order, the backward one
    // only in decreasing order
    void gs_sweep(Ctx &c, GLevel<V> &L, const V *dv, const int *skip, int kind, const V *dinv, double dmp)
    {
        if (kind == UG4GB_SMOOTHER_ILU) {
            ilu_apply<V>(c, L.ilu, L.crow, L.ncrow, dv, L.y.p, L.t.p, dmp, skip);
            return;
        }
        UG_LAUNCH_PDL(c, k_zero<V>, div_up(L.n, 256), 256, 0, L.n, L.t.p, skip);
        if (kind != UG4GB_SMOOTHER_MCBGS)
            for (size_t q = 0; q < L.crow.size(); ++q)
                if (L.ncrow[q] > 0) mcgs_colour<V>(c, L.At, L.crow[q].p, L.ncrow[q], dinv, dv, L.t.p, skip);
        if (kind == UG4GB_SMOOTHER_MCSGS || kind == UG4GB_SMOOTHER_MCBGS)
            for (size_t q = L.crow.size(); q-- > 0;)
                if (L.ncrow[q] > 0) mcgs_colour<V>(c, L.At, L.crow[q].p, L.ncrow[q], dinv, dv, L.t.p, skip);
        // SymmetricGaussSeidel (sgs_step, core_smoothers.h:189-206) is
        // (D/w + U)^{-1} D (D/w + L)^{-1}; the backward sweep above, which
        // updates the forward result by w/a_ii times the defect, gives
        // (2/w - 1) times that: with relaxation the result is rescaled
        if (kind == UG4GB_SMOOTHER_MCSGS && dmp != 1.0)
            UG_LAUNCH_PDL(c, k_vscale<V>, div_up(L.n, 256), 256, 0, L.n, L.t.p, (V)(dmp / (2.0 - dmp)), skip);
    }

    const double *apply(Ctx &c, const double *dtop, const int *skip, const double *r_rho, RedArgs *red,
                        int rho_kind, bool &rho_done, bool top_ready) override
    {
        rho_done = false;
        top_converted = top_ready && sizeof(V) == 4;
        lmgc(c, top(), cycle, dtop, true, skip, r_rho, red, rho_kind, rho_done);
        return z64.p ? z64.p : (const double *)lev.back().sc.p;
    }
    float *top_defect_buffer() override
    {
        if constexpr (sizeof(V) == 4) return (float *)lev.back().dA.p;
        return nullptr;
    }
};

// reuse: the multigrid of the previous init with the same hierarchy and
// structural settings (ug4gb_gmg_init checks): its level buffers and its
// transfers P, R (which depend on the grid only) are kept; the operators,
// smoother data and base factorisation are rebuilt.
template <class V>
static GmgBase *build_gmg(ug4gb_gmg *m, const ug4gb_matrix *A_top, GmgT<V> *reuse = nullptr)
{
    Ctx &c = m->ctx->c;
    const ug4gb_grid *g = m->disc->g;
    int nl = (int)g->lev.size();
    auto *G = reuse ? reuse : new GmgT<V>;
    std::unique_ptr<GmgT<V>> guard(G);
    const bool keep_transfers = reuse != nullptr;
    G->base = m->base;
    G->nu1 = m->nu1;
    G->nu2 = m->nu2;
    G->cycle = m->cycle;
    G->smoother = m->smoother;
    G->damp = m->damp;
    G->smoother2 = m->smoother2;
    G->damp2 = m->damp2;
    G->base_kind = m->base_kind;
    G->base_steps = m->base_steps;
    UG_REQUIRE((m->smoother == UG4GB_SMOOTHER_JACOBI) == (m->smoother2 == UG4GB_SMOOTHER_JACOBI) &&
                   (m->smoother != UG4GB_SMOOTHER_JACOBI || m->damp == m->damp2),
               UG4GB_ERR_INVALID,
               "GMG: a Jacobi smoother combines only with the same Jacobi smoother (it works on the column-scaled "
               "level operator); pre- and post-smoothers of the Gauss-Seidel kinds and ILU combine freely");
    G->lev.resize(nl);
    UG_REQUIRE(m->base >= 0 && m->base < nl, UG4GB_ERR_INVALID, "GMG: base level out of range");
    UG_REQUIRE(A_top->A.nrows == g->lev[nl - 1].nv, UG4GB_ERR_INVALID, "GMG: top operator size != top level");
    // transposed multigrid: A of the level = A^T with Dirichlet rows reset to
    // identity.  The level patterns (element cliques, and R A P of them) are
    // symmetric, so A^T has A's pattern and its values are swapped pairwise
    // in place (no second copy of the level); a non-symmetric pattern (a
    // user's top operator) is transposed explicitly
    auto transpose_level = [&](int l, bool same_pattern) {
        GLevel<V> &L = G->lev[l];
        if (!same_pattern || L.sym < 0) L.sym = csr_pattern_symmetric(c, L.A) ? 1 : 0;
        if (L.sym == 1) {
            csr_transpose_symmetric_inplace(c, L.A);
        } else {
            Csr T;
            csr_transpose(c, L.A, T, true);
            L.A = std::move(T);
        }
        UG_LAUNCH_PDL(c, k_dirichlet_identity, div_up(L.A.nrows, 256), 256, 0, g->lev[l].bnd.p, L.A.nrows, L.A.rowptr.p,
                  L.A.col.p, L.A.val.p);
    };
    if (!m->rap) {
        for (int l = m->base; l < nl; ++l) {
            GLevel<V> &L = G->lev[l];
            // the level's pattern is the one of the previous set-up (the top
            // level: the same assembled operator pattern as then)
            const bool same = keep_transfers && L.asm_ok &&
                              (l != nl - 1 || (A_top->pattern_key() && A_top->pattern_key() == G->top_key));
            Csr &dst = L.A;
            // level operator: copy of the surface operator on the top level,
            // re-assembled on coarser levels (assemble_level_operator, :528-750)
            if (l == nl - 1) {
                csr_copy(c, A_top->A, dst);
            } else {
                // re-assembled into the level's kept storage: the element
                // pattern is built once per multigrid
                ug4gb_matrix tmp;
                tmp.ctx = m->ctx;
                tmp.A = std::move(dst);
                if (same) {
                    tmp.pattern_grid = g->uid;
                    tmp.pattern_level = l;
                }
                // with a time discretisation: the jacobian M + sa0 A of its
                // current step (MultiStepTimeDiscretization::assemble_jacobian,
                // theta_time_step_impl.h:123-140)
                TimeScale ts{};
                if (m->td) ts = m->td->jacobian_scale();
                disc_assemble(m->disc, l, &tmp, nullptr, m->td ? &ts : nullptr);
                dst = std::move(tmp.A);
            }
            if (m->transposed) transpose_level(l, same);
            L.asm_ok = true;
            G->setup_level(c, L, g->lev[l], l, m->damp, l == m->base && m->base_kind == UG4GB_BASE_LU, same);
            if (l > m->base) {
                if (!keep_transfers) G->setup_transfers(c, L, g->lev[l], g->lev[l - 1], m->damp_prol, m->damp_res);
                if (L.grid_transfer && m->smoother == UG4GB_SMOOTHER_JACOBI)
                    L.sweep2 = sweep2_prepare<V>(c, L.At, L.gp);
            }
        }
    } else {
        // Galerkin coarse operators (init_rap_operator, :830-1012): the top
        // level's operator, then from the top down the transfers of a level
        // and R A P of it as the operator of the level below
        csr_copy(c, A_top->A, G->lev[nl - 1].A);
        if (m->transposed) transpose_level(nl - 1, false);
        for (int l = nl - 1; l > m->base; --l) {
            if (!keep_transfers) G->setup_transfers(c, G->lev[l], g->lev[l], g->lev[l - 1], m->damp_prol, m->damp_res);
            csr_rap(c, G->lev[l].R, G->lev[l].A, G->lev[l].P, G->lev[l - 1].A);
        }
        for (int l = m->base; l < nl; ++l) {
            GLevel<V> &L = G->lev[l];
            G->setup_level(c, L, g->lev[l], l, m->damp, l == m->base && m->base_kind == UG4GB_BASE_LU, false);
            if (l > m->base && L.grid_transfer && m->smoother == UG4GB_SMOOTHER_JACOBI)
                L.sweep2 = sweep2_prepare<V>(c, L.At, L.gp);
        }
    }
    G->setup_base(c);
    G->setup_coarse(c);
    if (sizeof(V) != sizeof(double)) G->z64.alloc(g->lev[nl - 1].nv);
    G->top_key = A_top->pattern_key();
    return guard.release();
}

}  // namespace ug4gb

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

static void drop_graph(ug4gb_gmg *m)
{
    if (m->graph) cudaGraphExecDestroy(m->graph);
    m->graph = nullptr;
    m->graph_d = nullptr;
    m->graph_c = nullptr;
}

extern "C" {

int ug4gb_gmg_create(ug4gb_ctx *ctx, ug4gb_disc *disc, ug4gb_gmg **out)
{
    if (!ctx || !disc || !out) return UG4GB_ERR_INVALID;
    ug4gb_gmg *m = new ug4gb_gmg;
    m->ctx = ctx;
    m->disc = disc;
    ug4gb_ctx_retain(ctx);
    *out = m;
    return UG4GB_OK;
}

static bool smoother_ok(int kind, double damp)
{
    // the symmetric sweep is an SSOR step: its factor lies in (0, 2)
    if (kind == UG4GB_SMOOTHER_MCSGS && !(damp < 2.0)) return false;
    return kind >= UG4GB_SMOOTHER_JACOBI && kind <= UG4GB_SMOOTHER_MCBGS && damp > 0.0 && std::isfinite(damp);
}

int ug4gb_gmg_set_smoother(ug4gb_gmg *m, int kind, double damp)
{
    if (!m || !smoother_ok(kind, damp)) return UG4GB_ERR_INVALID;
    m->smoother = m->smoother2 = kind;
    m->damp = m->damp2 = damp;
    return UG4GB_OK;
}

int ug4gb_gmg_set_base_solver(ug4gb_gmg *m, int kind, int steps)
{
    if (!m || (kind != UG4GB_BASE_LU && kind != UG4GB_BASE_SMOOTHER)) return UG4GB_ERR_INVALID;
    if (kind == UG4GB_BASE_SMOOTHER && (steps < 1 || steps > 1000)) return UG4GB_ERR_INVALID;
    m->base_kind = kind;
    m->base_steps = kind == UG4GB_BASE_SMOOTHER ? steps : 0;
    return UG4GB_OK;
}

int ug4gb_gmg_set_presmoother(ug4gb_gmg *m, int kind, double damp)
{
    if (!m || !smoother_ok(kind, damp)) return UG4GB_ERR_INVALID;
    m->smoother = kind;
    m->damp = damp;
    return UG4GB_OK;
}

int ug4gb_gmg_set_postsmoother(ug4gb_gmg *m, int kind, double damp)
{
    if (!m || !smoother_ok(kind, damp)) return UG4GB_ERR_INVALID;
    m->smoother2 = kind;
    m->damp2 = damp;
    return UG4GB_OK;
}

int ug4gb_gmg_set_cycle_type(ug4gb_gmg *m, int cycle)
{
    if (!m || !(cycle == -1 || (cycle >= 1 && cycle <= 4))) return UG4GB_ERR_INVALID;
    m->cycle = cycle;
    return UG4GB_OK;
}

int ug4gb_gmg_set_num_presmooth(ug4gb_gmg *m, int n)
{
    if (!m || n < 0 || n > 16) return UG4GB_ERR_INVALID;
    m->nu1 = n;
    return UG4GB_OK;
}

int ug4gb_gmg_set_num_postsmooth(ug4gb_gmg *m, int n)
{
    if (!m || n < 0 || n > 16) return UG4GB_ERR_INVALID;
    m->nu2 = n;
    return UG4GB_OK;
}

int ug4gb_gmg_set_base_level(ug4gb_gmg *m, int level)
{
    if (!m || level < 0) return UG4GB_ERR_INVALID;
    m->base = level;
    return UG4GB_OK;
}

int ug4gb_gmg_set_precision(ug4gb_gmg *m, int precision)
{
    if (!m || (precision != UG4GB_PREC_FP64 && precision != UG4GB_PREC_MIXED)) return UG4GB_ERR_INVALID;
    m->precision = precision;
    return UG4GB_OK;
}

int ug4gb_gmg_set_rap(ug4gb_gmg *m, int rap)
{
    if (!m) return UG4GB_ERR_INVALID;
    m->rap = rap ? 1 : 0;
    return UG4GB_OK;
}

int ug4gb_gmg_set_time_disc(ug4gb_gmg *m, ug4gb_timedisc *td)
{
    if (!m) return UG4GB_ERR_INVALID;
    if (td && td->disc != m->disc) {
        m->ctx->c.err = "set_time_disc: the time discretisation belongs to another discretisation";
        return UG4GB_ERR_INVALID;
    }
    m->td = td;
    return UG4GB_OK;
}

int ug4gb_gmg_set_prolongation_damping(ug4gb_gmg *m, double damp)
{
    if (!m || !(damp > 0.0) || !std::isfinite(damp)) return UG4GB_ERR_INVALID;
    m->damp_prol = damp;
    return UG4GB_OK;
}

int ug4gb_gmg_set_restriction_damping(ug4gb_gmg *m, double damp)
{
    if (!m || !(damp > 0.0) || !std::isfinite(damp)) return UG4GB_ERR_INVALID;
    m->damp_res = damp;
    return UG4GB_OK;
}

int ug4gb_gmg_set_transposed(ug4gb_gmg *m, int transposed)
{
    if (!m) return UG4GB_ERR_INVALID;
    m->transposed = transposed ? 1 : 0;
    return UG4GB_OK;
}

int ug4gb_gmg_init(ug4gb_gmg *m, const ug4gb_matrix *A_top)
{
    ug4gb::NvtxRange nvtx_("ug4gb:gmg_init");
    if (!m || !A_top) return UG4GB_ERR_INVALID;
    // what the cycle's launch sequence depends on besides the buffers
    const uint64_t settings = ((uint64_t)(m->cycle + 8) << 40) ^ ((uint64_t)m->nu1 << 20) ^ (uint64_t)m->nu2;
    bool keep_graphs = false;
    const int rc = guarded(m->ctx, [&] {
        // a re-init with the same hierarchy and structure (typically a new
        // operator every Newton, time or optimisation step) keeps the level
        // buffers and the transfers and refreshes the values in place
        // (the transposition is applied to the values in place: a flip between
        // the forward and the transposed cycle keeps the structure)
        const GmgKey key{m->disc->g->uid, (int)m->disc->g->lev.size(), m->base, m->smoother, m->damp, m->rap,
                         0, m->precision, m->ctx->c.allow_dia ? 1 : 0, m->damp_prol, m->damp_res, m->smoother2,
                         m->damp2, m->base_kind, m->base_steps};
        const bool reuse = m->impl && m->built == key;
        const uint64_t before = reuse ? (m->impl->signature() ^ m->built_settings) : 0;
        GmgBase *old = reuse ? m->impl.release() : nullptr;
        m->impl.reset();
        m->built = GmgKey{};
        if (m->precision == UG4GB_PREC_FP64)
            m->impl.reset(build_gmg<double>(m, A_top, static_cast<GmgT<double> *>(old)));
        else
            m->impl.reset(build_gmg<float>(m, A_top, static_cast<GmgT<float> *>(old)));
        m->built = key;
        m->built_settings = settings;
        m->n_top = A_top->A.nrows;
        // the same device buffers and launch sequence: the captured graphs
        // (this multigrid's and its solvers') replay the refreshed values
        keep_graphs = reuse && before == (m->impl->signature() ^ settings);
    });
    if (!keep_graphs) {
        drop_graph(m);
        m->gen++;
    }
    return rc;
}

int ug4gb_gmg_apply(ug4gb_gmg *m, ug4gb_vector *cvec, const ug4gb_vector *d)
{
    ug4gb::NvtxRange nvtx_("ug4gb:gmg_apply");
    if (!m || !cvec || !d) return UG4GB_ERR_INVALID;
    if (!m->impl) {
        m->ctx->c.err = "ug4gb_gmg_apply: init() not called";
        return UG4GB_ERR_STATE;
    }
    if (cvec->n != m->n_top || d->n != m->n_top) return UG4GB_ERR_INVALID;
    return guarded(m->ctx, [&] {
        Ctx &c = m->ctx->c;
        if (c.profiling) {
            bool rd = false;
            const double *z = m->impl->apply(c, d->d, nullptr, nullptr, nullptr, 0, rd);
            copy_z<double>(c, m->n_top, z, cvec->d, nullptr);
            UG_CUDA(cudaStreamSynchronize(c.stream));
            m->impl->check_base();
            check_device_error(c);
            return;
        }
        if (!m->graph || m->graph_d != d->d || m->graph_c != cvec->d) {
            drop_graph(m);
            cudaGraph_t gr;
            int64_t before = c.launches;
            UG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
            try {
                bool rd = false;
                const double *z = m->impl->apply(c, d->d, nullptr, nullptr, nullptr, 0, rd);
                copy_z<double>(c, m->n_top, z, cvec->d, nullptr);
            } catch (...) {
                cudaStreamEndCapture(c.stream, &gr);
                throw;
            }
            UG_CUDA(cudaStreamEndCapture(c.stream, &gr));
            m->graph_kernels = c.launches - before;
            c.launches = before;
            UG_CUDA(cudaGraphInstantiate(&m->graph, gr, 0));
            cudaGraphDestroy(gr);
            m->graph_d = d->d;
            m->graph_c = cvec->d;
        }
        UG_CUDA(cudaGraphLaunch(m->graph, c.stream));
        c.launches += m->graph_kernels;
        UG_CUDA(cudaStreamSynchronize(c.stream));
        m->impl->check_base();
        check_device_error(c);
    });
}

int ug4gb_gmg_transfer_info(const ug4gb_gmg *m, int level, int which, int *nrows, int *ncols, int64_t *nnz)
{
    if (!m || !m->impl || level <= m->base || level > m->impl->top()) return UG4GB_ERR_INVALID;
    const Csr &A = which ? m->impl->R(level) : m->impl->P(level);
    if (nrows) *nrows = A.nrows;
    if (ncols) *ncols = A.ncols;
    if (nnz) *nnz = A.nnz;
    return UG4GB_OK;
}

int ug4gb_gmg_export_transfer(const ug4gb_gmg *m, int level, int which, int *rowptr, int *col, double *val)
{
    if (!m || !m->impl || level <= m->base || level > m->impl->top()) return UG4GB_ERR_INVALID;
    return guarded(m->ctx, [&] {
        Ctx &c = m->ctx->c;
        const Csr &A = which ? m->impl->R(level) : m->impl->P(level);
        if (rowptr) copy_out(c, rowptr, A.rowptr.p, sizeof(int) * (size_t)(A.nrows + 1));
        if (col) copy_out(c, col, A.col.p, sizeof(int) * (size_t)A.nnz);
        if (val) copy_out(c, val, A.val.p, sizeof(double) * (size_t)A.nnz);
    });
}

int ug4gb_gmg_level_info(const ug4gb_gmg *m, int level, int *nrows, int64_t *nnz)
{
    if (!m || !m->impl || level < m->impl->base_level() || level > m->impl->top()) return UG4GB_ERR_INVALID;
    const Csr &A = m->impl->levelA(level);
    if (nrows) *nrows = A.nrows;
    if (nnz) *nnz = A.nnz;
    return UG4GB_OK;
}

int ug4gb_gmg_export_level(const ug4gb_gmg *m, int level, int *rowptr, int *col, double *val)
{
    if (!m || !m->impl || level < m->impl->base_level() || level > m->impl->top()) return UG4GB_ERR_INVALID;
    return guarded(m->ctx, [&] {
        Ctx &c = m->ctx->c;
        const Csr &A = m->impl->levelA(level);
        if (rowptr) copy_out(c, rowptr, A.rowptr.p, sizeof(int) * (size_t)(A.nrows + 1));
        if (col) copy_out(c, col, A.col.p, sizeof(int) * (size_t)A.nnz);
        if (val) copy_out(c, val, A.val.p, sizeof(double) * (size_t)A.nnz);
    });
}

void ug4gb_gmg_destroy(ug4gb_gmg *m)
{
    if (!m) return;
    ug4gb_ctx *ctx = m->ctx;
    cudaStreamSynchronize(ctx->c.stream);
    drop_graph(m);
    delete m;
    ug4gb_ctx_release(ctx);
}

}  // extern "C"

// k_solve.cu -- SpMV-based multigrid and Krylov kernels (SELL-32 or diagonal).
//
// Every kernel is HBM-bound: one thread per row, matrix values streamed with
// evict-first loads (coalesced 32-wide), the gathered vector kept in L1/L2.
// Two operator layouts share the kernels through a "matrix view":
//   SELL-32   general sparsity: 32-row slices, column-major in the slice;
//   diagonal  <= 27 constant offsets (structured levels): values only, the
//             column of entry k is row + off[k]; no column stream and no
//             load that depends on another load.
// Row-local vector work is fused into the SpMV epilogue so each sweep reads
// the operator once:
//   Jacobi step     t = dinv*d ; d -= A t ; sc += t
//                   (Jacobi::step, lib_algebra/operator/preconditioner/
//                    jacobi.h:222; AssembledMultiGridCycle::
//                    presmooth_and_restriction / prolongation_and_postsmooth,
//                    mg_solver_impl.hpp:1687-1966) becomes one pass over the
//                   column-scaled operator At = A*diag(dinv): d_new = d - At x.
//   prolongation    t = P sc_c ; sc += t ; w = t / dinv (so that A t = At w)
//                   (StdTransfer::prolongate, std_transfer_impl.h:721)
//   restriction     d_c = R d (StdTransfer::do_restrict, std_transfer_impl.h:776)
//   CG              q = A z + beta q, p = z + beta p and lambda = (q,p) in one
//                   pass (CG::apply_return_defect, cg.h:163-226)
// Reductions are deterministic (grid_reduce: fixed-order tree per block,
// block partials summed in block order by the last block).
#include "k_solve.cuh"

namespace ug4gb {

constexpr int NT = 256;

int row_grid(const Ctx &c, int nrows)
{
    int need = (int)div_up(nrows > 0 ? nrows : 1, NT);
    int cap = c.num_sms * 8;
    return need < cap ? need : cap;
}

// widening to FP64 of a level-precision value (identity for FP64)
__device__ __forceinline__ double f32_to_f64_t(double v) { return v; }
__device__ __forceinline__ double f32_to_f64_t(float v) { return f32_to_f64(v); }

// ------------------------------------------------------------ views ------
template <class V>
struct SellMV {
    static constexpr int kCache = 8;   // entries of a row loaded ahead (the rest after the wait)
    SellView<V> s;
    struct Cache {
        int base, w;
        int col[kCache];
        V val[kCache];
    };
    __device__ __forceinline__ int rows() const { return s.nrows; }
    __device__ __forceinline__ void prefetch(int row, Cache &c) const
    {
        const int sl = row >> 5, lane = row & 31;
        c.base = __ldg(s.sptr + sl) + lane;
        c.w = __ldg(s.swidth + sl);
#pragma unroll
        for (int k = 0; k < kCache; ++k) {
            if (k < c.w) {
                c.col[k] = __ldg(s.col + c.base + k * kSliceH);
                c.val[k] = __ldg(s.val + c.base + k * kSliceH);
            }
        }
    }
    // dot with a prefetched row; same order of operations as dot
    template <class ACC, class XT>
    __device__ __forceinline__ ACC dot_cached(const XT *__restrict__ x, int, const Cache &c) const
    {
        ACC acc = (ACC)0;
#pragma unroll
        for (int k = 0; k < kCache; ++k)
            if (k < c.w) acc += (ACC)c.val[k] * (ACC)x[c.col[k]];
        for (int k = kCache; k < c.w; ++k) {
            const int idx = c.base + k * kSliceH;
            acc += (ACC)ld_stream(s.val + idx) * (ACC)x[ld_stream(s.col + idx)];
        }
        return acc;
    }
    template <class ACC, class XT>
    __device__ __forceinline__ ACC dot(const XT *__restrict__ x, int row) const
    {
        const int sl = row >> 5, lane = row & 31;
        const int base = __ldg(s.sptr + sl) + lane;
        const int w = __ldg(s.swidth + sl);
        ACC acc = (ACC)0;
#pragma unroll 4
        for (int k = 0; k < w; ++k) {
            const int idx = base + k * kSliceH;
            acc += (ACC)ld_stream(s.val + idx) * (ACC)x[ld_stream(s.col + idx)];
        }
        return acc;
    }
};

template <class V, int S>
struct DiaMV {
    static constexpr int kS = S;
    int n, ncols, ld;
    const V *__restrict__ val;
    Offs off;
    struct Cache {
        V a[S];
    };
    __device__ __forceinline__ int rows() const { return n; }
    __device__ __forceinline__ void prefetch(int i, Cache &c) const
    {
#pragma unroll
        for (int k = 0; k < S; ++k) c.a[k] = ld_stream(val + (size_t)k * ld + i);
    }
    template <class ACC, class XT>
    __device__ __forceinline__ ACC dot_cached(const XT *__restrict__ x, int i, const Cache &c) const
    {
        ACC acc = (ACC)0;
#pragma unroll
        for (int k = 0; k < S; ++k) {
            int j = i + off.o[k];
            j = j < 0 ? 0 : (j >= ncols ? ncols - 1 : j);
            acc = fma_rn((ACC)c.a[k], (ACC)x[j], acc);
        }
        return acc;
    }
    template <class ACC, class XT>
    __device__ __forceinline__ ACC dot(const XT *__restrict__ x, int i) const
    {
        ACC acc = (ACC)0;
#pragma unroll
        for (int k = 0; k < S; ++k) {
            int j = i + off.o[k];
            j = j < 0 ? 0 : (j >= ncols ? ncols - 1 : j);
            acc = fma_rn((ACC)ld_stream(val + (size_t)k * ld + i), (ACC)x[j], acc);
        }
        return acc;
    }
    // W consecutive rows i0..i0+W-1 (i0 % W == 0, all < n): one 16-byte
    // value load per diagonal instead of W scalar ones
    template <int W, class XT>
    __device__ __forceinline__ void dot_w(const XT *__restrict__ x, int i0, V (&acc)[W]) const
    {
#pragma unroll
        for (int e = 0; e < W; ++e) acc[e] = (V)0;
        // diagonals in three batches: S/3 packs in flight per thread keeps
        // the register count low enough for a full SM
        constexpr int B = S / 3;
        static_assert(B * 3 == S, "S must be a multiple of 3");
#pragma unroll 1
        for (int kb = 0; kb < S; kb += B) {
            Pack<V, W> a[B];
#pragma unroll
            for (int k = 0; k < B; ++k) a[k] = ld_stream_pack<V, W>(val + (size_t)(kb + k) * ld + i0);
#pragma unroll
            for (int k = 0; k < B; ++k) {
                const int j = i0 + off.o[kb + k];
#pragma unroll
                for (int e = 0; e < W; ++e) {
                    int jj = j + e;
                    jj = jj < 0 ? 0 : (jj >= ncols ? ncols - 1 : jj);
                    acc[e] = fma_rn(a[k].v[e], (V)x[jj], acc[e]);
                }
            }
        }
    }
};

// calls f(view) with the view type matching the operator's layout
template <class V, class F>
void with_mv(const OpMat<V> &m, F &&f)
{
    if (m.kind == 0) {
        f(SellMV<V>{view(m.sell)});
        return;
    }
    const Dia<V> &d = m.dia;
    switch (d.S) {
    case 9: f(DiaMV<V, 9>{d.nrows, d.ncols, d.ld, d.vals(), d.off}); break;
    case 15: f(DiaMV<V, 15>{d.nrows, d.ncols, d.ld, d.vals(), d.off}); break;
    case 27: f(DiaMV<V, 27>{d.nrows, d.ncols, d.ld, d.vals(), d.off}); break;
    default: throw Error{UG4GB_ERR_INVALID, "diagonal operator with unsupported width"};
    }
}

__device__ __forceinline__ bool conv_valid(double v)
{
    if (v == 0.0) return true;
    return v >= 2.2250738585072014e-308 && v <= 1.7976931348623157e308 && v == v && v >= 0.0;
}

__device__ __forceinline__ bool conv_ended(const KScal *ks)
{
    if (!conv_valid(ks->dcur)) return true;
    if (ks->step >= ks->maxit) return true;
    if (ks->dcur < ks->min_def) return true;
    if (ks->dcur / ks->d0 < ks->rel_red) return true;
    return false;
}

__device__ __forceinline__ void conv_update(KScal *ks, double d, int done_value)
{
    ks->dcur = d;
    ks->step += 1;
    if (ks->hist && ks->step < ks->hist_cap) ks->hist[ks->step] = d;
    if (conv_ended(ks)) ks->done = done_value;
}

// ------------------------------------------------------- smoothing step --
// PF (levels of at most one wave of rows, where latency rules): this
// thread's first row of the operator and its Jacobi factor are loaded
// before waiting for the predecessor (no solve kernel writes them).  Large
// levels skip it: the cached row would cost registers, hence occupancy.
template <class MV, class V, class XT, class DT, bool RHO, bool PF>
__global__ void __launch_bounds__(NT) k_smooth(MV A, const XT *__restrict__ x, const DT *__restrict__ dbase,
                                               const V *__restrict__ dinv, V *__restrict__ sc, V *__restrict__ dout,
                                               int sc_mode, const int *skip, const double *__restrict__ r_rho,
                                               RedArgs red, int rho_kind, double *__restrict__ z64)
{
    const int stride = gridDim.x * NT, n = A.rows(), row0 = blockIdx.x * NT + threadIdx.x;
    typename MV::Cache cache;
    V dinv0 = (V)0;
    if constexpr (PF) {
        pdl_trigger();
        if (row0 < n) {
            A.prefetch(row0, cache);
            dinv0 = dinv[row0];
        }
        pdl_wait();
    } else {
        PDL_ENTRY();
    }
    if (skip && *skip) return;
    double rsum = 0.0;
    for (int row = row0; row < n; row += stride) {
        const bool first = PF && (row == row0);
        V acc = first ? A.template dot_cached<V>(x, row, cache) : A.template dot<V>(x, row);
        V db = (V)dbase[row];
        V s;
        V dn = jacobi_row<V>(acc, db, first ? dinv0 : dinv[row], sc_mode,
                             sc_mode == SC_SET_FROM_BASE ? (V)0 : sc[row], s);
        if (dout) dout[row] = dn;
        sc[row] = s;
        if (RHO || z64) {
            const double s64 = f32_to_f64_t(s);   // one conversion per row, only where needed
            if (z64) z64[row] = s64;
            if (RHO) rsum += s64 * r_rho[row];
        }
    }
    if (RHO) {
        double v[1] = {rsum};
        KScal *ks = red.ks;
        grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) {
            if (rho_kind == 0) {
                ks->rho_old = tot[0];
            } else {
                ks->rho = tot[0];
                ks->beta = tot[0] / ks->rho_old;
                ks->rho_old = tot[0];
            }
        });
    }
}

// The same step on the diagonal layout with W = 16/sizeof(V) consecutive rows
// per thread: every value and row-vector access is one 16-byte load or
// store (the gathered x stays scalar).  A tail of n % W rows is done by the
// thread that owns the last, partial group.  Per row the arithmetic is that
// of k_smooth.  32 registers (8 blocks of 256 threads per SM): the sweep is
// bound by memory latency, and the extra resident warps gave 2-4% per sweep.
template <class V, int S, bool RHO>
__global__ void __launch_bounds__(NT, 8) k_smooth_dia(DiaMV<V, S> A, const V *__restrict__ x, const V *__restrict__ dbase,
                                                   const V *__restrict__ dinv, V *__restrict__ sc, V *__restrict__ dout,
                                                   int sc_mode, const int *skip, const double *__restrict__ r_rho,
                                                   RedArgs red, int rho_kind, double *__restrict__ z64)
{
    constexpr int W = 16 / sizeof(V);
    PDL_ENTRY();
    if (skip && *skip) return;
    double rsum = 0.0;
    const int n = A.rows(), ng = (n + W - 1) / W, stride = gridDim.x * NT;
    const bool wide64 = (((uintptr_t)z64 | (uintptr_t)r_rho) & 15u) == 0;
    for (int g = blockIdx.x * NT + threadIdx.x; g < ng; g += stride) {
        const int r0 = g * W;
        if (r0 + W <= n) {
            V acc[W];
            A.template dot_w<W>(x, r0, acc);
            Pack<V, W> db = ld_pack<V, W>(dbase + r0), di = ld_pack<V, W>(dinv + r0), s, dn;
            if (sc_mode != SC_SET_FROM_BASE) s = ld_pack<V, W>(sc + r0);
#pragma unroll
            for (int e = 0; e < W; ++e)
                dn.v[e] = jacobi_row<V>(acc[e], db.v[e], di.v[e], sc_mode,
                                        sc_mode == SC_SET_FROM_BASE ? (V)0 : s.v[e], s.v[e]);
            if (dout) st_pack<V, W>(dout + r0, dn);
            st_pack<V, W>(sc + r0, s);
            if (RHO || z64) {
                double s64[W];
#pragma unroll
                for (int e = 0; e < W; ++e) s64[e] = f32_to_f64_t(s.v[e]);
                if constexpr (W % 2 == 0) {
                    // FP64 side in 16-byte pairs when both arrays allow it
                    if (wide64) {
#pragma unroll
                        for (int e = 0; e < W; e += 2) {
                            if (z64) st_pack<double, 2>(z64 + r0 + e, Pack<double, 2>{{s64[e], s64[e + 1]}});
                            if (RHO) {
                                Pack<double, 2> rr = ld_pack<double, 2>(r_rho + r0 + e);
                                rsum += s64[e] * rr.v[0];
                                rsum += s64[e + 1] * rr.v[1];
                            }
                        }
                        continue;
                    }
                }
#pragma unroll
                for (int e = 0; e < W; ++e) {
                    if (z64) z64[r0 + e] = s64[e];
                    if (RHO) rsum += s64[e] * r_rho[r0 + e];
                }
            }
        } else {
            for (int row = r0; row < n; ++row) {
                V acc = A.template dot<V>(x, row);
                V s;
                V dn = jacobi_row<V>(acc, dbase[row], dinv[row], sc_mode,
                                     sc_mode == SC_SET_FROM_BASE ? (V)0 : sc[row], s);
                if (dout) dout[row] = dn;
                sc[row] = s;
                if (RHO || z64) {
                    const double s64 = f32_to_f64_t(s);
                    if (z64) z64[row] = s64;
                    if (RHO) rsum += s64 * r_rho[row];
                }
            }
        }
    }
    if (RHO) {
        double v[1] = {rsum};
        KScal *ks = red.ks;
        grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) {
            if (rho_kind == 0) {
                ks->rho_old = tot[0];
            } else {
                ks->rho = tot[0];
                ks->beta = tot[0] / ks->rho_old;
                ks->rho_old = tot[0];
            }
        });
    }
}

template <class MV>
struct is_dia : std::false_type {};
template <class V, int S>
struct is_dia<DiaMV<V, S>> : std::true_type {};

inline bool aligned16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

template <class V, class XT, class DT>
void smooth_step(Ctx &c, const OpMat<V> &At, const XT *x, const DT *dbase, const V *dinv, V *sc, V *dout, int sc_mode,
                 const int *skip, const double *r_rho, RedArgs *red, int rho_kind, double *z64)
{
    const int g = row_grid(c, At.nrows);
    with_mv(At, [&](auto mv) {
        using MV = decltype(mv);
        if constexpr (is_dia<MV>::value && std::is_same<XT, V>::value && std::is_same<DT, V>::value) {
            // FP32 levels of at least three full waves of one-row threads:
            // there the wider loads pay (8-9% per sweep on GB300).  FP64 sweeps
            // are bound by the FP64 FMA rate and smaller levels by latency;
            // there the one-row-per-thread kernel is as fast or faster.
            const bool wide = sizeof(V) == 4 && At.nrows >= c.num_sms * 2048 * 3;
            if (wide && aligned16(dbase) && aligned16(dinv) && aligned16(sc) && aligned16(dout)) {
                constexpr int W = 16 / sizeof(V);
                const int groups = (At.nrows + W - 1) / W;
                int gv = (int)div_up(groups > 0 ? groups : 1, NT);
                if (gv > kRedMaxBlocks) gv = kRedMaxBlocks;
                if (r_rho) {
                    // with the fused (z, r) reduction: one resident wave of blocks
                    // (8 per SM), so the blocks' reduction tails overlap and the
                    // last block sums fewer partials (-12% on the 129^3 tet level)
                    const int gr = gv < c.num_sms * 8 ? gv : c.num_sms * 8;
                    UG_LAUNCH_PDL(c, (k_smooth_dia<V, MV::kS, true>), gr, NT, 0, mv, x, dbase, dinv, sc, dout, sc_mode,
                                  skip, r_rho, *red, rho_kind, z64);
                } else {
                    RedArgs none{nullptr, nullptr, nullptr};
                    UG_LAUNCH_PDL(c, (k_smooth_dia<V, MV::kS, false>), gv, NT, 0, mv, x, dbase, dinv, sc, dout,
                                  sc_mode, skip, (const double *)nullptr, none, 0, z64);
                }
                return;
            }
        }
        const bool pf = At.nrows <= c.num_sms * NT;
        RedArgs none{nullptr, nullptr, nullptr};
        if (r_rho && pf) {
            UG_LAUNCH_PDL(c, (k_smooth<MV, V, XT, DT, true, true>), g, NT, 0, mv, x, dbase, dinv, sc, dout, sc_mode,
                          skip, r_rho, *red, rho_kind, z64);
        } else if (r_rho) {
            UG_LAUNCH_PDL(c, (k_smooth<MV, V, XT, DT, true, false>), g, NT, 0, mv, x, dbase, dinv, sc, dout, sc_mode,
                          skip, r_rho, *red, rho_kind, z64);
        } else if (pf) {
            UG_LAUNCH_PDL(c, (k_smooth<MV, V, XT, DT, false, true>), g, NT, 0, mv, x, dbase, dinv, sc, dout, sc_mode,
                          skip, (const double *)nullptr, none, 0, z64);
        } else {
            UG_LAUNCH_PDL(c, (k_smooth<MV, V, XT, DT, false, false>), g, NT, 0, mv, x, dbase, dinv, sc, dout, sc_mode,
                          skip, (const double *)nullptr, none, 0, z64);
        }
    });
}

#define INST_SMOOTH(V, XT, DT)                                                                              \
    template void smooth_step<V, XT, DT>(Ctx &, const OpMat<V> &, const XT *, const DT *, const V *, V *, V *, int, \
                                         const int *, const double *, RedArgs *, int, double *);
INST_SMOOTH(double, double, double)
INST_SMOOTH(float, float, float)

// --------------------------------------------------------- transfers -----
template <class MV, class V, bool PF>
__global__ void __launch_bounds__(NT) k_restrict(MV R, const V *__restrict__ d, V *__restrict__ dc, const int *skip)
{
    const int stride = gridDim.x * NT, n = R.rows(), row0 = blockIdx.x * NT + threadIdx.x;
    typename MV::Cache cache;
    if constexpr (PF) {
        pdl_trigger();
        if (row0 < n) R.prefetch(row0, cache);
        pdl_wait();
    } else {
        PDL_ENTRY();
    }
    if (skip && *skip) return;
    for (int row = row0; row < n; row += stride)
        dc[row] = (PF && row == row0) ? R.template dot_cached<V>(d, row, cache) : R.template dot<V>(d, row);
}

template <class V>
void restrict_apply(Ctx &c, const OpMat<V> &R, const V *d, V *dc, const int *skip)
{
    with_mv(R, [&](auto mv) {
        if (R.nrows <= c.num_sms * NT)
            UG_LAUNCH_PDL(c, (k_restrict<decltype(mv), V, true>), row_grid(c, R.nrows), NT, 0, mv, d, dc, skip);
        else
            UG_LAUNCH_PDL(c, (k_restrict<decltype(mv), V, false>), row_grid(c, R.nrows), NT, 0, mv, d, dc, skip);
    });
}

template <class MV, class V, bool PF>
__global__ void __launch_bounds__(NT) k_prolong(MV P, const V *__restrict__ scc, V *__restrict__ sc,
                                                const V *__restrict__ dfac, V *__restrict__ w, const int *skip)
{
    const int stride = gridDim.x * NT, n = P.rows(), row0 = blockIdx.x * NT + threadIdx.x;
    typename MV::Cache cache;
    V dfac0 = (V)0;
    if constexpr (PF) {
        pdl_trigger();
        if (row0 < n) {
            P.prefetch(row0, cache);
            if (w) dfac0 = dfac[row0];
        }
        pdl_wait();
    } else {
        PDL_ENTRY();
    }
    if (skip && *skip) return;
    for (int row = row0; row < n; row += stride) {
        const bool first = PF && (row == row0);
        V t = first ? P.template dot_cached<V>(scc, row, cache) : P.template dot<V>(scc, row);
        sc[row] += t;
        if (w) w[row] = t * (first ? dfac0 : dfac[row]);
    }
}

template <class V>
void prolong_apply(Ctx &c, const OpMat<V> &P, const V *scc, V *sc, const V *dfac, V *w, const int *skip)
{
    with_mv(P, [&](auto mv) {
        if (P.nrows <= c.num_sms * NT)
            UG_LAUNCH_PDL(c, (k_prolong<decltype(mv), V, true>), row_grid(c, P.nrows), NT, 0, mv, scc, sc, dfac, w,
                          skip);
        else
            UG_LAUNCH_PDL(c, (k_prolong<decltype(mv), V, false>), row_grid(c, P.nrows), NT, 0, mv, scc, sc, dfac, w,
                          skip);
    });
}

// ------------------------------------------- grid-index transfers ---------

// The transfer kernels run in one of two thread layouts.  TILED: a 2D grid
// of 32 x 8 vertex tiles of the (x, y) plane, each thread walking z with the
// grid's z stride, so that a thread knows its grid indices without integer
// divisions by runtime extents (FP32 levels: +15% on the 129^3 prolongation).
// Else one vertex per thread of a 1D grid-stride loop, every lane busy:
// FP64 levels are bound by the FP64 issue rate, where a partly filled warp
// costs as much as a full one.
// t = P scc for fine vertex (i, j, k); sc += t; w = t * dfac (k_prolong on the assembled P)
template <class V>
__device__ __forceinline__ void prolong_row(const GridPair &g, const V *__restrict__ scc, V *__restrict__ sc,
                                            const V *__restrict__ dfac, V *__restrict__ w, int i, int j, int k)
{
    const int f = i + g.nx * (j + g.ny * k);
    V t = prolong_value<V>(g, scc, i, j, k);
    if (g.dprol != 1.0) t = mul_rn(t, (V)g.dprol);
    sc[f] = add_rn(sc[f], t);
    if (w) w[f] = mul_rn(t, dfac[f]);
}

template <class V, bool TILED>
__global__ void __launch_bounds__(NT) k_prolong_grid(GridPair g, const V *__restrict__ scc, V *__restrict__ sc,
                                                     const V *__restrict__ dfac, V *__restrict__ w, const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    if constexpr (TILED) {
        const int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 8 + threadIdx.y;
        if (i >= g.nx || j >= g.ny) return;
        for (int k = blockIdx.z; k < g.nz; k += gridDim.z) prolong_row<V>(g, scc, sc, dfac, w, i, j, k);
    } else {
        const int n = g.nx * g.ny * g.nz, stride = gridDim.x * NT;
        for (int f = blockIdx.x * NT + threadIdx.x; f < n; f += stride)
            prolong_row<V>(g, scc, sc, dfac, w, f % g.nx, (f / g.nx) % g.ny, f / (g.nx * g.ny));
    }
}

template <class V, bool TILED>
__global__ void __launch_bounds__(NT) k_restrict_grid(GridPair g, const V *__restrict__ d, V *__restrict__ dc,
                                                      const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    if constexpr (TILED) {
        const int I = blockIdx.x * 32 + threadIdx.x, J = blockIdx.y * 8 + threadIdx.y;
        if (I >= g.cnx || J >= g.cny) return;
        for (int K = blockIdx.z; K < g.cnz; K += gridDim.z) restrict_row<V>(g, d, dc, I, J, K);
    } else {
        const int n = g.cnx * g.cny * g.cnz, stride = gridDim.x * NT;
        for (int c = blockIdx.x * NT + threadIdx.x; c < n; c += stride)
            restrict_row<V>(g, d, dc, c % g.cnx, (c / g.cnx) % g.cny, c / (g.cnx * g.cny));
    }
}

// grid of 32 x 8 tiles over (x, y) and enough z slices for about four
// resident waves of blocks
static dim3 transfer_grid(const Ctx &c, int nx, int ny, int nz)
{
    const unsigned gx = div_up(nx, 32), gy = div_up(ny, 8);
    int gz = (int)((size_t)c.num_sms * 8 * 4 / ((size_t)gx * gy));
    gz = gz < 1 ? 1 : (gz > nz ? nz : gz);
    return dim3(gx, gy, (unsigned)gz);
}

template <class V>
void prolong_grid(Ctx &c, const GridPair &g, const V *scc, V *sc, const V *dfac, V *w, const int *skip)
{
    if constexpr (sizeof(V) == 4)
        UG_LAUNCH_PDL(c, (k_prolong_grid<V, true>), transfer_grid(c, g.nx, g.ny, g.nz), dim3(32, 8), 0, g, scc, sc,
                      dfac, w, skip);
    else
        UG_LAUNCH_PDL(c, (k_prolong_grid<V, false>), row_grid(c, g.nx * g.ny * g.nz), NT, 0, g, scc, sc, dfac, w,
                      skip);
}

template <class V>
void restrict_grid(Ctx &c, const GridPair &g, const V *d, V *dc, const int *skip)
{
    if constexpr (sizeof(V) == 4)
        UG_LAUNCH_PDL(c, (k_restrict_grid<V, true>), transfer_grid(c, g.cnx, g.cny, g.cnz), dim3(32, 8), 0, g, d, dc,
                      skip);
    else
        UG_LAUNCH_PDL(c, (k_restrict_grid<V, false>), row_grid(c, g.cnx * g.cny * g.cnz), NT, 0, g, d, dc, skip);
}
template void prolong_grid<double>(Ctx &, const GridPair &, const double *, double *, const double *, double *,
                                   const int *);
template void prolong_grid<float>(Ctx &, const GridPair &, const float *, float *, const float *, float *,
                                  const int *);
template void restrict_grid<double>(Ctx &, const GridPair &, const double *, double *, const int *);
template void restrict_grid<float>(Ctx &, const GridPair &, const float *, float *, const int *);

// dense base solve with the LU-factored inverse, FP64: one warp per row of
// Ainv, eight rows per block.  Each lane's first entries of its row are read
// before the launch wait (Ainv is set up once), the defect is staged in
// shared memory, and the row sum is a fixed-order warp reduction of the
// lanes' explicitly fused partial sums (the fused coarse cycle, k_coarse.cu,
// repeats them).
constexpr int kBaseRowsPerBlock = NT / 32;
constexpr int kBasePre = 8;   // entries per lane read before the wait (rows up to 256 wide)

template <class V>
__global__ void __launch_bounds__(NT) k_base_solve(const double *__restrict__ Ainv, int n, const V *__restrict__ d,
                                                   V *__restrict__ sc, const int *skip)
{
    extern __shared__ double dsh[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int row = blockIdx.x * kBaseRowsPerBlock + warp;
    const double *arow = Ainv + (size_t)(row < n ? row : 0) * n;
    double a[kBasePre];
#pragma unroll
    for (int t = 0; t < kBasePre; ++t) {
        const int j = lane + 32 * t;
        a[t] = (row < n && j < n) ? __ldg(arow + j) : 0.0;
    }
    pdl_trigger();
    pdl_wait();
    if (skip && *skip) return;
    for (int j = threadIdx.x; j < n; j += blockDim.x) dsh[j] = (double)d[j];
    __syncthreads();
    if (row >= n) return;
    double s = 0.0;
#pragma unroll
    for (int t = 0; t < kBasePre; ++t) {
        const int j = lane + 32 * t;
        if (j < n) s = fma_rn(a[t], dsh[j], s);
    }
    for (int j = lane + 32 * kBasePre; j < n; j += 32) s = fma_rn(__ldg(arow + j), dsh[j], s);
    s = warp_sum(s);
    if (lane == 0) sc[row] = (V)s;
}

template <class V>
void base_solve(Ctx &c, const double *Ainv, int n, const V *d, V *sc, const int *skip)
{
    UG_LAUNCH_PDL(c, k_base_solve<V>, div_up(n, kBaseRowsPerBlock), NT, (size_t)n * sizeof(double), Ainv, n, d, sc,
                  skip);
}

// multicolour Gauss-Seidel: rows of one colour, t_i = relax (d_i - (A t)_i) / a_ii
// (t_i is still 0 when its colour is processed)
template <class MV, class V>
__global__ void __launch_bounds__(NT) k_mcgs(MV A, const int *__restrict__ rows, int nrows_c,
                                             const V *__restrict__ dr, const V *__restrict__ d, V *__restrict__ t,
                                             const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    const int stride = gridDim.x * NT;
    for (int q = blockIdx.x * NT + threadIdx.x; q < nrows_c; q += stride) {
        int row = rows[q];
        V acc = A.template dot<V>(t, row);
        // t_i += w/a_ii (d_i - (A t)_i): the forward sweep starts from t = 0,
        // the backward sweep of the symmetric smoother updates its result
        t[row] = t[row] + dr[row] * (d[row] - acc);
    }
}

template <class V>
void mcgs_colour(Ctx &c, const OpMat<V> &A, const int *rows, int nrows_c, const V *dinv_relax, const V *d, V *t,
                 const int *skip)
{
    with_mv(A, [&](auto mv) {
        UG_LAUNCH_PDL(c, (k_mcgs<decltype(mv), V>), row_grid(c, nrows_c), NT, 0, mv, rows, nrows_c, dinv_relax, d, t,
                  skip);
    });
}

template <class MV, class V, class DT>
__global__ void __launch_bounds__(NT) k_resupd(MV A, const V *__restrict__ t, const DT *__restrict__ dbase,
                                               V *__restrict__ dout, V *__restrict__ sc, int sc_mode, const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    const int stride = gridDim.x * NT, n = A.rows();
    for (int row = blockIdx.x * NT + threadIdx.x; row < n; row += stride) {
        V acc = A.template dot<V>(t, row);
        dout[row] = (V)dbase[row] - acc;
        if (sc_mode == 1) sc[row] = t[row];
        else if (sc_mode == 0) sc[row] += t[row];
    }
}

template <class V, class DT>
void residual_update(Ctx &c, const OpMat<V> &A, const V *t, const DT *dbase, V *dout, V *sc, int sc_mode,
                     const int *skip)
{
    with_mv(A, [&](auto mv) {
        UG_LAUNCH_PDL(c, (k_resupd<decltype(mv), V, DT>), row_grid(c, A.nrows), NT, 0, mv, t, dbase, dout, sc, sc_mode,
                  skip);
    });
}

template void restrict_apply<double>(Ctx &, const OpMat<double> &, const double *, double *, const int *);
template void restrict_apply<float>(Ctx &, const OpMat<float> &, const float *, float *, const int *);
template void prolong_apply<double>(Ctx &, const OpMat<double> &, const double *, double *, const double *, double *,
                                    const int *);
template void prolong_apply<float>(Ctx &, const OpMat<float> &, const float *, float *, const float *, float *,
                                   const int *);
template void base_solve<double>(Ctx &, const double *, int, const double *, double *, const int *);
template void base_solve<float>(Ctx &, const double *, int, const float *, float *, const int *);
template void mcgs_colour<double>(Ctx &, const OpMat<double> &, const int *, int, const double *, const double *,
                                  double *, const int *);
template void mcgs_colour<float>(Ctx &, const OpMat<float> &, const int *, int, const float *, const float *, float *,
                                 const int *);
template void residual_update<double, double>(Ctx &, const OpMat<double> &, const double *, const double *, double *,
                                              double *, int, const int *);
template void residual_update<float, float>(Ctx &, const OpMat<float> &, const float *, const float *, float *,
                                            float *, int, const int *);
template void residual_update<float, double>(Ctx &, const OpMat<float> &, const float *, const double *, float *,
                                             float *, int, const int *);

// ------------------------------------------------------------ Krylov -----
// r = b - A x (r holds b on entry); start the convergence check with |r|
template <class MV>
__global__ void __launch_bounds__(NT) k_krylov_start(MV A, const double *__restrict__ x, double *__restrict__ r,
                                                     float *__restrict__ r32, RedArgs red)
{
    PDL_ENTRY();
    double sum = 0.0;
    const int stride = gridDim.x * NT, n = A.rows();
    for (int row = blockIdx.x * NT + threadIdx.x; row < n; row += stride) {
        double ax = A.template dot<double>(x, row);
        double rv = r[row] - ax;
        r[row] = rv;
        if (r32) r32[row] = f64_to_f32(rv);
        sum += rv * rv;
    }
    double v[1] = {sum};
    KScal *ks = red.ks;
    grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) {
        double d = sqrt(tot[0]);
        ks->d0 = d;
        ks->dcur = d;
        ks->step = 0;
        ks->done = 0;
        ks->fail = 0;
        ks->restart = 1;
        if (ks->hist && ks->hist_cap > 0) ks->hist[0] = d;
        if (conv_ended(ks)) ks->done = 1;
    });
}

void krylov_start(Ctx &c, const OpMat<double> &A, const double *x, double *r, RedArgs red, float *r32)
{
    with_mv(A, [&](auto mv) {
        UG_LAUNCH_PDL(c, k_krylov_start<decltype(mv)>, row_grid(c, A.nrows), NT, 0, mv, x, r, r32, red);
    });
}

// first: p = z, q = A z ; else p = z + beta p, q = A z + beta q ; lambda = (q,p)
template <class MV, class ZT>
__global__ void __launch_bounds__(NT) k_cg_spmv_dot(MV A, const ZT *__restrict__ z, double *__restrict__ p,
                                                    double *__restrict__ q, int first, RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    const double beta = first ? 0.0 : ks->beta;
    double sum = 0.0;
    const int stride = gridDim.x * NT, n = A.rows();
    for (int row = blockIdx.x * NT + threadIdx.x; row < n; row += stride) {
        double az = A.template dot<double>(z, row);
        double pn = first ? (double)z[row] : (double)z[row] + beta * p[row];
        double qn = first ? az : az + beta * q[row];
        p[row] = pn;
        q[row] = qn;
        sum += qn * pn;
    }
    double v[1] = {sum};
    grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) {
        ks->lambda = tot[0];
        if (tot[0] == 0.0) {
            ks->fail = 1;
            ks->done = 1;
        }
        ks->alpha = ks->rho_old / tot[0];
    });
}

template <class ZT>
void cg_spmv_dot_t(Ctx &c, const OpMat<double> &A, const ZT *z, double *p, double *q, int first, RedArgs red)
{
    with_mv(A, [&](auto mv) {
        UG_LAUNCH_PDL(c, (k_cg_spmv_dot<decltype(mv), ZT>), row_grid(c, A.nrows), NT, 0, mv, z, p, q, first, red);
    });
}
template void cg_spmv_dot_t<double>(Ctx &, const OpMat<double> &, const double *, double *, double *, int, RedArgs);
template void cg_spmv_dot_t<float>(Ctx &, const OpMat<double> &, const float *, double *, double *, int, RedArgs);

// x += alpha p ; r -= alpha q ; |r| -> convergence check; optionally
// r32 = (float) r, the FP32 defect the mixed-precision multigrid starts from.
// Two entries per thread with 16-byte accesses (all pointers 16-byte
// aligned; the odd last entry alone).
__global__ void __launch_bounds__(NT) k_cg_update(int n, double *__restrict__ x, double *__restrict__ r,
                                                  const double *__restrict__ p, const double *__restrict__ q,
                                                  float *__restrict__ r32, RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    const double alpha = ks->alpha;
    double sum = 0.0;
    const int stride = gridDim.x * NT, npair = (n + 1) / 2;
    for (int k = blockIdx.x * NT + threadIdx.x; k < npair; k += stride) {
        const int i = 2 * k;
        if (i + 1 < n) {
            Pack<double, 2> xv = ld_pack<double, 2>(x + i), pv = ld_pack<double, 2>(p + i);
            Pack<double, 2> rv = ld_pack<double, 2>(r + i), qv = ld_pack<double, 2>(q + i);
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                xv.v[e] = xv.v[e] + alpha * pv.v[e];
                rv.v[e] = rv.v[e] + (-alpha) * qv.v[e];
                sum += rv.v[e] * rv.v[e];
            }
            st_pack<double, 2>(x + i, xv);
            st_pack<double, 2>(r + i, rv);
            if (r32) {
                float2 f = make_float2(f64_to_f32(rv.v[0]), f64_to_f32(rv.v[1]));
                *reinterpret_cast<float2 *>(r32 + i) = f;
            }
        } else {
            x[i] = x[i] + alpha * p[i];
            double rv = r[i] + (-alpha) * q[i];
            r[i] = rv;
            sum += rv * rv;
            if (r32) r32[i] = f64_to_f32(rv);
        }
    }
    double v[1] = {sum};
    grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) { conv_update(ks, sqrt(tot[0]), 1); });
}

// the same one entry per thread (pointers not 16-byte aligned)
__global__ void __launch_bounds__(NT) k_cg_update1(int n, double *__restrict__ x, double *__restrict__ r,
                                                   const double *__restrict__ p, const double *__restrict__ q,
                                                   float *__restrict__ r32, RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    const double alpha = ks->alpha;
    double sum = 0.0;
    const int stride = gridDim.x * NT;
    for (int i = blockIdx.x * NT + threadIdx.x; i < n; i += stride) {
        x[i] = x[i] + alpha * p[i];
        double rv = r[i] + (-alpha) * q[i];
        r[i] = rv;
        sum += rv * rv;
        if (r32) r32[i] = f64_to_f32(rv);
    }
    double v[1] = {sum};
    grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) { conv_update(ks, sqrt(tot[0]), 1); });
}

static inline bool al16(const void *p) { return ((uintptr_t)p & 15u) == 0; }

void cg_update(Ctx &c, int n, double *x, double *r, const double *p, const double *q, RedArgs red, float *r32)
{
    if (al16(x) && al16(r) && al16(p) && al16(q) && (!r32 || ((uintptr_t)r32 & 7u) == 0))
        UG_LAUNCH_PDL(c, k_cg_update, row_grid(c, (n + 1) / 2), NT, 0, n, x, r, p, q, r32, red);
    else
        UG_LAUNCH_PDL(c, k_cg_update1, row_grid(c, n), NT, 0, n, x, r, p, q, r32, red);
}

// rho = (z, r) when the preconditioner could not fuse it (kind 0: first, 1: loop)
template <class ZT>
__global__ void __launch_bounds__(NT) k_rho(int n, const ZT *__restrict__ z, const double *__restrict__ r, int kind,
                                            RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    double sum = 0.0;
    const int stride = gridDim.x * NT;
    for (int i = blockIdx.x * NT + threadIdx.x; i < n; i += stride) sum += (double)z[i] * r[i];
    double v[1] = {sum};
    grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) {
        if (kind == 0) {
            ks->rho_old = tot[0];
        } else {
            ks->rho = tot[0];
            ks->beta = tot[0] / ks->rho_old;
            ks->rho_old = tot[0];
        }
    });
}

template <class ZT>
void rho_dot(Ctx &c, int n, const ZT *z, const double *r, int kind, RedArgs red)
{
    UG_LAUNCH_PDL(c, k_rho<ZT>, row_grid(c, n), NT, 0, n, z, r, kind, red);
}
template void rho_dot<double>(Ctx &, int, const double *, const double *, int, RedArgs);
template void rho_dot<float>(Ctx &, int, const float *, const double *, int, RedArgs);

template <class ZT>
__global__ void k_copy_z(int n, const ZT *__restrict__ z, double *__restrict__ out, const int *skip)
{
    PDL_ENTRY();
    if (skip && *skip) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = f32_to_f64_t(z[i]);
}

template <class ZT>
void copy_z(Ctx &c, int n, const ZT *z, double *out, const int *skip)
{
    UG_LAUNCH_PDL(c, k_copy_z<ZT>, div_up(n, NT), NT, 0, n, z, out, skip);
}
template void copy_z<double>(Ctx &, int, const double *, double *, const int *);
template void copy_z<float>(Ctx &, int, const float *, double *, const int *);

// ------------------------------------------------------------ BiCGStab ---
// (BiCGStab::apply_return_defect, bicgstab.h:158-390).  A restart at the top
// of an iteration comes from the previous iteration's orthogonality test
// (ks->restart) or from the fixed restart period (step % num_restarts == 0,
// bicgstab.h:161-170; the check counts half steps).
__device__ __forceinline__ bool bicg_restarting(const KScal *ks)
{
    return ks->restart || (ks->num_restarts > 0 && ks->step % ks->num_restarts == 0);
}

__global__ void k_bicg_restart(int n, const double *__restrict__ r, double *__restrict__ r0, double *__restrict__ p,
                               double *__restrict__ v, KScal *ks)
{
    PDL_ENTRY();
    if (ks->done || !bicg_restarting(ks)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        r0[i] = r[i];
        p[i] = 0.0;
        v[i] = 0.0;
    }
}

void bicg_restart(Ctx &c, int n, const double *r, double *r0, double *p, double *v, RedArgs red)
{
    UG_LAUNCH_PDL(c, k_bicg_restart, div_up(n, NT), NT, 0, n, r, r0, p, v, red.ks);
}

__global__ void __launch_bounds__(NT) k_bicg_rho(int n, const double *__restrict__ r0, const double *__restrict__ r,
                                                 RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    double sum = 0.0;
    const int stride = gridDim.x * NT;
    for (int i = blockIdx.x * NT + threadIdx.x; i < n; i += stride) sum += r0[i] * r[i];
    double v[1] = {sum};
    grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) {
        if (bicg_restarting(ks)) {
            ks->alpha = 0.0;
            ks->omega = 1.0;
            ks->rho = 1.0;
            ks->norm_r0 = ks->dcur;
            ks->restart = 0;
        }
        const double rho_old = ks->rho;
        ks->rho_old = rho_old;
        ks->rho = tot[0];
        // restart in the next iteration when (r, r0) <= minOrtho |r| |r0|
        // (bicgstab.h:206-215)
        if (fabs(tot[0]) / (ks->dcur * ks->norm_r0) <= ks->min_ortho) ks->restart = 1;
        if (rho_old == 0.0) {
            ks->fail = 1;
            ks->done = 1;
        }
        ks->beta = (tot[0] / rho_old) * (ks->alpha / ks->omega);
    });
}

void bicg_rho(Ctx &c, int n, const double *r0, const double *r, RedArgs red)
{
    UG_LAUNCH_PDL(c, k_bicg_rho, row_grid(c, n), NT, 0, n, r0, r, red);
}

__global__ void k_bicg_p(int n, const double *__restrict__ r, double *__restrict__ p, const double *__restrict__ v,
                         const KScal *ks)
{
    PDL_ENTRY();
    if (ks->done) return;
    const double beta = ks->beta, bo = -ks->beta * ks->omega;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = 1.0 * r[i] + beta * p[i] + bo * v[i];
}

void bicg_p(Ctx &c, int n, const double *r, double *p, const double *v, RedArgs red)
{
    UG_LAUNCH_PDL(c, k_bicg_p, div_up(n, NT), NT, 0, n, r, p, v, red.ks);
}

template <class MV, class ZT>
__global__ void __launch_bounds__(NT) k_bicg_spmv_dot(MV A, const ZT *__restrict__ q, double *__restrict__ v,
                                                      const double *__restrict__ r0, RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    double sum = 0.0;
    const int stride = gridDim.x * NT, n = A.rows();
    for (int row = blockIdx.x * NT + threadIdx.x; row < n; row += stride) {
        double av = A.template dot<double>(q, row);
        v[row] = av;
        sum += av * r0[row];
    }
    double vv[1] = {sum};
    grid_reduce<NT, 1>(vv, red.partials, red.counter, [&](const double(&tot)[1]) {
        if (tot[0] == 0.0) {
            ks->fail = 1;
            ks->done = 1;
        }
        ks->alpha = ks->rho / tot[0];
    });
}

template <class ZT>
void bicg_spmv_dot_t(Ctx &c, const OpMat<double> &A, const ZT *q, double *v, const double *r0, RedArgs red)
{
    with_mv(A, [&](auto mv) {
        UG_LAUNCH_PDL(c, (k_bicg_spmv_dot<decltype(mv), ZT>), row_grid(c, A.nrows), NT, 0, mv, q, v, r0, red);
    });
}
template void bicg_spmv_dot_t<double>(Ctx &, const OpMat<double> &, const double *, double *, const double *, RedArgs);
template void bicg_spmv_dot_t<float>(Ctx &, const OpMat<double> &, const float *, double *, const double *, RedArgs);

template <class ZT>
__global__ void __launch_bounds__(NT) k_bicg_x_s(int n, double *__restrict__ x, const ZT *__restrict__ q,
                                                 const double *__restrict__ r, const double *__restrict__ v,
                                                 double *__restrict__ s, RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    const double alpha = ks->alpha;
    double sum = 0.0;
    const int stride = gridDim.x * NT;
    for (int i = blockIdx.x * NT + threadIdx.x; i < n; i += stride) {
        x[i] = 1.0 * x[i] + alpha * (double)q[i];
        double sv = 1.0 * r[i] + (-alpha) * v[i];
        s[i] = sv;
        sum += sv * sv;
    }
    double vv[1] = {sum};
    grid_reduce<NT, 1>(vv, red.partials, red.counter, [&](const double(&tot)[1]) { conv_update(ks, sqrt(tot[0]), 2); });
}

template <class ZT>
void bicg_x_s(Ctx &c, int n, double *x, const ZT *q, const double *r, const double *v, double *s, RedArgs red)
{
    UG_LAUNCH_PDL(c, k_bicg_x_s<ZT>, row_grid(c, n), NT, 0, n, x, q, r, v, s, red);
}
template void bicg_x_s<double>(Ctx &, int, double *, const double *, const double *, const double *, double *, RedArgs);
template void bicg_x_s<float>(Ctx &, int, double *, const float *, const double *, const double *, double *, RedArgs);

__global__ void k_bicg_s_to_r(int n, const double *__restrict__ s, double *__restrict__ r, const KScal *ks)
{
    PDL_ENTRY();
    if (ks->done != 2) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) r[i] = s[i];
}

void bicg_s_to_r(Ctx &c, int n, const double *s, double *r, RedArgs red)
{
    UG_LAUNCH_PDL(c, k_bicg_s_to_r, div_up(n, NT), NT, 0, n, s, r, red.ks);
}

template <class MV, class ZT>
__global__ void __launch_bounds__(NT) k_bicg_spmv_2dot(MV A, const ZT *__restrict__ q, double *__restrict__ t,
                                                       const double *__restrict__ s, RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    double tt = 0.0, st = 0.0;
    const int stride = gridDim.x * NT, n = A.rows();
    for (int row = blockIdx.x * NT + threadIdx.x; row < n; row += stride) {
        double av = A.template dot<double>(q, row);
        t[row] = av;
        tt += av * av;
        st += s[row] * av;
    }
    double vv[2] = {tt, st};
    grid_reduce<NT, 2>(vv, red.partials, red.counter, [&](const double(&tot)[2]) {
        if (tot[0] == 0.0) {
            ks->fail = 1;
            ks->done = 1;
        }
        ks->omega = tot[1] / tot[0];
    });
}

template <class ZT>
void bicg_spmv_2dot_t(Ctx &c, const OpMat<double> &A, const ZT *q, double *t, const double *s, RedArgs red)
{
    with_mv(A, [&](auto mv) {
        UG_LAUNCH_PDL(c, (k_bicg_spmv_2dot<decltype(mv), ZT>), row_grid(c, A.nrows), NT, 0, mv, q, t, s, red);
    });
}
template void bicg_spmv_2dot_t<double>(Ctx &, const OpMat<double> &, const double *, double *, const double *,
                                       RedArgs);
template void bicg_spmv_2dot_t<float>(Ctx &, const OpMat<double> &, const float *, double *, const double *, RedArgs);

template <class ZT>
__global__ void __launch_bounds__(NT) k_bicg_x_r(int n, double *__restrict__ x, const ZT *__restrict__ q,
                                                 const double *__restrict__ s, const double *__restrict__ t,
                                                 double *__restrict__ r, RedArgs red)
{
    PDL_ENTRY();
    KScal *ks = red.ks;
    if (ks->done) return;
    const double omega = ks->omega;
    double sum = 0.0;
    const int stride = gridDim.x * NT;
    for (int i = blockIdx.x * NT + threadIdx.x; i < n; i += stride) {
        x[i] = 1.0 * x[i] + omega * (double)q[i];
        double rv = 1.0 * s[i] + (-omega) * t[i];
        r[i] = rv;
        sum += rv * rv;
    }
    double vv[1] = {sum};
    grid_reduce<NT, 1>(vv, red.partials, red.counter, [&](const double(&tot)[1]) {
        conv_update(ks, sqrt(tot[0]), 1);
        if (ks->omega == 0.0) {
            ks->fail = 1;
            ks->done = 1;
        }
    });
}

template <class ZT>
void bicg_x_r(Ctx &c, int n, double *x, const ZT *q, const double *s, const double *t, double *r, RedArgs red)
{
    UG_LAUNCH_PDL(c, k_bicg_x_r<ZT>, row_grid(c, n), NT, 0, n, x, q, s, t, r, red);
}
template void bicg_x_r<double>(Ctx &, int, double *, const double *, const double *, const double *, double *, RedArgs);
template void bicg_x_r<float>(Ctx &, int, double *, const float *, const double *, const double *, double *, RedArgs);

// ------------------------------------------------------ vector/matrix API --
__global__ void __launch_bounds__(NT) k_vec_dot(int n, const double *__restrict__ a, const double *__restrict__ b,
                                                RedArgs red)
{
    PDL_ENTRY();
    double sum = 0.0;
    const int stride = gridDim.x * NT;
    for (int i = blockIdx.x * NT + threadIdx.x; i < n; i += stride) sum += a[i] * b[i];
    double v[1] = {sum};
    KScal *ks = red.ks;
    grid_reduce<NT, 1>(v, red.partials, red.counter, [&](const double(&tot)[1]) { ks->dot_out[0] = tot[0]; });
}

void vec_dot(Ctx &c, int n, const double *a, const double *b, RedArgs red)
{
    UG_LAUNCH_PDL(c, k_vec_dot, row_grid(c, n), NT, 0, n, a, b, red);
}

__global__ void k_vec_scale_add(int n, double *dest, double alpha, const double *a, double beta, const double *b)
{
    PDL_ENTRY();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dest[i] = alpha * a[i] + beta * b[i];
}

void vec_scale_add(Ctx &c, int n, double *dest, double alpha, const double *a, double beta, const double *b)
{
    UG_LAUNCH_PDL(c, k_vec_scale_add, div_up(n, NT), NT, 0, n, dest, alpha, a, beta, b);
}

// dest = alpha*v1 + beta*A*w1 (SparseMatrix::axpy, sparsematrix_impl.h:294-342)
template <class MV>
__global__ void __launch_bounds__(NT) k_op_axpy(MV A, double *dest, double alpha, const double *v1, double beta,
                                                const double *__restrict__ w1)
{
    PDL_ENTRY();
    const int stride = gridDim.x * NT, n = A.rows();
    for (int row = blockIdx.x * NT + threadIdx.x; row < n; row += stride) {
        double aw = A.template dot<double>(w1, row);
        dest[row] = (alpha == 0.0 ? 0.0 : alpha * v1[row]) + beta * aw;
    }
}

void op_axpy(Ctx &c, const OpMat<double> &A, double *dest, double alpha, const double *v1, double beta,
             const double *w1)
{
    with_mv(A, [&](auto mv) {
        UG_LAUNCH_PDL(c, k_op_axpy<decltype(mv)>, row_grid(c, A.nrows), NT, 0, mv, dest, alpha, v1, beta, w1);
    });
}

// dest += beta * A^T w1 (atomics; API path only)
__global__ void k_csr_axpy_t(int nrows, const int *rowptr, const int *col, const double *val, double *dest,
                             double beta, const double *w1)
{
    PDL_ENTRY();
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrows) return;
    double wr = beta * w1[r];
    for (int a = rowptr[r]; a < rowptr[r + 1]; ++a)
        if (val[a] != 0.0) atomicAdd(dest + col[a], val[a] * wr);
}

void csr_axpy_transposed(Ctx &c, const Csr &A, double *dest, double beta, const double *w1)
{
    UG_LAUNCH_PDL(c, k_csr_axpy_t, div_up(A.nrows, NT), NT, 0, A.nrows, A.rowptr.p, A.col.p, A.val.p, dest, beta, w1);
}

template <class TO, class TI>
__global__ void k_convert(int n, const TI *in, TO *out)
{
    PDL_ENTRY();
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (TO)in[i];
}

template <class TO, class TI>
void convert(Ctx &c, int n, const TI *in, TO *out)
{
    UG_LAUNCH_PDL(c, (k_convert<TO, TI>), div_up(n, NT), NT, 0, n, in, out);
}
template void convert<float, double>(Ctx &, int, const double *, float *);
template void convert<double, float>(Ctx &, int, const float *, double *);
template void convert<double, double>(Ctx &, int, const double *, double *);

}  // namespace ug4gb

// k_solve.cuh -- device-side state of the Krylov solvers and the launch
// wrappers of the multigrid / Krylov kernels (implemented in k_solve.cu).
// Every operator argument is an OpMat (SELL-32 or diagonal layout); the
// wrappers dispatch to the kernel instantiated for that layout.
#pragma once

#include <memory>

#include "common.cuh"

namespace ug4gb {

// Scalars of one Krylov solve, resident in device memory.  The finishing
// block of each reduction updates them, so no host round trip is needed
// between kernels.  Convergence follows StdConvCheck
// (lib_algebra/operator/convergence_check_impl.h:85-172).
struct KScal {
    int step, done, fail, restart;
    int maxit, hist_cap;
    double min_def, rel_red;
    double d0, dcur;
    double rho, rho_old, alpha, beta, lambda;   // CG
    double omega, norm_r0;                      // BiCGStab
    int num_restarts;                           // BiCGStab::set_restart (0: off)
    double min_ortho;                           // BiCGStab::set_min_orthogonality
    double dot_out[2];                          // plain reductions
    double *hist;                               // hist_cap entries
};

enum ScMode { SC_SET_FROM_BASE = 0, SC_ADD_FROM_BASE = 1, SC_ADD_FROM_NEW = 2 };

// Explicitly rounded arithmetic of the smoothing and transfer row updates.
// Every kernel that applies a damped-Jacobi step (one step per launch, or two
// fused) or the prolongation goes through these, so the compiler cannot
// contract them differently in different kernels: the results of all
// variants are bit-identical.
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

// One damped-Jacobi row update after the row's SpMV value acc = (At x)_i:
// dn = db - acc; t = dinv * (dn or db); sc (=|+=) t.  Returns dn; sc is
// updated in place (sc_in is only read when the mode adds).
template <class V>
__device__ __forceinline__ V jacobi_row(V acc, V db, V dinv, int mode, V sc_in, V &sc_out)
{
    const V dn = sub_rn(db, acc);
    const V t = mul_rn(dinv, mode == SC_ADD_FROM_NEW ? dn : db);
    sc_out = (mode == SC_SET_FROM_BASE) ? t : add_rn(sc_in, t);
    return dn;
}

struct RedArgs {
    double *partials;
    unsigned int *counter;
    KScal *ks;
};

// grid size used by every row-parallel kernel (grid-stride loops)
int row_grid(const Ctx &c, int nrows);

// ---- multigrid level kernels (V = level precision) ----
// dnew = dbase - At*x ; sc (=|+=) dinv*(dbase|dnew) ; optional dout = dnew;
// optional rho = sum sc_i * r_i (final top-level step inside a Krylov solve);
// optional z64 = (double) sc (mixed precision: FP64 correction for the Krylov loop)
template <class V, class XT, class DT>
void smooth_step(Ctx &c, const OpMat<V> &At, const XT *x, const DT *dbase, const V *dinv, V *sc, V *dout,
                 int sc_mode, const int *skip, const double *r_rho, RedArgs *red, int rho_kind,
                 double *z64 = nullptr);
struct GridPair;
// The operator of a structured 3D FP32 level prepared for smooth_pair: a copy
// with 16-byte aligned grid lines and its TMA tensor descriptor (k_sweep2.cu).
struct Sweep2Op;
// Set-up (may synchronise): null unless At is a 15- or 27-diagonal FP32
// operator of the structured level gp (nx, ny, nz) with the stencil of that
// level's element type and no nonzero entry towards a vertex outside it.
template <class V>
std::shared_ptr<Sweep2Op> sweep2_prepare(Ctx &c, const OpMat<V> &At, const GridPair &gp);
// Two consecutive damped-Jacobi steps of a structured 3D FP32 level in one
// pass over the operator (k_sweep2.cu):
//   step A: d1 = dbA - At xA,  sc (=|+=) dinv*(dbA|d1)   (modeA)
//   step B: d2 = d1 - At d1,   sc += dinv*(d1|d2)        (modeB)
// dbA == nullptr: dbA = xA.  dout (nullable) receives d2; r_rho / z64 as in
// smooth_step.  Returns false (and launches nothing) when op is null or the
// level does not qualify (see Ctx::sweep_fusion); the caller then applies the
// steps one by one.  Results are bit-identical to two smooth_step calls; only
// the summation order of the optional rho reduction differs.
template <class V>
bool smooth_pair(Ctx &c, const Sweep2Op *op, const GridPair &gp, const V *xA, const V *dbA, const V *dinv, V *sc,
                 V *dout, int modeA, int modeB, const int *skip, const double *r_rho, RedArgs *red, int rho_kind,
                 double *z64);
template <class V>
void restrict_apply(Ctx &c, const OpMat<V> &R, const V *d, V *dc, const int *skip);
template <class V>
void prolong_apply(Ctx &c, const OpMat<V> &P, const V *scc, V *sc, const V *dfac, V *w, const int *skip);
// StdTransfer on a structured hierarchy without a stored matrix: the
// parents of a fine vertex and the weights (1, 1/2, 1/4, 1/8; Dirichlet rows
// adjusted as in the assembled P and R) follow from its grid indices.  Same
// entries, same order of summation as the assembled P and R = P^T.
struct GridPair {
    int nx, ny, nz;      // fine level vertices per direction (nz = 1 in 2D)
    int cnx, cny, cnz;   // coarse level
    int dim, tet;        // tet: Kuhn split (two parents per edge midpoint)
    // StdTransfer::set_prolongation_damping / set_restriction_damping: factors
    // of the applied transfers (std_transfer_impl.h:740,792), 1 = none
    double dprol = 1.0, dres = 1.0;
};
__device__ __forceinline__ bool on_box_boundary(int i, int j, int k, int nx, int ny, int nz, int dim)
{
    return i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || (dim == 3 && (k == 0 || k == nz - 1));
}

// StdTransfer weight of a parent along `nodd` odd directions: 1, 1/2, 1/4, 1/8
template <class V>
__device__ __forceinline__ V grid_weight(int nodd)
{
    return nodd == 0 ? (V)1 : (nodd == 1 ? (V)0.5 : (nodd == 2 ? (V)0.25 : (V)0.125));
}

// t = (P scc)_f for the fine vertex f = (i, j, k): parents in increasing
// coarse index, as the rows of the assembled P (StdTransfer::
// assemble_prolongation_p1, std_transfer_impl.h:47-168, with
// DirichletBoundary::adjust_prolongation: a Dirichlet fine vertex keeps only
// a coinciding coarse parent, weight 1).
template <class V>
__device__ __forceinline__ V prolong_value(const GridPair &g, const V *__restrict__ scc, int i, int j, int k)
{
    const int p0 = i & 1, p1 = j & 1, p2 = k & 1, b0 = i >> 1, b1 = j >> 1, b2 = k >> 1;
    const bool bnd = on_box_boundary(i, j, k, g.nx, g.ny, g.nz, g.dim);
    V t = (V)0;
    if (g.tet) {
        const bool odd = (p0 | p1 | p2) != 0;
        const V wt = odd ? (bnd ? (V)0 : (V)0.5) : (V)1;
        t = fma_rn(wt, scc[b0 + g.cnx * (b1 + g.cny * b2)], t);
        if (odd) t = fma_rn(wt, scc[(b0 + p0) + g.cnx * ((b1 + p1) + g.cny * (b2 + p2))], t);
    } else {
        const int np = 1 << (p0 + p1 + p2);
        const V wt = bnd ? (np == 1 ? (V)1 : (V)0) : grid_weight<V>(p0 + p1 + p2);
        for (int dk = 0; dk <= p2; ++dk)
            for (int dj = 0; dj <= p1; ++dj)
                for (int di = 0; di <= p0; ++di)
                    t = fma_rn(wt, scc[(b0 + di) + g.cnx * ((b1 + dj) + g.cny * (b2 + dk))], t);
    }
    return t;
}

// dc = R d for coarse vertex (I, J, K): R = P^T, Dirichlet coarse rows =
// injection (k_restrict on the assembled R); children in increasing fine index
template <class V>
__device__ __forceinline__ void restrict_row(const GridPair &g, const V *__restrict__ d, V *__restrict__ dc, int I,
                                             int J, int K)
{
    const int c = I + g.cnx * (J + g.cny * K);
    const int fv = 2 * I + g.nx * (2 * J + g.ny * 2 * K);
    if (on_box_boundary(I, J, K, g.cnx, g.cny, g.cnz, g.dim)) {
        const V v = (V)0 + (V)1 * d[fv];
        dc[c] = (g.dres != 1.0) ? mul_rn(v, (V)g.dres) : v;
        return;
    }
    const int kr = (g.dim == 3) ? 1 : 0;
    V acc = (V)0;
    for (int dk = -kr; dk <= kr; ++dk)
        for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di) {
                const int nodd = (di != 0) + (dj != 0) + (dk != 0);
                V wt;
                if (g.tet) {
                    const bool pos = di > 0 || dj > 0 || dk > 0, neg = di < 0 || dj < 0 || dk < 0;
                    if (pos && neg) continue;   // not a Kuhn edge through this vertex
                    wt = nodd ? (V)0.5 : (V)1;
                } else {
                    wt = grid_weight<V>(nodd);
                }
                acc += wt * d[fv + di + g.nx * (dj + g.ny * dk)];
            }
    dc[c] = (g.dres != 1.0) ? mul_rn(acc, (V)g.dres) : acc;
}

template <class V>
void prolong_grid(Ctx &c, const GridPair &g, const V *scc, V *sc, const V *dfac, V *w, const int *skip);
template <class V>
void restrict_grid(Ctx &c, const GridPair &g, const V *d, V *dc, const int *skip);
template <class V>
void base_solve(Ctx &c, const double *Ainv, int n, const V *d, V *sc, const int *skip);

// ---- the coarse end of a V-cycle in one launch (k_coarse.cu) ----
// Levels [0] (the base, dense LU inverse) .. [m-1] (the entry level) of a
// structured hierarchy with damped-Jacobi smoothing on diagonal-layout
// operators and grid transfers; the entry level's defect arrives in d_in
// (its dA) and its correction leaves in sc_out (its sc), bit-identical to
// the separate launches of lmgc.  The kernel keeps everything in shared
// memory: Ainv (nbase^2 doubles) at byte 0 followed by the base defect in
// FP64 (nbase doubles), then the level-precision region
// at byte vbase holding, per level, the operator (S x ld), the Jacobi
// factors and the vectors, at the element offsets below (the operator and
// the factors 16-byte aligned).
constexpr int kCoarseMaxLevels = 8;
template <class V>
struct alignas(16) CoarseLevel {
    const V *val;           // column-scaled operator At, diagonal layout (Dia::vals(), S x ld)
    const V *dinv, *dfac;   // Jacobi factors (unused on the base level)
    int n, ncols, ld, S;
    int off[kMaxDiag];
    GridPair gp;            // this level and the next coarser one (unused on the base level)
    int aofs;               // operator values (S * ld elements)
    int iofs, fofs;         // dinv, dfac (n elements each)
    int vofs;               // vectors sc, dA[, dB, w] (n elements each)
};
template <class V>
struct alignas(16) CoarsePlan {
    int m, nu1, nu2, nbase;
    const double *Ainv;     // nbase x nbase, row-major
    const V *d_in;
    V *sc_out;
    int vbase;              // byte offset of the level-precision region
    CoarseLevel<V> lev[kCoarseMaxLevels];
};
// plan_dev: the plan in device memory (written at set-up); S: the stencil
// width of every level above the base (coarse_width_ok); smem_bytes: the
// extent of the layout above
template <class V>
void coarse_cycle(Ctx &c, const CoarsePlan<V> *plan_dev, int S, size_t smem_bytes, const int *skip);
bool coarse_width_ok(int S);
// set-up: allows launches with up to smem_bytes of dynamic shared memory
template <class V>
void coarse_prepare(size_t smem_bytes);
template <class V>
void mcgs_colour(Ctx &c, const OpMat<V> &A, const int *rows, int nrows_c, const V *dinv_relax, const V *d, V *t,
                 const int *skip);
// d_out = d_base - A t ; sc_mode 1: sc = t, 0: sc += t, 2: sc untouched
template <class V, class DT>
void residual_update(Ctx &c, const OpMat<V> &A, const V *t, const DT *dbase, V *dout, V *sc, int sc_mode,
                     const int *skip);

// ILU(0) in multicolour order (k_ilu.cu): level CRS rows re-ordered by
// (colour, column), L multipliers before the diagonal, U from the diagonal on
template <class V>
struct IluFactors {
    int n = 0;
    DevBuf<int> rowptr, col, nlow;   // nlow[i]: position of the diagonal in row i
    DevBuf<V> val, uinv;
};
// factorise the level operator A (FP64) with the vertex colours `color` and the
// rows of each colour; throws UG4GB_ERR_SINGULAR on a zero pivot
template <class V>
void ilu_setup(Ctx &c, const Csr &A, const int *color, const std::vector<DevBuf<int>> &crow,
               const std::vector<int> &ncrow, IluFactors<V> &F);
// t = damp (L U)^{-1} d (y: scratch of the forward substitution)
template <class V>
void ilu_apply(Ctx &c, const IluFactors<V> &F, const std::vector<DevBuf<int>> &crow, const std::vector<int> &ncrow,
               const V *d, V *y, V *t, double damp, const int *skip);

// ---- Krylov kernels (FP64 outer vectors; z may be FP32 in mixed mode) ----
// r -= A x, |r| starts the check; optionally r32 = (float) r
void krylov_start(Ctx &c, const OpMat<double> &A, const double *x, double *r, RedArgs red, float *r32 = nullptr);
// first: p = z, q = A z; else p = z + beta p, q = A z + beta q; lambda = (q,p), alpha = rho_old/lambda
template <class ZT>
void cg_spmv_dot_t(Ctx &c, const OpMat<double> &A, const ZT *z, double *p, double *q, int first, RedArgs red);
// x += alpha p, r -= alpha q, |r| -> check; optionally r32 = (float) r
void cg_update(Ctx &c, int n, double *x, double *r, const double *p, const double *q, RedArgs red,
               float *r32 = nullptr);
// rho = (z, r); kind 0: rho_old = rho (first), 1: beta = rho/rho_old, rho_old = rho
template <class ZT>
void rho_dot(Ctx &c, int n, const ZT *z, const double *r, int kind, RedArgs red);
template <class ZT>
void copy_z(Ctx &c, int n, const ZT *z, double *out, const int *skip);

void bicg_restart(Ctx &c, int n, const double *r, double *r0, double *p, double *v, RedArgs red);
void bicg_rho(Ctx &c, int n, const double *r0, const double *r, RedArgs red);
void bicg_p(Ctx &c, int n, const double *r, double *p, const double *v, RedArgs red);
template <class ZT>
void bicg_spmv_dot_t(Ctx &c, const OpMat<double> &A, const ZT *q, double *v, const double *r0, RedArgs red);
template <class ZT>
void bicg_x_s(Ctx &c, int n, double *x, const ZT *q, const double *r, const double *v, double *s, RedArgs red);
void bicg_s_to_r(Ctx &c, int n, const double *s, double *r, RedArgs red);
template <class ZT>
void bicg_spmv_2dot_t(Ctx &c, const OpMat<double> &A, const ZT *q, double *t, const double *s, RedArgs red);
template <class ZT>
void bicg_x_r(Ctx &c, int n, double *x, const ZT *q, const double *s, const double *t, double *r, RedArgs red);

// ---- BLAS-1 / SpMV for the public vector and matrix API ----
void vec_dot(Ctx &c, int n, const double *a, const double *b, RedArgs red);
void vec_scale_add(Ctx &c, int n, double *dest, double alpha, const double *a, double beta, const double *b);
void op_axpy(Ctx &c, const OpMat<double> &A, double *dest, double alpha, const double *v1, double beta,
             const double *w1);
void csr_axpy_transposed(Ctx &c, const Csr &A, double *dest, double beta, const double *w1);
template <class TO, class TI>
void convert(Ctx &c, int n, const TI *in, TO *out);

}  // namespace ug4gb

// k_solve.cuh -- device-side state of the Krylov solvers and the launch
// wrappers of the multigrid / Krylov kernels (implemented in k_solve.cu).
// Every operator argument is an OpMat (SELL-32 or diagonal layout); the
// wrappers dispatch to the kernel instantiated for that layout.
#pragma once

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
    double dot_out[2];                          // plain reductions
    double *hist;                               // hist_cap entries
};

enum ScMode { SC_SET_FROM_BASE = 0, SC_ADD_FROM_BASE = 1, SC_ADD_FROM_NEW = 2 };

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
};
template <class V>
void prolong_grid(Ctx &c, const GridPair &g, const V *scc, V *sc, const V *dfac, V *w, const int *skip);
template <class V>
void restrict_grid(Ctx &c, const GridPair &g, const V *d, V *dc, const int *skip);
template <class V>
void base_solve(Ctx &c, const double *Ainv, int n, const V *d, V *sc, const int *skip);
// once per base size, outside stream capture: allows the shared-memory copy of Ainv
template <class V>
void base_solve_prepare(int n);
template <class V>
void mcgs_colour(Ctx &c, const OpMat<V> &A, const int *rows, int nrows_c, const V *dinv_relax, const V *d, V *t,
                 const int *skip);
// d_out = d_base - A t ; sc_mode 1: sc = t, 0: sc += t, 2: sc untouched
template <class V, class DT>
void residual_update(Ctx &c, const OpMat<V> &A, const V *t, const DT *dbase, V *dout, V *sc, int sc_mode,
                     const int *skip);

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

/*
 * ug4_oracle_solve.c -- oracle: transfers, smoothers, LU, GMG, CG, BiCGStab.
 *
 * TEST INFRASTRUCTURE ONLY (see ug4_oracle.h).
 *
 *  - StdTransfer::assemble_prolongation_p1
 *    (lib_disc/operator/linear_operator/std_transfer_impl.h:47-168): vertex
 *    parent 1, edge 1/2, quadrilateral 1/4, hexahedron 1/8.
 *  - DirichletBoundary::adjust_prolongation / adjust_restriction
 *    (lib_disc/spatial_disc/constraints/dirichlet_boundary/
 *     lagrange_dirichlet_boundary_impl.h:545-616,677-752): Dirichlet fine rows
 *    of P set to 0 (pattern kept) and P(f, vertex parent) = 1; R = P^T by
 *    set_as_transpose_of (std_transfer_impl.h:695), then rows of coarse
 *    Dirichlet vertices 0 and R(c, child) = 1.
 *  - Jacobi<TAlgebra>::preprocess/step (lib_algebra/operator/preconditioner/
 *    jacobi.h:155-253): diagInv = 1 / (a_ii * (1/damp)); c = diagInv * d.
 *  - LU (lib_algebra/operator/linear_solver/lu.h:236-300) dense path with
 *    LUDecomp / SolveLU (lib_algebra/small_algebra/no_lapack/lu_decomp.h:48-200).
 *  - AssembledMultiGridCycle::apply / lmgc / presmooth_and_restriction /
 *    prolongation_and_postsmooth / base_solve
 *    (lib_disc/operator/linear_operator/multi_grid_solver/
 *     mg_solver_impl.hpp:176-275,1687-2140) for a fully refined hierarchy
 *    (m_LocalFullRefLevel == top level).
 *  - CG<TVector>::apply_return_defect (lib_algebra/operator/linear_solver/cg.h:103-230)
 *  - BiCGStab<TVector>::apply_return_defect
 *    (lib_algebra/operator/linear_solver/bicgstab.h:112-400), restarts off,
 *    minOrtho 0 (the defaults, bicgstab.h:85-97).
 *  - StdConvCheck<TVector> (lib_algebra/operator/convergence_check_impl.h:85-172).
 */
#include "ug4_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------ transfers -- */
int orc_prolongation(const orc_level *F, const orc_level *C, orc_crs *P)
{
    memset(P, 0, sizeof(*P));
    P->n_rows = F->nv; P->n_cols = C->nv;
    P->rowptr = (int *)calloc((size_t)F->nv + 1, sizeof(int));
    for (int v = 0; v < F->nv; ++v) P->rowptr[v + 1] = P->rowptr[v] + F->npar[v];
    P->nnz = P->rowptr[F->nv];
    P->col = (int *)malloc(sizeof(int) * (size_t)P->nnz);
    P->val = (double *)malloc(sizeof(double) * (size_t)P->nnz);
    if (!P->rowptr || !P->col || !P->val) return -1;
    for (int v = 0; v < F->nv; ++v) {
        int n = F->npar[v];
        double w = (n == 1) ? 1.0 : (n == 2 ? 0.5 : (n == 4 ? 0.25 : 0.125));
        for (int j = 0; j < n; ++j) {
            P->col[P->rowptr[v] + j] = F->par[8 * (size_t)v + j];
            P->val[P->rowptr[v] + j] = w;
        }
        /* Dirichlet adjustment */
        if (F->bnd[v]) {
            for (int a = P->rowptr[v]; a < P->rowptr[v + 1]; ++a) P->val[a] = 0.0;
            if (n == 1) P->val[P->rowptr[v]] = 1.0;
        }
    }
    return 0;
}

int orc_restriction(const orc_level *F, const orc_level *C, const orc_crs *P, orc_crs *R)
{
    if (orc_crs_transpose(P, 1, R)) return -1;
    for (int v = 0; v < F->nv; ++v) {
        if (!F->bnd[v] || F->npar[v] != 1) continue;
        int c = F->par[8 * (size_t)v];
        for (int a = R->rowptr[c]; a < R->rowptr[c + 1]; ++a) R->val[a] = 0.0;
        R->val[orc_crs_find(R, c, v)] = 1.0;
    }
    (void)C;
    return 0;
}

/* ----------------------------------------------------- Galerkin R A P -- */
static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

int orc_rap(const orc_crs *R, const orc_crs *A, const orc_crs *P, orc_crs *M)
{
    memset(M, 0, sizeof(*M));
    const int nr = R->n_rows, nc = P->n_cols;
    M->n_rows = nr; M->n_cols = nc;
    double *acc = (double *)calloc((size_t)nc, sizeof(double));
    int *mark = (int *)malloc(sizeof(int) * (size_t)nc);
    int *list = (int *)malloc(sizeof(int) * (size_t)nc);
    M->rowptr = (int *)calloc((size_t)nr + 1, sizeof(int));
    int64_t cap = 16 * (int64_t)nr + 16;
    M->col = (int *)malloc(sizeof(int) * (size_t)cap);
    M->val = (double *)malloc(sizeof(double) * (size_t)cap);
    if (!acc || !mark || !list || !M->rowptr || !M->col || !M->val) return -1;
    for (int j = 0; j < nc; ++j) mark[j] = -1;
    int64_t nnz = 0;
    for (int i = 0; i < nr; ++i) {
        int nl = 0;
        for (int a = R->rowptr[i]; a < R->rowptr[i + 1]; ++a) {
            if (R->val[a] == 0.0) continue;
            const int k = R->col[a];
            for (int b = A->rowptr[k]; b < A->rowptr[k + 1]; ++b) {
                if (A->val[b] == 0.0) continue;
                const int l = A->col[b];
                const double ab = R->val[a] * A->val[b];
                for (int c = P->rowptr[l]; c < P->rowptr[l + 1]; ++c) {
                    if (P->val[c] == 0.0) continue;
                    const int j = P->col[c];
                    if (mark[j] != i) { mark[j] = i; acc[j] = 0.0; list[nl++] = j; }
                    acc[j] = acc[j] + ab * P->val[c];
                }
            }
        }
        qsort(list, (size_t)nl, sizeof(int), cmp_int);
        if (nnz + nl > cap) {
            while (nnz + nl > cap) cap *= 2;
            M->col = (int *)realloc(M->col, sizeof(int) * (size_t)cap);
            M->val = (double *)realloc(M->val, sizeof(double) * (size_t)cap);
            if (!M->col || !M->val) return -1;
        }
        for (int t = 0; t < nl; ++t) {
            M->col[nnz] = list[t];
            M->val[nnz] = acc[list[t]];
            ++nnz;
        }
        M->rowptr[i + 1] = (int)nnz;
    }
    M->nnz = nnz;
    free(acc); free(mark); free(list);
    return 0;
}

/* ------------------------------------------------------------------ LU -- */
int orc_lu_init(orc_lu *F, const orc_crs *A)
{
    int n = A->n_rows;
    F->n = n;
    F->LU = (double *)calloc((size_t)n * n, sizeof(double));
    F->piv = (int *)calloc((size_t)n, sizeof(int));
    if (!F->LU || !F->piv) return -1;
    for (int r = 0; r < n; ++r)
        for (int a = A->rowptr[r]; a < A->rowptr[r + 1]; ++a) F->LU[(size_t)r * n + A->col[a]] = A->val[a];
    double *M = F->LU;
    for (int k = 0; k < n; ++k) {
        int big = k;
        for (int j = k + 1; j < n; ++j)
            if (fabs(M[(size_t)big * n + k]) < fabs(M[(size_t)j * n + k])) big = j;
        if (big != k)
            for (int j = 0; j < n; ++j) {
                double t = M[(size_t)k * n + j]; M[(size_t)k * n + j] = M[(size_t)big * n + j]; M[(size_t)big * n + j] = t;
            }
        F->piv[k] = big;
        if (fabs(M[(size_t)k * n + k]) < 1e-10) return -2;
        for (int i = k + 1; i < n; ++i) {
            M[(size_t)i * n + k] = M[(size_t)i * n + k] / M[(size_t)k * n + k];
            for (int j = k + 1; j < n; ++j)
                M[(size_t)i * n + j] = M[(size_t)i * n + j] - M[(size_t)i * n + k] * M[(size_t)k * n + j];
        }
    }
    return 0;
}

void orc_lu_apply(const orc_lu *F, double *x, const double *b)
{
    int n = F->n;
    const double *M = F->LU;
    for (int i = 0; i < n; ++i) x[i] = b[i];
    for (int i = 0; i < n; ++i)
        if (i < F->piv[i]) { double t = x[i]; x[i] = x[F->piv[i]]; x[F->piv[i]] = t; }
    for (int i = 0; i < n; ++i) {
        double s = x[i];
        for (int k = 0; k < i; ++k) s -= M[(size_t)i * n + k] * x[k];
        x[i] = s;
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = x[i];
        for (int k = i + 1; k < n; ++k) s -= M[(size_t)i * n + k] * x[k];
        x[i] = s / M[(size_t)i * n + i];
    }
}

void orc_lu_free(orc_lu *F) { free(F->LU); free(F->piv); F->LU = NULL; F->piv = NULL; }

/* ----------------------------------------------------------------- GMG -- */
static double *dvec(int n) { return (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }

/* ILU(0) in multicolour order (ILU, lib_algebra/operator/preconditioner/
   ilu.h:109-210, of the colour-permuted operator): rows re-ordered by
   (colour, column), IKJ elimination on A's pattern, colour by colour in
   increasing order (rows of one colour are not coupled) */
static long long ilu_key(const int *color, int n, int j) { return (long long)color[j] * n + j; }

static int ilu_factor(const orc_crs *A, const int *color, int ncolor, orc_crs *F, int **diag_out)
{
    const int n = A->n_rows;
    F->n_rows = F->n_cols = n;
    F->nnz = A->nnz;
    F->rowptr = (int *)malloc(sizeof(int) * (size_t)(n + 1));
    F->col = (int *)malloc(sizeof(int) * (size_t)(A->nnz > 0 ? A->nnz : 1));
    F->val = (double *)malloc(sizeof(double) * (size_t)(A->nnz > 0 ? A->nnz : 1));
    int *dg = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!F->rowptr || !F->col || !F->val || !dg) return -1;
    memcpy(F->rowptr, A->rowptr, sizeof(int) * (size_t)(n + 1));
    memcpy(F->col, A->col, sizeof(int) * (size_t)A->nnz);
    memcpy(F->val, A->val, sizeof(double) * (size_t)A->nnz);
    for (int r = 0; r < n; ++r) {
        const int a0 = F->rowptr[r], a1 = F->rowptr[r + 1];
        for (int a = a0 + 1; a < a1; ++a) {          /* insertion sort by key */
            const int cc = F->col[a];
            const double vv = F->val[a];
            const long long kk = ilu_key(color, n, cc);
            int b = a - 1;
            while (b >= a0 && ilu_key(color, n, F->col[b]) > kk) {
                F->col[b + 1] = F->col[b]; F->val[b + 1] = F->val[b]; --b;
            }
            F->col[b + 1] = cc; F->val[b + 1] = vv;
        }
        int lo = 0;
        for (int a = a0; a < a1; ++a) lo += ilu_key(color, n, F->col[a]) < ilu_key(color, n, r);
        dg[r] = a0 + lo;
    }
    for (int c = 0; c < ncolor; ++c)
        for (int i = 0; i < n; ++i) {
            if (color[i] != c) continue;
            const int a1 = F->rowptr[i + 1];
            for (int p = F->rowptr[i]; p < dg[i]; ++p) {
                const int k = F->col[p];
                const double ukk = F->val[dg[k]];
                if (ukk == 0.0) return -2;
                const double l = F->val[p] / ukk;
                F->val[p] = l;
                for (int s = p + 1; s < a1; ++s) {
                    const long long js = ilu_key(color, n, F->col[s]);
                    for (int q = dg[k] + 1; q < F->rowptr[k + 1]; ++q)
                        if (ilu_key(color, n, F->col[q]) == js) { F->val[s] -= l * F->val[q]; break; }
                }
            }
            if (F->val[dg[i]] == 0.0) return -2;
        }
    *diag_out = dg;
    return 0;
}

/* c = damp (L U)^{-1} d: forward over the colours, then backward */
static void ilu_apply(const orc_crs *F, const int *dg, const int *color, int ncolor, double damp, double *c,
                      const double *d, double *y)
{
    const int n = F->n_rows;
    for (int col = 0; col < ncolor; ++col)
        for (int i = 0; i < n; ++i) {
            if (color[i] != col) continue;
            double s = d[i];
            for (int a = F->rowptr[i]; a < dg[i]; ++a) s -= F->val[a] * y[F->col[a]];
            y[i] = s;
        }
    for (int col = ncolor - 1; col >= 0; --col)
        for (int i = 0; i < n; ++i) {
            if (color[i] != col) continue;
            double s = y[i];
            for (int a = dg[i] + 1; a < F->rowptr[i + 1]; ++a) s -= F->val[a] * c[F->col[a]];
            c[i] = s * (1.0 / F->val[dg[i]]);
        }
    if (damp != 1.0)
        for (int i = 0; i < n; ++i) c[i] *= damp;
}

int orc_gmg_init(orc_gmg *G, const orc_hier *H, orc_crs *levA, int smoother, double damp,
                 int nu1, int nu2, int cycle, int base, int rap)
{
    return orc_gmg_init_ex(G, H, levA, smoother, damp, nu1, nu2, cycle, base, rap, 0);
}

int orc_gmg_init_ex(orc_gmg *G, const orc_hier *H, orc_crs *levA, int smoother, double damp,
                    int nu1, int nu2, int cycle, int base, int rap, int base_steps)
{
    memset(G, 0, sizeof(*G));
    G->base_kind = base_steps > 0 ? 1 : 0;
    G->base_steps = base_steps;
    G->nlev = H->nlev; G->base = base; G->cycle = cycle; G->nu1 = nu1; G->nu2 = nu2;
    G->smoother = smoother; G->damp = damp;
    G->smoother2 = smoother; G->damp2 = damp;
    G->damp_prol = 1.0; G->damp_res = 1.0;
    G->A = levA;
    G->P = (orc_crs *)calloc((size_t)G->nlev, sizeof(orc_crs));
    G->R = (orc_crs *)calloc((size_t)G->nlev, sizeof(orc_crs));
    if (rap) {
        /* transfers first, then the coarse operators from the top down */
        const int top = G->nlev - 1;
        G->Arap = (orc_crs *)calloc((size_t)G->nlev, sizeof(orc_crs));
        G->Arap[top] = levA[top];
        for (int l = top; l > base; --l) {
            if (orc_prolongation(&H->lev[l], &H->lev[l - 1], &G->P[l])) return -1;
            if (orc_restriction(&H->lev[l], &H->lev[l - 1], &G->P[l], &G->R[l])) return -1;
            if (orc_rap(&G->R[l], &G->Arap[l], &G->P[l], &G->Arap[l - 1])) return -1;
        }
        levA = G->Arap;
        G->A = levA;
    }
    G->diaginv = (double **)calloc((size_t)G->nlev, sizeof(double *));
    G->color = (int **)calloc((size_t)G->nlev, sizeof(int *));
    G->ncolor = (int *)calloc((size_t)G->nlev, sizeof(int));
    G->sc = (double **)calloc((size_t)G->nlev, sizeof(double *));
    G->sd = (double **)calloc((size_t)G->nlev, sizeof(double *));
    G->st = (double **)calloc((size_t)G->nlev, sizeof(double *));
    for (int l = base; l < G->nlev; ++l) {
        const orc_level *L = &H->lev[l];
        int n = L->nv;
        G->sc[l] = dvec(n); G->sd[l] = dvec(n); G->st[l] = dvec(n);
        if (l > base && !rap) {
            if (orc_prolongation(L, &H->lev[l - 1], &G->P[l])) return -1;
            if (orc_restriction(L, &H->lev[l - 1], &G->P[l], &G->R[l])) return -1;
        }
        /* smoother data on every level above the base, and on the base level
           when it smooths instead of the LU */
        if (l > base || G->base_kind == 1) {
            G->diaginv[l] = dvec(n);
            for (int i = 0; i < n; ++i) {
                double m = levA[l].val[orc_crs_find(&levA[l], i, i)];
                m *= 1. / damp;
                G->diaginv[l][i] = 1. / m;
            }
            /* parity colouring of the structured level (valid for the 9-, 27-
               and 15-point stencils: neighbours differ in at least one parity) */
            G->color[l] = (int *)malloc(sizeof(int) * (size_t)n);
            G->ncolor[l] = 1 << L->dim;
            for (int k = 0; k < L->nz; ++k)
                for (int j = 0; j < L->ny; ++j)
                    for (int i = 0; i < L->nx; ++i)
                        G->color[l][i + L->nx * (j + L->ny * k)] = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2);
        }
    }
    if (G->smoother == ORC_SMOOTH_ILU) {
        G->ilu = (orc_crs *)calloc((size_t)G->nlev, sizeof(orc_crs));
        G->ilu_diag = (int **)calloc((size_t)G->nlev, sizeof(int *));
        for (int l = base + 1 - G->base_kind; l < G->nlev; ++l)
            if (ilu_factor(&levA[l], G->color[l], G->ncolor[l], &G->ilu[l], &G->ilu_diag[l])) return -3;
    }
    if (G->base_kind == 0 && orc_lu_init(&G->lu, &levA[base])) return -2;
    return 0;
}

int orc_gmg_set_postsmoother(orc_gmg *G, int smoother, double damp)
{
    G->smoother2 = smoother;
    G->damp2 = damp;
    if (smoother == ORC_SMOOTH_JACOBI) {
        if (!G->diaginv2) G->diaginv2 = (double **)calloc((size_t)G->nlev, sizeof(double *));
        for (int l = G->base + 1; l < G->nlev; ++l) {
            int n = G->A[l].n_rows;
            free(G->diaginv2[l]);
            G->diaginv2[l] = dvec(n);
            for (int i = 0; i < n; ++i) {
                double m = G->A[l].val[orc_crs_find(&G->A[l], i, i)];
                m *= 1. / damp;
                G->diaginv2[l][i] = 1. / m;
            }
        }
    }
    if (smoother == ORC_SMOOTH_ILU && !G->ilu) {
        G->ilu = (orc_crs *)calloc((size_t)G->nlev, sizeof(orc_crs));
        G->ilu_diag = (int **)calloc((size_t)G->nlev, sizeof(int *));
        for (int l = G->base + 1; l < G->nlev; ++l)
            if (ilu_factor(&G->A[l], G->color[l], G->ncolor[l], &G->ilu[l], &G->ilu_diag[l])) return -3;
    }
    return 0;
}

/* multicolour Gauss-Seidel sweep from zero: c = B d */
static void mcgs_apply(const orc_crs *A, const int *color, int ncolor, double relax, double *c, const double *d)
{
    int n = A->n_rows;
    memset(c, 0, sizeof(double) * (size_t)n);
    for (int col = 0; col < ncolor; ++col)
        for (int i = 0; i < n; ++i) {
            if (color[i] != col) continue;
            double s = d[i], diag = 1.0;
            for (int a = A->rowptr[i]; a < A->rowptr[i + 1]; ++a) {
                if (A->col[a] == i) diag = A->val[a];
                else s -= A->val[a] * c[A->col[a]];
            }
            c[i] = relax * s / diag;
        }
}

/* the symmetric sweep's second half (sgs_step, lib_algebra/algebra_common/
   core_smoothers.h:189-206, in colour order): c2 = D c1, then gs_step_UR
   (:150-172) in place, c_i = relax (c2_i - sum over later colours of
   a_ij c_j) / a_ii, colours descending */
static void mcsgs_backward(const orc_crs *A, const int *color, int ncolor, double relax, double *c)
{
    int n = A->n_rows;
    for (int i = 0; i < n; ++i) c[i] = 1.0 * A->val[orc_crs_find(A, i, i)] * c[i];
    for (int col = ncolor - 1; col >= 0; --col)
        for (int i = 0; i < n; ++i) {
            if (color[i] != col) continue;
            double s = c[i], diag = 1.0;
            for (int a = A->rowptr[i]; a < A->rowptr[i + 1]; ++a) {
                const int j = A->col[a];
                if (j == i) diag = A->val[a];
                else if (color[j] > col) s -= A->val[a] * c[j];
            }
            c[i] = relax * s / diag;
        }
}

/* backward multicolour sweep on c (BackwardGaussSeidel, gauss_seidel.h:316,
   in colour order): c_i += relax (d_i - (A c)_i) / a_ii, colours descending */
static void mcgs_backward(const orc_crs *A, const int *color, int ncolor, double relax, double *c, const double *d)
{
    int n = A->n_rows;
    for (int col = ncolor - 1; col >= 0; --col)
        for (int i = 0; i < n; ++i) {
            if (color[i] != col) continue;
            double s = d[i], diag = 1.0;
            for (int a = A->rowptr[i]; a < A->rowptr[i + 1]; ++a) {
                if (A->col[a] == i) diag = A->val[a];
                s -= A->val[a] * c[A->col[a]];
            }
            c[i] += relax * s / diag;
        }
}

/* one smoothing step c = B d from zero: the pre-smoother (post = 0) or the
   post-smoother (post = 1) */
static void smooth(orc_gmg *G, int l, double *c, const double *d, int post)
{
    int n = G->A[l].n_rows;
    const int kind = post ? G->smoother2 : G->smoother;
    const double damp = post ? G->damp2 : G->damp;
    if (kind == ORC_SMOOTH_JACOBI) {
        const double *di = (post && G->diaginv2) ? G->diaginv2[l] : G->diaginv[l];
        for (int i = 0; i < n; ++i) c[i] = di[i] * d[i];
    } else {
        if (kind == ORC_SMOOTH_ILU) {
            double *y = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
            ilu_apply(&G->ilu[l], G->ilu_diag[l], G->color[l], G->ncolor[l], damp, c, d, y);
            free(y);
            return;
        }
        if (kind == ORC_SMOOTH_MCBGS) {
            memset(c, 0, sizeof(double) * (size_t)n);
            mcgs_backward(&G->A[l], G->color[l], G->ncolor[l], damp, c, d);
            return;
        }
        mcgs_apply(&G->A[l], G->color[l], G->ncolor[l], damp, c, d);
        if (kind == ORC_SMOOTH_MCSGS) mcsgs_backward(&G->A[l], G->color[l], G->ncolor[l], damp, c);
    }
}

static void vadd(int n, double *a, const double *b);

static void base_solve(orc_gmg *G, int l)
{
    if (G->base_kind == 1) {
        /* LinearSolver::apply_return_defect (linear_solver.h) on a copy of
           the defect: c = B d, x += c, d -= A c, base_steps times */
        int n = G->A[l].n_rows;
        double *d = dvec(n), *c = dvec(n);
        memcpy(d, G->sd[l], sizeof(double) * (size_t)n);
        memset(G->sc[l], 0, sizeof(double) * (size_t)n);
        for (int k = 0; k < G->base_steps; ++k) {
            smooth(G, l, c, d, 0);
            vadd(n, G->sc[l], c);
            orc_crs_matmul_minus(&G->A[l], d, c);
        }
        free(d);
        free(c);
    } else {
        orc_lu_apply(&G->lu, G->sc[l], G->sd[l]);
    }
    if (l >= G->nlev - 1) orc_crs_matmul_minus(&G->A[l], G->sd[l], G->sc[l]);
}

static void vadd(int n, double *a, const double *b) { for (int i = 0; i < n; ++i) a[i] += b[i]; }

static void presmooth_and_restriction(orc_gmg *G, int l)
{
    int n = G->A[l].n_rows, nc = G->A[l - 1].n_rows;
    for (int nu = 0; nu < G->nu1; ++nu) {
        smooth(G, l, G->st[l], G->sd[l], 0);
        orc_crs_matmul_minus(&G->A[l], G->sd[l], G->st[l]);
        if (nu < G->nu1 - 1) vadd(n, G->sc[l], G->st[l]);
    }
    memset(G->sc[l - 1], 0, sizeof(double) * (size_t)nc);
    if (G->nu1 > 0) vadd(n, G->sc[l], G->st[l]);
    /* StdTransfer::do_restrict (std_transfer_impl.h:776-806): R applied
       with the restriction damping as its factor */
    orc_crs_apply_ignore_zero_rows(&G->R[l], G->sd[l - 1], G->damp_res, G->sd[l]);
}

static void prolongation_and_postsmooth(orc_gmg *G, int l)
{
    int n = G->A[l].n_rows;
    /* StdTransfer::prolongate (std_transfer_impl.h:721-772): P.axpy with the
       prolongation damping as its factor */
    orc_crs_axpy(&G->P[l], G->st[l], 0.0, G->st[l], G->damp_prol, G->sc[l - 1]);
    vadd(n, G->sc[l], G->st[l]);
    for (int nu = 0; nu < G->nu2; ++nu) {
        orc_crs_matmul_minus(&G->A[l], G->sd[l], G->st[l]);
        smooth(G, l, G->st[l], G->sd[l], 1);
        vadd(n, G->sc[l], G->st[l]);
    }
    if (l >= G->nlev - 1) orc_crs_matmul_minus(&G->A[l], G->sd[l], G->st[l]);
}

/* AssembledMultiGridCycle::lmgc (mg_solver_impl.hpp:2091-2134): cycle type
   gamma >= 1 (V = 1, W = 2) visits the coarser level gamma times; the
   F-cycle (-1) visits it once as an F-cycle, then once as a V-cycle */
static void lmgc(orc_gmg *G, int l, int ctype)
{
    int top = G->nlev - 1;
    if (l == G->base) { base_solve(G, top); return; }
    presmooth_and_restriction(G, l);
    if (l - 1 == G->base) base_solve(G, l - 1);
    else if (ctype == -1) { lmgc(G, l - 1, -1); lmgc(G, l - 1, 1); }
    else for (int i = 0; i < ctype; ++i) lmgc(G, l - 1, ctype);
    prolongation_and_postsmooth(G, l);
}

void orc_gmg_apply(orc_gmg *G, double *c, const double *d)
{
    int top = G->nlev - 1, n = G->A[top].n_rows;
    memcpy(G->sd[top], d, sizeof(double) * (size_t)n);
    memset(c, 0, sizeof(double) * (size_t)n);
    memset(G->sc[top], 0, sizeof(double) * (size_t)n);
    lmgc(G, top, G->cycle);
    for (int i = 0; i < n; ++i) c[i] += G->sc[top][i];
}

void orc_gmg_free(orc_gmg *G)
{
    for (int l = 0; l < G->nlev; ++l) {
        if (G->P) orc_crs_free(&G->P[l]);
        if (G->R) orc_crs_free(&G->R[l]);
        if (G->diaginv) free(G->diaginv[l]);
        if (G->diaginv2) free(G->diaginv2[l]);
        if (G->color) free(G->color[l]);
        if (G->sc) { free(G->sc[l]); free(G->sd[l]); free(G->st[l]); }
    }
    if (G->ilu) {
        for (int l = 0; l < G->nlev; ++l) { orc_crs_free(&G->ilu[l]); free(G->ilu_diag[l]); }
        free(G->ilu); free(G->ilu_diag);
    }
    free(G->diaginv2);
    free(G->P); free(G->R); free(G->diaginv); free(G->color); free(G->ncolor);
    free(G->sc); free(G->sd); free(G->st);
    if (G->Arap) {
        /* the top entry is the caller's operator (shallow copy) */
        for (int l = 0; l < G->nlev - 1; ++l) orc_crs_free(&G->Arap[l]);
        free(G->Arap);
    }
    orc_lu_free(&G->lu);
    memset(G, 0, sizeof(*G));
}

/* -------------------------------------------------------------- Krylov -- */
static double vdot(int n, const double *a, const double *b)
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}
static double vnorm(int n, const double *a) { return sqrt(vdot(n, a, a)); }

static int conv_valid(double v)
{
    if (v == 0.0) return 1;
    return (v >= 2.2250738585072014e-308 && v <= 1.7976931348623157e308 && v == v && v >= 0.0);
}

static void conv_start(orc_conv *C, double d)
{
    C->initial_defect = C->final_defect = d;
    C->steps = 0;
    if (C->history && C->hist_cap > 0) C->history[0] = d;
}

static void conv_update(orc_conv *C, double d)
{
    C->final_defect = d;
    C->steps++;
    if (C->history && C->steps < C->hist_cap) C->history[C->steps] = d;
}

static int conv_ended(const orc_conv *C)
{
    if (!conv_valid(C->final_defect)) return 1;
    if (C->steps >= C->maxit) return 1;
    if (C->final_defect < C->min_defect) return 1;
    if (C->final_defect / C->initial_defect < C->rel_red) return 1;
    return 0;
}

static int conv_post(orc_conv *C)
{
    C->converged = (C->final_defect < C->min_defect) || (C->final_defect / C->initial_defect < C->rel_red);
    return C->converged;
}

/* StdConvCheck for callers outside this file (the Newton loop) */
void orc_conv_start(orc_conv *C, double d) { conv_start(C, d); }
void orc_conv_update(orc_conv *C, double d) { conv_update(C, d); }
int orc_conv_ended(const orc_conv *C) { return conv_ended(C); }
int orc_conv_post(orc_conv *C) { return conv_post(C); }
double orc_vnorm(int n, const double *a) { return vnorm(n, a); }

int orc_cg(const orc_crs *A, orc_gmg *M, double *x, double *b, orc_conv *C)
{
    int n = A->n_rows;
    double *r = b;
    orc_crs_matmul_minus(A, r, x);
    double *q = dvec(n), *z = dvec(n), *p = dvec(n);
    if (M) orc_gmg_apply(M, z, r); else memcpy(z, r, sizeof(double) * (size_t)n);
    conv_start(C, vnorm(n, r));
    memcpy(p, z, sizeof(double) * (size_t)n);
    double rhoOld = vdot(n, z, r), rho;
    int ok = 1;
    while (!conv_ended(C)) {
        orc_crs_axpy(A, q, 0.0, q, 1.0, p);
        double lambda = vdot(n, q, p);
        if (lambda == 0.0) { ok = 0; break; }
        const double alpha = rhoOld / lambda;
        for (int i = 0; i < n; ++i) x[i] = 1.0 * x[i] + alpha * p[i];
        for (int i = 0; i < n; ++i) r[i] = 1.0 * r[i] + (-alpha) * q[i];
        conv_update(C, vnorm(n, r));
        if (conv_ended(C)) break;
        if (M) orc_gmg_apply(M, z, r); else memcpy(z, r, sizeof(double) * (size_t)n);
        rho = vdot(n, z, r);
        const double beta = rho / rhoOld;
        for (int i = 0; i < n; ++i) p[i] = beta * p[i] + 1.0 * z[i];
        rhoOld = rho;
    }
    free(q); free(z); free(p);
    return ok ? conv_post(C) : 0;
}

int orc_bicgstab(const orc_crs *A, orc_gmg *M, double *x, double *b, orc_conv *C)
{
    int n = A->n_rows;
    orc_crs_matmul_minus(A, b, x);
    double *r = b;
    double *r0 = dvec(n), *p = dvec(n), *v = dvec(n), *t = dvec(n), *s = dvec(n), *q = dvec(n);
    conv_start(C, vnorm(n, r));
    double rho = 1, alpha = 1, omega = 1, norm_r0 = 0.0;
    int bRestart = 1, ok = 1;
    while (!conv_ended(C)) {
        /* restart by period (bicgstab.h:161-170; the check counts half steps) */
        if (C->restart > 0 && C->steps % C->restart == 0) bRestart = 1;
        if (bRestart) {
            memcpy(r0, r, sizeof(double) * (size_t)n);
            memset(p, 0, sizeof(double) * (size_t)n); alpha = 0.0;
            memset(v, 0, sizeof(double) * (size_t)n); omega = 1.0;
            rho = 1.0;
            norm_r0 = C->final_defect;
            bRestart = 0;
        }
        const double rhoOld = rho;
        rho = vdot(n, r0, r);
        const double norm_r = C->final_defect;
        /* restart in the next iteration when the orthogonality is lost (:206-215) */
        if (fabs(rho) / (norm_r * norm_r0) <= C->min_ortho) bRestart = 1;
        if (rhoOld == 0.0) { ok = 0; break; }
        const double beta = (rho / rhoOld) * (alpha / omega);
        for (int i = 0; i < n; ++i) p[i] = 1.0 * r[i] + beta * p[i] + (-beta * omega) * v[i];
        if (M) orc_gmg_apply(M, q, p); else memcpy(q, p, sizeof(double) * (size_t)n);
        orc_crs_axpy(A, v, 0.0, v, 1.0, q);
        alpha = vdot(n, v, r0);
        if (alpha == 0.0) { ok = 0; break; }
        alpha = rho / alpha;
        for (int i = 0; i < n; ++i) x[i] = 1.0 * x[i] + alpha * q[i];
        for (int i = 0; i < n; ++i) s[i] = 1.0 * r[i] + (-alpha) * v[i];
        conv_update(C, vnorm(n, s));
        if (conv_ended(C)) { memcpy(r, s, sizeof(double) * (size_t)n); break; }
        if (M) orc_gmg_apply(M, q, s); else memcpy(q, s, sizeof(double) * (size_t)n);
        orc_crs_axpy(A, t, 0.0, t, 1.0, q);
        double tt = vdot(n, t, t);
        omega = vdot(n, s, t);
        if (tt == 0.0) { ok = 0; break; }
        omega = omega / tt;
        for (int i = 0; i < n; ++i) x[i] = 1.0 * x[i] + omega * q[i];
        for (int i = 0; i < n; ++i) r[i] = 1.0 * s[i] + (-omega) * t[i];
        conv_update(C, vnorm(n, r));
        if (omega == 0.0) { ok = 0; break; }
    }
    free(r0); free(p); free(v); free(t); free(s); free(q);
    return ok ? conv_post(C) : 0;
}

/* ------------------------------------------------------- coefficients -- */
/* Children of coarse element e on the next finer level (structured split):
   quad -> 4, hex -> 8 (same type); Kuhn tet -> the 8 fine Kuhn tets it
   contains.  Coarse coefficients are the mean of the children's log K
   (geometric mean), applied level by level from the top. */
static void coarsen_logk(const orc_level *F, const orc_level *C, const double *logf, double *logc)
{
    int *cnt = (int *)calloc((size_t)C->ne, sizeof(int));
    memset(logc, 0, sizeof(double) * (size_t)C->ne);
    if (F->nx == 0) {
        /* unstructured hierarchy: the children of coarse element ce are the
           fine elements ce*nchild .. ce*nchild + nchild - 1 */
        const int nchild = (F->dim == 2) ? 4 : 8;
        for (int e = 0; e < F->ne; ++e) {
            logc[e / nchild] += logf[e];
            cnt[e / nchild]++;
        }
        for (int e = 0; e < C->ne; ++e) logc[e] /= (double)(cnt[e] ? cnt[e] : 1);
        free(cnt);
        return;
    }
    int cx = C->nx - 1, cy = C->ny - 1;
    int fx = F->nx - 1, fy = F->ny - 1;
    for (int e = 0; e < F->ne; ++e) {
        int ce;
        if (F->elem_type == ORC_QUAD) {
            int i = e % fx, j = e / fx;
            ce = (i >> 1) + cx * (j >> 1);
        } else if (F->elem_type == ORC_HEX) {
            int i = e % fx, j = (e / fx) % fy, k = e / (fx * fy);
            ce = (i >> 1) + cx * ((j >> 1) + cy * (k >> 1));
        } else {
            /* a fine Kuhn tet lies in the coarse Kuhn tet whose permutation
               orders the fine centroid's offsets inside the coarse hex */
            int h = e / 6;
            int i = h % fx, j = (h / fx) % fy, k = h / (fx * fy);
            double c[3] = {0, 0, 0};
            const int *ev = F->elems + 4 * (size_t)e;
            for (int a = 0; a < 4; ++a)
                for (int d = 0; d < 3; ++d) c[d] += F->coords[3 * (size_t)ev[a] + d];
            double off[3];
            int ci[3] = {i >> 1, j >> 1, k >> 1};
            for (int d = 0; d < 3; ++d) off[d] = c[d] * 0.25 * (double)(C->nx - 1) - (double)ci[d];
            /* Kuhn tet (a,b,c) holds points with off[a] >= off[b] >= off[c] */
            int p;
            if (off[0] >= off[1] && off[1] >= off[2]) p = 0;
            else if (off[0] >= off[2] && off[2] >= off[1]) p = 1;
            else if (off[1] >= off[0] && off[0] >= off[2]) p = 2;
            else if (off[1] >= off[2] && off[2] >= off[0]) p = 3;
            else if (off[2] >= off[0] && off[0] >= off[1]) p = 4;
            else p = 5;
            ce = 6 * (ci[0] + cx * (ci[1] + cy * ci[2])) + p;
        }
        logc[ce] += logf[e];
        cnt[ce]++;
    }
    for (int e = 0; e < C->ne; ++e) logc[e] /= (double)(cnt[e] ? cnt[e] : 1);
    free(cnt);
}

int orc_problem_coefficients(const orc_problem *P, const orc_hier *H, double **Klev)
{
    int top = H->nlev - 1;
    if (P->coef_kind == 0) {
        for (int l = 0; l < H->nlev; ++l) {
            Klev[l] = dvec(H->lev[l].ne);
            for (int e = 0; e < H->lev[l].ne; ++e) Klev[l][e] = 1.0;
        }
        return 0;
    }
    if (P->coef_kind == 1) {
        orc_field F;
        orc_field_scalar_init(&F, H->lev[top].dim, P->coef_modes, P->coef_kmax, P->seed ^ 0xC0EFULL);
        for (int l = 0; l < H->nlev; ++l) {
            const orc_level *L = &H->lev[l];
            double *c = dvec(L->ne * L->dim);
            orc_level_centroids(L, c);
            Klev[l] = dvec(L->ne);
            for (int e = 0; e < L->ne; ++e) Klev[l][e] = exp(2.0 * orc_field_scalar_eval(&F, c + (size_t)e * L->dim));
            free(c);
        }
        orc_field_free(&F);
        return 0;
    }
    /* coef_kind 2: K = exp(m) given on the top level */
    double **logk = (double **)calloc((size_t)H->nlev, sizeof(double *));
    logk[top] = dvec(H->lev[top].ne);
    memcpy(logk[top], P->m_top, sizeof(double) * (size_t)H->lev[top].ne);
    for (int l = top - 1; l >= 0; --l) {
        logk[l] = dvec(H->lev[l].ne);
        coarsen_logk(&H->lev[l + 1], &H->lev[l], logk[l + 1], logk[l]);
    }
    for (int l = 0; l < H->nlev; ++l) {
        Klev[l] = dvec(H->lev[l].ne);
        for (int e = 0; e < H->lev[l].ne; ++e) Klev[l][e] = exp(logk[l][e]);
        free(logk[l]);
    }
    free(logk);
    return 0;
}

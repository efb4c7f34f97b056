/*
 * ug4_oracle_api.c -- oracle: flat problem-level API for the tests (ctypes).
 *
 * TEST INFRASTRUCTURE ONLY (see ug4_oracle.h).
 *
 * A "problem" bundles what a ugcore Lua script sets up for this path
 * (util.solver.SolveLinearProblem, scripts/util/solver_util.lua:1182):
 * domain hierarchy, DomainDiscretization with the FV1 convection-diffusion
 * element disc and a zero DirichletBoundary, assemble_linear on the top
 * level, GMG (re-assembled level operators, StdTransfer, Jacobi/GS, LU base),
 * and a CG or BiCGStab solve from x = 0 with StdConvCheck.
 * The adjoint part (no reference counterpart) solves A^T lambda = g with the
 * same GMG on the transposed level operators (Dirichlet rows reset to
 * identity) and forms dJ/d(log K) per element and dJ/d(f) per vertex.
 */
#include "ug4_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

int orc_grad_logk(const orc_level *L, const double *K, const double *u, const double *lam, double *g);

/* orc_params: ug4_oracle.h */

struct orc_prob {
    orc_params p;
    orc_hier H;
    double **K;          /* per level per element */
    orc_field vf;
    int has_vf;
    double *f;           /* top-level source */
    orc_crs *A;          /* per level */
    double *b;           /* top rhs */
    orc_gmg G;
    int gmg_ready;
    orc_crs *AT;         /* transposed level operators (adjoint) */
    orc_gmg GT;
    int gmgT_ready;
};

static int assemble_all(orc_prob *P)
{
    int nl = P->H.nlev, top = nl - 1;
    P->A = (orc_crs *)calloc((size_t)nl, sizeof(orc_crs));
    P->b = (double *)calloc((size_t)P->H.lev[top].nv, sizeof(double));
    for (int l = 0; l < nl; ++l) {
        orc_disc D;
        memset(&D, 0, sizeof(D));
        D.K = P->K[l];
        D.upwind = P->has_vf ? 1 : 0;
        D.vfield = P->has_vf ? &P->vf : NULL;
        D.f = (l == top) ? P->f : NULL;
        D.dirichlet = 1;
        if (orc_assemble(&P->H.lev[l], &D, &P->A[l], (l == top) ? P->b : NULL)) return -1;
    }
    return 0;
}

static orc_prob *prob_setup(orc_prob *P, const orc_params *p, const double *m_top, const double *f_top);

orc_prob *orc_prob_create(const orc_params *p, const double *m_top, const double *f_top)
{
    orc_prob *P = (orc_prob *)calloc(1, sizeof(orc_prob));
    if (!P) return NULL;
    P->p = *p;
    if (orc_hier_create(&P->H, p->elem_type, p->mx, p->my, p->mz, p->nref)) { free(P); return NULL; }
    return prob_setup(P, p, m_top, f_top);
}

/* problem on a given hierarchy (unstructured grids): no velocity field;
   coefficient kind 2 takes m_top (coarse m = mean of the children) */
orc_prob *orc_prob_create_ext(const orc_params *p, int nlev, const int *nv, const int *ne,
                              const double *const *coords, const int *const *elems,
                              const unsigned char *const *bnd, const int *const *npar, const int *const *par,
                              const double *m_top, const double *f_top)
{
    if ((p->coef_kind == 2 && !m_top) || p->vel_kind != 0) return NULL;
    orc_prob *P = (orc_prob *)calloc(1, sizeof(orc_prob));
    if (!P) return NULL;
    P->p = *p;
    if (orc_hier_from_arrays(&P->H, p->elem_type, nlev, nv, ne, coords, elems, bnd, npar, par)) {
        free(P);
        return NULL;
    }
    return prob_setup(P, p, m_top, f_top);
}

static orc_prob *prob_setup(orc_prob *P, const orc_params *p, const double *m_top, const double *f_top)
{
    int nl = P->H.nlev, top = nl - 1;
    P->K = (double **)calloc((size_t)nl, sizeof(double *));
    if (p->coef_kind == 3) {
        for (int l = 0; l < nl; ++l) {
            P->K[l] = (double *)malloc(sizeof(double) * (size_t)P->H.lev[l].ne);
            for (int e = 0; e < P->H.lev[l].ne; ++e) P->K[l][e] = p->diffusion;
        }
    } else {
        orc_problem pr;
        memset(&pr, 0, sizeof(pr));
        pr.seed = p->seed; pr.coef_kind = p->coef_kind; pr.coef_modes = p->coef_modes;
        pr.coef_kmax = p->coef_kmax; pr.m_top = m_top;
        orc_problem_coefficients(&pr, &P->H, P->K);
    }
    if (p->vel_kind == 1) {
        orc_field_curl_init(&P->vf, p->vel_modes, p->vel_kmax, p->seed ^ 0x7E10C17ULL);
        P->vf.scale *= p->peclet * 2.0 * p->diffusion * (double)(P->H.lev[top].nx - 1);
        P->has_vf = 1;
    }
    int nv = P->H.lev[top].nv;
    P->f = (double *)malloc(sizeof(double) * (size_t)nv);
    if (f_top) memcpy(P->f, f_top, sizeof(double) * (size_t)nv);
    else orc_source_uniform(p->seed, nv, P->f);
    if (assemble_all(P)) return NULL;
    return P;
}

int orc_prob_num_levels(const orc_prob *P) { return P->H.nlev; }
int orc_prob_level_nv(const orc_prob *P, int l) { return P->H.lev[l].nv; }
int orc_prob_level_ne(const orc_prob *P, int l) { return P->H.lev[l].ne; }
int64_t orc_prob_level_nnz(const orc_prob *P, int l) { return P->A[l].nnz; }

static void crs_out(const orc_crs *A, int *rowptr, int *col, double *val)
{
    if (rowptr) memcpy(rowptr, A->rowptr, sizeof(int) * ((size_t)A->n_rows + 1));
    if (col) memcpy(col, A->col, sizeof(int) * (size_t)A->nnz);
    if (val) memcpy(val, A->val, sizeof(double) * (size_t)A->nnz);
}

void orc_prob_level_matrix(const orc_prob *P, int l, int *rowptr, int *col, double *val)
{
    crs_out(&P->A[l], rowptr, col, val);
}

void orc_prob_level_coef(const orc_prob *P, int l, double *K)
{
    memcpy(K, P->K[l], sizeof(double) * (size_t)P->H.lev[l].ne);
}

void orc_prob_level_elems(const orc_prob *P, int l, int *elems, double *coords, unsigned char *bnd)
{
    const orc_level *L = &P->H.lev[l];
    if (elems) memcpy(elems, L->elems, sizeof(int) * (size_t)L->ne * L->k);
    if (coords) memcpy(coords, L->coords, sizeof(double) * (size_t)L->nv * L->dim);
    if (bnd) memcpy(bnd, L->bnd, (size_t)L->nv);
}

void orc_prob_rhs(const orc_prob *P, double *b)
{
    memcpy(b, P->b, sizeof(double) * (size_t)P->H.lev[P->H.nlev - 1].nv);
}

void orc_prob_source(const orc_prob *P, double *f)
{
    memcpy(f, P->f, sizeof(double) * (size_t)P->H.lev[P->H.nlev - 1].nv);
}

/* orc_gmg_init with the problem's smoother, cycle and transfer damping */
static int gmg_init_p(orc_gmg *G, const orc_prob *P, orc_crs *levA)
{
    const orc_params *p = &P->p;
    int rc = orc_gmg_init_ex(G, &P->H, levA, p->smoother, p->damp, p->nu1, p->nu2, p->cycle, p->base, p->rap,
                             p->base_steps);
    if (rc) return rc;
    if (p->post_smoother >= 0) {
        rc = orc_gmg_set_postsmoother(G, p->post_smoother, p->post_damp);
        if (rc) return rc;
    }
    G->damp_prol = p->damp_prol > 0.0 ? p->damp_prol : 1.0;
    G->damp_res = p->damp_res > 0.0 ? p->damp_res : 1.0;
    return 0;
}

static int ensure_gmg(orc_prob *P)
{
    if (P->gmg_ready) return 0;
    int rc = gmg_init_p(&P->G, P, P->A);
    if (rc) return rc;
    P->gmg_ready = 1;
    return 0;
}

/* the multigrid's operator of level l (re-assembled, or R A P with rap) */
int64_t orc_prob_gmg_level_nnz(orc_prob *P, int l)
{
    if (ensure_gmg(P)) return -1;
    return P->G.A[l].nnz;
}

void orc_prob_gmg_level(orc_prob *P, int l, int *rowptr, int *col, double *val)
{
    if (ensure_gmg(P)) return;
    crs_out(&P->G.A[l], rowptr, col, val);
}

int64_t orc_prob_transfer_nnz(orc_prob *P, int l, int which)
{
    if (ensure_gmg(P)) return -1;
    return which ? P->G.R[l].nnz : P->G.P[l].nnz;
}

void orc_prob_transfer(orc_prob *P, int l, int which, int *rowptr, int *col, double *val)
{
    if (ensure_gmg(P)) return;
    crs_out(which ? &P->G.R[l] : &P->G.P[l], rowptr, col, val);
}

int orc_prob_apply_gmg(orc_prob *P, double *c, const double *d)
{
    if (ensure_gmg(P)) return -1;
    orc_gmg_apply(&P->G, c, d);
    return 0;
}

static int run_solver(const orc_params *p, const orc_crs *A, orc_gmg *G, double *x, double *rhs,
                      int *steps, double *d0, double *d1, double *hist, int hist_cap)
{
    orc_conv C;
    memset(&C, 0, sizeof(C));
    C.maxit = p->maxit; C.min_defect = p->min_defect; C.rel_red = p->rel_red;
    C.history = hist; C.hist_cap = hist_cap;
    C.restart = p->bicg_restart; C.min_ortho = p->bicg_min_ortho;
    int ok = (p->solver == 0) ? orc_cg(A, G, x, rhs, &C) : orc_bicgstab(A, G, x, rhs, &C);
    if (steps) *steps = C.steps;
    if (d0) *d0 = C.initial_defect;
    if (d1) *d1 = C.final_defect;
    return ok ? 0 : 1;
}

/* forward solve from x = 0; returns 0 if converged */
int orc_prob_solve(orc_prob *P, double *x, int *steps, double *d0, double *d1, double *hist, int hist_cap)
{
    if (ensure_gmg(P)) return -1;
    int top = P->H.nlev - 1, nv = P->H.lev[top].nv;
    double *rhs = (double *)malloc(sizeof(double) * (size_t)nv);
    memcpy(rhs, P->b, sizeof(double) * (size_t)nv);
    memset(x, 0, sizeof(double) * (size_t)nv);
    int rc = run_solver(&P->p, &P->A[top], &P->G, x, rhs, steps, d0, d1, hist, hist_cap);
    free(rhs);
    return rc;
}

/* ---- ThetaTimeStep ------------------------------------------------------ */
/* the time-discrete operator of level l (sm0 M + sa0 A) and, with b, the
   right-hand side of one step from u_old (top level) for the time scalings
   vScaleMass = (sm0, sm1), vScaleStiff = (sa0, sa1) a multi-step
   discretisation passes to the domain discretisation
   (IDomainDiscretization::assemble_linear, domain_disc_interface.h) */
static int scaled_assemble(const orc_prob *P, int l, double sm0, double sa0, double sm1, double sa1,
                           const double *u_old, orc_crs *A, double *b)
{
    const int top = P->H.nlev - 1;
    orc_disc D;
    memset(&D, 0, sizeof(D));
    D.K = P->K[l];
    D.upwind = P->has_vf ? 1 : 0;
    D.vfield = P->has_vf ? &P->vf : NULL;
    D.f = (l == top) ? P->f : NULL;
    D.dirichlet = 1;
    D.inst = 1;
    D.sm0 = sm0; D.sa0 = sa0; D.sm1 = sm1; D.sa1 = sa1;
    D.u_old = u_old;
    return orc_assemble(&P->H.lev[l], &D, A, b);
}

/* the theta step's scalings (ThetaTimeStep::update_scaling,
   theta_time_step.h): s_m = (1, -1), s_a = (theta dt, (1 - theta) dt) */
static int theta_assemble(const orc_prob *P, int l, double theta, double dt, const double *u_old, orc_crs *A,
                          double *b)
{
    return scaled_assemble(P, l, 1.0, theta * dt, -1.0, (1.0 - theta) * dt, u_old, A, b);
}

int orc_prob_scaled_system(const orc_prob *P, double sm0, double sa0, double sm1, double sa1, const double *u_old,
                           int *rowptr, int *col, double *val, double *b)
{
    orc_crs A;
    memset(&A, 0, sizeof(A));
    if (scaled_assemble(P, P->H.nlev - 1, sm0, sa0, sm1, sa1, u_old, &A, b)) return -1;
    crs_out(&A, rowptr, col, val);
    orc_crs_free(&A);
    return 0;
}

/* top-level time-discrete system of one step (CRS pattern = the level's) */
int orc_prob_theta_system(const orc_prob *P, double theta, double dt, const double *u_old, int *rowptr, int *col,
                          double *val, double *b)
{
    orc_crs A;
    memset(&A, 0, sizeof(A));
    if (theta_assemble(P, P->H.nlev - 1, theta, dt, u_old, &A, b)) return -1;
    crs_out(&A, rowptr, col, val);
    orc_crs_free(&A);
    return 0;
}

/* the time-discrete operator M + theta dt A of level l (the jacobian the
   coarse multigrid levels are assembled with) */
int orc_prob_theta_jacobian(const orc_prob *P, int l, double theta, double dt, int *rowptr, int *col, double *val)
{
    orc_crs A;
    memset(&A, 0, sizeof(A));
    if (l < 0 || l >= P->H.nlev || theta_assemble(P, l, theta, dt, NULL, &A, NULL)) return -1;
    crs_out(&A, rowptr, col, val);
    orc_crs_free(&A);
    return 0;
}

/* nsteps theta steps of constant size dt from u (in/out), as ugcore's
   SolveLinearTimeProblem (scripts/util/time_step_util.lua:643-870): the
   matrix and the multigrid (coarse levels: the time-discrete jacobians) are
   set up once for the step size, every step assembles its right-hand side
   from the previous solution and applies the solver with the previous
   solution as the initial guess.  steps[s] = iterations of step s. */
int orc_prob_theta_steps(orc_prob *P, double theta, double dt, int nsteps, double *u, int *steps)
{
    const int nl = P->H.nlev, top = nl - 1, nv = P->H.lev[top].nv;
    orc_crs *At = (orc_crs *)calloc((size_t)nl, sizeof(orc_crs));
    double *b = (double *)malloc(sizeof(double) * (size_t)nv);
    double *u_old = (double *)malloc(sizeof(double) * (size_t)nv);
    if (!At || !b || !u_old) return -1;
    int rc = 0;
    orc_gmg G;
    memset(&G, 0, sizeof(G));
    for (int l = 0; l < top; ++l)
        if (theta_assemble(P, l, theta, dt, NULL, &At[l], NULL)) return -1;
    for (int s = 0; s < nsteps && rc == 0; ++s) {
        memcpy(u_old, u, sizeof(double) * (size_t)nv);
        if (s == 0) {
            if (theta_assemble(P, top, theta, dt, u_old, &At[top], b)) return -1;
            if (gmg_init_p(&G, P, At)) return -2;
        } else {
            orc_crs T;
            memset(&T, 0, sizeof(T));
            if (theta_assemble(P, top, theta, dt, u_old, &T, b)) return -1;
            orc_crs_free(&T);
        }
        int st = 0;
        rc = run_solver(&P->p, &At[top], &G, u, b, &st, NULL, NULL, NULL, 0);
        if (steps) steps[s] = st;
    }
    orc_gmg_free(&G);
    for (int l = 0; l < nl; ++l) orc_crs_free(&At[l]);
    free(At); free(b); free(u_old);
    return rc;
}

/* ---- defect and Newton ----------------------------------------------- */
static void prob_disc(const orc_prob *P, int l, orc_disc *D)
{
    memset(D, 0, sizeof(*D));
    D->K = P->K[l];
    D->upwind = P->has_vf ? 1 : 0;
    D->vfield = P->has_vf ? &P->vf : NULL;
    D->f = (l == P->H.nlev - 1) ? P->f : NULL;
    D->dirichlet = 1;
}

/* top-level defect of u: stationary (theta < 0) or of one theta step from
   u_old (ThetaTimeStep::assemble_defect, s_m = (1, -1),
   s_a = (theta dt, (1 - theta) dt)) */
/* the time-discrete defect of u for the scalings s_m = (sm0, sm1),
   s_a = (sa0, sa1) from u_old (IDomainDiscretization::assemble_defect) */
int orc_prob_scaled_defect(const orc_prob *P, double sm0, double sa0, double sm1, double sa1, const double *u_old,
                           const double *u, double *d)
{
    const int top = P->H.nlev - 1;
    orc_disc D;
    prob_disc(P, top, &D);
    if (!u_old) return -1;
    D.inst = 1;
    D.sm0 = sm0; D.sa0 = sa0; D.sm1 = sm1; D.sa1 = sa1;
    D.u_old = u_old;
    return orc_assemble_defect(&P->H.lev[top], &D, u, d);
}

int orc_prob_defect(const orc_prob *P, double theta, double dt, const double *u_old, const double *u, double *d)
{
    const int top = P->H.nlev - 1;
    if (theta >= 0.0) return orc_prob_scaled_defect(P, 1.0, theta * dt, -1.0, (1.0 - theta) * dt, u_old, u, d);
    orc_disc D;
    prob_disc(P, top, &D);
    return orc_assemble_defect(&P->H.lev[top], &D, u, d);
}

/* parameters of StandardLineSearch (its setters) */
typedef struct {
    int max_steps;              /* <= 64 */
    double lambda_start, lambda_reduce, alpha, max_defect;
    int accept_best, check_all;
} orc_line_search;

/* StandardLineSearch::search (lib_disc/operator/non_linear_operator/
   line_search.h:186-400) along the correction c from s = u with the start
   defect norm norm_old: tries u = u - lambda c (lambda = start, start*reduce,
   ...), accepting the first with |N(u)| / norm_old <= 1 - alpha |lambda|
   (all max_steps tries with check_all); after max_steps tries, with
   accept_best, u = s - start reduce^best c for the first smallest ratio,
   failing when its defect exceeds max_defect; without accept_best it fails.
   d = N(u) on return.  Returns 0, or 3 when the search failed. */
static int line_search(orc_prob *P, double theta, double dt, const double *u_old, const orc_level *L,
                       const orc_line_search *LS, double *u, const double *c, double *d, double *s, double norm_old,
                       double *norm, int *tries, double *lambda_out)
{
    const int nv = L->nv;
    double lambda = LS->lambda_start, nrm = 0.0;
    double rho[64];
    memcpy(s, u, sizeof(double) * (size_t)nv);
    for (int k = 1; k <= LS->max_steps; ++k) {
        for (int i = 0; i < nv; ++i) u[i] = 1.0 * u[i] + (-lambda) * c[i];
        for (int i = 0; i < nv; ++i) if (L->bnd[i]) u[i] = 0.0;      /* prepare */
        if (orc_prob_defect(P, theta, dt, u_old, u, d)) return -1;
        nrm = orc_vnorm(nv, d);
        *tries = k;
        *lambda_out = lambda;
        rho[k - 1] = nrm / norm_old;
        if (rho[k - 1] <= 1.0 - LS->alpha * fabs(lambda) && !LS->check_all) break;
        lambda *= LS->lambda_reduce;
        if (k == LS->max_steps) {
            if (!LS->accept_best) return 3;
            int best = 0;
            for (int i = 1; i < k; ++i)
                if (rho[best] > rho[i]) best = i;
            const double lb = LS->lambda_start * pow(LS->lambda_reduce, (double)best);
            *lambda_out = lb;
            for (int i = 0; i < nv; ++i) u[i] = 1.0 * s[i] + (-lb) * c[i];
            for (int i = 0; i < nv; ++i) if (L->bnd[i]) u[i] = 0.0;
            if (orc_prob_defect(P, theta, dt, u_old, u, d)) return -1;
            nrm = orc_vnorm(nv, d);
            if (nrm > LS->max_defect) return 3;
            break;
        }
        memcpy(u, s, sizeof(double) * (size_t)nv);
    }
    *norm = nrm;
    return 0;
}

/* The linear solver's multigrid for a Newton step: the jacobian of every
   level (stationary, theta < 0, or the theta step's M + theta dt A; the FV1
   operator is linear, so it does not depend on u) and the problem's GMG on
   them.  J: nlev matrices, owned by the caller (orc_prob_newton_gmg_free). */
int orc_prob_newton_gmg(orc_prob *P, double theta, double dt, orc_gmg *G, orc_crs *J)
{
    const int nl = P->H.nlev;
    for (int l = 0; l < nl; ++l) {
        orc_crs_free(&J[l]);
        orc_disc D;
        prob_disc(P, l, &D);
        D.f = NULL;
        if (theta >= 0.0) {
            D.inst = 1;
            D.sm0 = 1.0; D.sa0 = theta * dt; D.sm1 = 0.0; D.sa1 = 0.0;
        }
        if (orc_assemble(&P->H.lev[l], &D, &J[l], NULL)) return -1;
    }
    memset(G, 0, sizeof(*G));
    return gmg_init_p(G, P, J) ? -2 : 0;
}

void orc_prob_newton_gmg_free(orc_prob *P, orc_gmg *G, orc_crs *J)
{
    orc_gmg_free(G);
    for (int l = 0; l < P->H.nlev; ++l) orc_crs_free(&J[l]);
}

/* NewtonSolver::apply (newton_impl.h:171-340) with the problem's
   GMG-preconditioned Krylov solver as the linear solver (its own convergence
   parameters) on the stationary operator (theta < 0) or the theta step from
   u_old, without (LS NULL) or with StandardLineSearch.  u in/out.  Returns 0
   if Newton converged, 1 if not, 2 if a linear solve failed, 3 if a line
   search failed, < 0 on set-up errors.  steps: Newton steps; lin_steps[s],
   defects[s] (s <= maxit, defects[0] the start defect); ls_tries[s],
   ls_lambda[s] per step with a line search. */
int orc_prob_newton_ls(orc_prob *P, double theta, double dt, const double *u_old, double *u, int maxit,
                       double min_defect, double reduction, const orc_line_search *LS, int *steps, int *lin_steps,
                       double *defects, int *ls_tries, double *ls_lambda)
{
    const int nl = P->H.nlev, top = nl - 1, nv = P->H.lev[top].nv;
    const orc_level *L = &P->H.lev[top];
    double *d = (double *)malloc(sizeof(double) * (size_t)nv);
    double *c = (double *)malloc(sizeof(double) * (size_t)nv);
    double *rhs = (double *)malloc(sizeof(double) * (size_t)nv);
    double *s = (double *)malloc(sizeof(double) * (size_t)nv);
    orc_crs *J = (orc_crs *)calloc((size_t)nl, sizeof(orc_crs));
    if (!d || !c || !rhs || !s || !J) return -1;
    if (LS && (LS->max_steps < 1 || LS->max_steps > 64)) return -1;
    int rc = 0;
    orc_conv NC;
    memset(&NC, 0, sizeof(NC));
    NC.maxit = maxit; NC.min_defect = min_defect; NC.rel_red = reduction;
    for (int i = 0; i < nv; ++i) if (L->bnd[i]) u[i] = 0.0;          /* prepare */
    if (orc_prob_defect(P, theta, dt, u_old, u, d)) return -1;
    orc_conv_start(&NC, orc_vnorm(nv, d));
    if (defects) defects[0] = NC.initial_defect;
    while (!orc_conv_ended(&NC)) {
        memset(c, 0, sizeof(double) * (size_t)nv);
        /* jacobian of every level (the linear solver's multigrid is set up with it) */
        orc_gmg G;
        const int grc = orc_prob_newton_gmg(P, theta, dt, &G, J);
        if (grc) return grc;
        const orc_params *p = &P->p;
        memcpy(rhs, d, sizeof(double) * (size_t)nv);
        int ls = 0;
        const int lrc = run_solver(p, &J[top], &G, c, rhs, &ls, NULL, NULL, NULL, 0);
        orc_gmg_free(&G);
        if (lin_steps) lin_steps[NC.steps] = ls;
        if (lrc) { rc = 2; break; }
        double nd = 0.0;
        if (LS) {
            int tr = 0;
            double lam = 0.0;
            const int src = line_search(P, theta, dt, u_old, L, LS, u, c, d, s, NC.final_defect, &nd, &tr, &lam);
            if (ls_tries) ls_tries[NC.steps] = tr;
            if (ls_lambda) ls_lambda[NC.steps] = lam;
            if (src < 0) return -1;
            if (src) { rc = 3; break; }
        } else {
            for (int i = 0; i < nv; ++i) u[i] -= c[i];
            for (int i = 0; i < nv; ++i) if (L->bnd[i]) u[i] = 0.0;      /* prepare */
            if (orc_prob_defect(P, theta, dt, u_old, u, d)) return -1;
            nd = orc_vnorm(nv, d);
        }
        orc_conv_update(&NC, nd);
        if (defects) defects[NC.steps] = NC.final_defect;
    }
    if (rc == 0) rc = orc_conv_post(&NC) ? 0 : 1;
    if (steps) *steps = NC.steps;
    for (int l = 0; l < nl; ++l) orc_crs_free(&J[l]);
    free(J); free(d); free(c); free(rhs); free(s);
    return rc;
}

int orc_prob_newton(orc_prob *P, double theta, double dt, const double *u_old, double *u, int maxit,
                    double min_defect, double reduction, int *steps, int *lin_steps, double *defects)
{
    return orc_prob_newton_ls(P, theta, dt, u_old, u, maxit, min_defect, reduction, NULL, steps, lin_steps, defects,
                              NULL, NULL);
}

/* transposed operator with Dirichlet rows reset to identity */
static int transpose_dirichlet(const orc_crs *A, const orc_level *L, orc_crs *T)
{
    if (orc_crs_transpose(A, 1, T)) return -1;
    for (int v = 0; v < L->nv; ++v) {
        if (!L->bnd[v]) continue;
        for (int a = T->rowptr[v]; a < T->rowptr[v + 1]; ++a) T->val[a] = 0.0;
        T->val[orc_crs_find(T, v, v)] = 1.0;
    }
    return 0;
}

int orc_prob_adjoint(orc_prob *P, const double *g, double *lam, int *steps, double *d0, double *d1)
{
    int nl = P->H.nlev, top = nl - 1, nv = P->H.lev[top].nv;
    if (!P->gmgT_ready) {
        P->AT = (orc_crs *)calloc((size_t)nl, sizeof(orc_crs));
        for (int l = 0; l < nl; ++l)
            if (transpose_dirichlet(&P->A[l], &P->H.lev[l], &P->AT[l])) return -1;
        int rc = gmg_init_p(&P->GT, P, P->AT);
        if (rc) return rc;
        P->gmgT_ready = 1;
    }
    double *rhs = (double *)malloc(sizeof(double) * (size_t)nv);
    for (int i = 0; i < nv; ++i) rhs[i] = P->H.lev[top].bnd[i] ? 0.0 : g[i];
    memset(lam, 0, sizeof(double) * (size_t)nv);
    int rc = run_solver(&P->p, &P->AT[top], &P->GT, lam, rhs, steps, d0, d1, NULL, 0);
    free(rhs);
    return rc;
}

void orc_prob_grad_logk(const orc_prob *P, const double *u, const double *lam, double *grad)
{
    int top = P->H.nlev - 1;
    orc_grad_logk(&P->H.lev[top], P->K[top], u, lam, grad);
}

void orc_prob_grad_source(const orc_prob *P, const double *lam, double *grad)
{
    int top = P->H.nlev - 1;
    const orc_level *L = &P->H.lev[top];
    orc_scv_volume_sum(L, grad);
    for (int i = 0; i < L->nv; ++i) grad[i] = L->bnd[i] ? 0.0 : grad[i] * lam[i];
}

void orc_prob_free(orc_prob *P)
{
    if (!P) return;
    int nl = P->H.nlev;
    if (P->gmg_ready) orc_gmg_free(&P->G);
    if (P->gmgT_ready) orc_gmg_free(&P->GT);
    for (int l = 0; l < nl; ++l) {
        if (P->A) orc_crs_free(&P->A[l]);
        if (P->AT) orc_crs_free(&P->AT[l]);
        if (P->K) free(P->K[l]);
    }
    free(P->A); free(P->AT); free(P->K); free(P->b); free(P->f);
    if (P->has_vf) orc_field_free(&P->vf);
    orc_hier_free(&P->H);
    free(P);
}

/* standalone transpose on caller CRS arrays (pins set_as_transpose_of[2]) */
int64_t orc_transpose_nnz(int n_rows, int n_cols, const int *rowptr, const int *col, const double *val,
                          int keep_zeros)
{
    orc_crs B = {n_rows, n_cols, rowptr[n_rows], (int *)rowptr, (int *)col, (double *)val};
    orc_crs T;
    if (orc_crs_transpose(&B, keep_zeros, &T)) return -1;
    int64_t nnz = T.nnz;
    orc_crs_free(&T);
    return nnz;
}

/* parameters of the seeded fields (kind 0 scalar, 1 curl); for the tests that
   pin the product's host-side generator to the oracle's */
int orc_field_params(int kind, int dim, int nmodes, double kmax, uint64_t seed, double *k, double *phase, double *c,
                     double *amp_scale)
{
    orc_field F;
    if (kind == 0) orc_field_scalar_init(&F, dim, nmodes, kmax, seed);
    else orc_field_curl_init(&F, nmodes, kmax, seed);
    memcpy(k, F.k, sizeof(double) * (size_t)nmodes * F.dim);
    memcpy(phase, F.phase, sizeof(double) * (size_t)nmodes);
    if (kind == 1) memcpy(c, F.a, sizeof(double) * (size_t)nmodes * 3);
    *amp_scale = (kind == 0) ? F.amp : F.scale;
    orc_field_free(&F);
    return 0;
}

/* FV1 geometry of one element (for geometry unit tests) */
int orc_geometry(int elem_type, const double *corner, double *normals, double *vols, double *grads,
                 int *from, int *to, double *ips)
{
    orc_fv1geom G;
    orc_fv1_geometry(elem_type, corner, &G);
    int dim = (elem_type == ORC_QUAD || elem_type == ORC_TRI) ? 2 : 3;
    for (int i = 0; i < G.nscvf; ++i) {
        from[i] = G.from[i]; to[i] = G.to[i];
        for (int d = 0; d < dim; ++d) normals[i * dim + d] = G.normal[i][d];
        if (ips)
            for (int d = 0; d < dim; ++d) ips[i * dim + d] = G.gip[i][d];
        for (int s = 0; s < G.nscv; ++s)
            for (int d = 0; d < dim; ++d) grads[(i * G.nscv + s) * dim + d] = G.grad[i][s][d];
    }
    for (int s = 0; s < G.nscv; ++s) vols[s] = G.vol[s];
    return G.nscvf;
}

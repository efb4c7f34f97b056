/*
 * ug4_oracle.h -- CPU restatement of UG4/ugcore's assemble-and-solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * GB300 kernels in ugcore_gb300/csrc.  Only tests/, __graft_entry__.smoke()
 * and the CPU-baseline legs of bench.py may load it; the product path never
 * does.  Every routine cites the reference file:line whose behaviour it
 * restates (paths relative to the ugcore source tree, ugbase/...).
 *
 * Scope (all FP64, single-threaded like the reference hot path):
 *   - structured grid hierarchies (quad 2D, hex 3D, Kuhn 6-tet 3D) with
 *     lexicographic DoF numbering and parent tables;
 *   - FV1 (box-method) element assembly of -div(K grad u) + div(v u) = f with
 *     full upwind, Dirichlet rows kept in the pattern;
 *   - StdTransfer P1 prolongation, R = P^T, Dirichlet adjustment of both;
 *   - damped Jacobi, multicolour Gauss-Seidel, dense pivoted LU;
 *   - AssembledMultiGridCycle V/W cycle, CG and BiCGStab with StdConvCheck;
 *   - the discrete adjoint (transposed solve, element/vertex gradients).
 */
#ifndef UG4_ORACLE_H
#define UG4_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_QUAD = 0, ORC_HEX = 1, ORC_TET = 2, ORC_TRI = 3 };

typedef struct {
    int n_rows, n_cols;
    int64_t nnz;
    int *rowptr;   /* n_rows + 1 */
    int *col;      /* nnz, sorted per row */
    double *val;   /* nnz */
} orc_crs;

typedef struct {
    int elem_type, dim, k;      /* k = corners per element */
    int nx, ny, nz;             /* vertices per axis (nz = 1 in 2D) */
    int nv, ne;
    double *coords;             /* nv * dim */
    int *elems;                 /* ne * k, corners in reference order */
    unsigned char *bnd;         /* nv: 1 = Dirichlet boundary vertex */
    int *npar;                  /* nv: number of coarse parents (level > 0) */
    int *par;                   /* nv * 8: coarse parent vertex ids, sorted */
} orc_level;

typedef struct {
    int nlev;
    orc_level *lev;
} orc_hier;

/* random fields (seeded, counter-based) */
typedef struct {
    int nmodes;
    int dim;
    double amp;          /* sqrt(2/nmodes) * sigma */
    double *k;           /* nmodes * dim wavevectors */
    double *phase;       /* nmodes */
    double *a;           /* nmodes * 3 vector amplitudes (curl field only) */
    double scale;        /* post-scale (curl field) */
} orc_field;

uint64_t orc_splitmix64(uint64_t *state);
double orc_hash_uniform(uint64_t seed, uint64_t i);   /* U[0,1) from (seed,i) */
void orc_source_uniform(uint64_t seed, int n, double *f); /* U[-1,1] */

int orc_field_scalar_init(orc_field *F, int dim, int nmodes, double kmax, uint64_t seed);
int orc_field_curl_init(orc_field *F, int nmodes, double kmax, uint64_t seed);
double orc_field_scalar_eval(const orc_field *F, const double *x);
void orc_field_curl_eval(const orc_field *F, const double *x, double *v);
void orc_field_free(orc_field *F);

/* hierarchy */
int orc_hier_create(orc_hier *H, int elem_type, int mx, int my, int mz, int nref);
void orc_hier_free(orc_hier *H);
int orc_hier_from_arrays(orc_hier *H, int elem_type, int nlev, const int *nv, const int *ne,
                         const double *const *coords, const int *const *elems, const unsigned char *const *bnd,
                         const int *const *npar, const int *const *par);
void orc_level_centroids(const orc_level *L, double *c);

/* CRS */
void orc_crs_free(orc_crs *A);
int orc_crs_pattern_from_elems(const orc_level *L, orc_crs *A);
int orc_crs_transpose(const orc_crs *B, int keep_zeros, orc_crs *T);
void orc_crs_axpy(const orc_crs *A, double *dest, double alpha1, const double *v1,
                  double beta1, const double *w1);
void orc_crs_matmul_minus(const orc_crs *A, double *res, const double *x);
void orc_crs_apply_ignore_zero_rows(const orc_crs *A, double *dest, double beta, const double *w);
int orc_crs_find(const orc_crs *A, int r, int c);

/* FV1 element geometry (one element, arbitrary corner coords) */
typedef struct {
    int nscv, nscvf;
    int from[12], to[12];
    double normal[12][3];
    double gip[12][3];       /* global SCVF integration points */
    double grad[12][8][3];   /* global shape gradients at SCVF ips */
    double vol[8];           /* SCV volumes */
} orc_fv1geom;

int orc_fv1_geometry(int elem_type, const double *corner, orc_fv1geom *G);

/* assembly: K per element (NULL = 1), vel per element per scvf ip (NULL = 0)
   or velocity field F (if vel == NULL and F != NULL), f per vertex (NULL = 0). */
typedef struct {
    const double *K;         /* ne */
    const double *vel;       /* ne * nscvf * dim */
    const orc_field *vfield; /* evaluated at scvf ips if vel == NULL */
    const double *f;         /* nv */
    int upwind;              /* 0 = none (no convection), 1 = full upwind */
    int dirichlet;           /* 1 = zero Dirichlet on the boundary */
    /* instationary (ThetaTimeStep): element matrix sm0 M_e + sa0 A_e with the
       lumped mass M_e = diag(|SCV_i|); rhs sa0 f_e - sm1 M_e u_old
       - sa1 A_e u_old + sa1 f_e (elem_disc_assemble_util.h:1124-1205) */
    int inst;
    double sm0, sa0, sm1, sa1;
    const double *u_old;     /* nv (top level), for the rhs */
} orc_disc;

int orc_assemble(const orc_level *L, const orc_disc *D, orc_crs *A, double *b);
int orc_assemble_defect(const orc_level *L, const orc_disc *D, const double *u, double *d);
void orc_scv_volume_sum(const orc_level *L, double *vol);
int orc_element_matrix(const orc_level *L, int e, double K, const orc_field *vf, int upwind,
                       double *Aloc, double *vol);
int orc_grad_logk(const orc_level *L, const double *K, const double *u, const double *lam, double *g);

/* transfers */
int orc_prolongation(const orc_level *fine, const orc_level *coarse, orc_crs *P);
int orc_restriction(const orc_level *fine, const orc_level *coarse, const orc_crs *P, orc_crs *R);

/* dense LU (no-LAPACK path) */
typedef struct { int n; double *LU; int *piv; } orc_lu;
int orc_lu_init(orc_lu *F, const orc_crs *A);
void orc_lu_apply(const orc_lu *F, double *x, const double *b);
void orc_lu_free(orc_lu *F);

/* GMG */
/* MCBGS: backward Gauss-Seidel (BackwardGaussSeidel, gauss_seidel.h:316),
   colours in decreasing order */
enum { ORC_SMOOTH_JACOBI = 0, ORC_SMOOTH_MCGS = 1, ORC_SMOOTH_MCSGS = 2, ORC_SMOOTH_ILU = 3, ORC_SMOOTH_MCBGS = 4 };
typedef struct {
    int nlev, base, cycle, nu1, nu2, smoother;
    double damp;
    /* post-smoother (set_postsmoother, mg_solver.h:179-183); the same as
       the pre-smoother after orc_gmg_init */
    int smoother2;
    double damp2;
    double **diaginv2;   /* Jacobi post-smoother with its own damping, else NULL */
    /* base solver (set_base_solver, mg_solver.h:136): 0 = dense LU, 1 =
       base_steps steps of the pre-smoother from zero (LinearSolver with
       StdConvCheck(base_steps, 0, 0), unsuccessful ends suppressed) */
    int base_kind, base_steps;
    orc_crs *A;          /* per level */
    orc_crs *P, *R;      /* per level (index = fine level) */
    double **diaginv;
    int **color;         /* multicolour GS / ILU: colour of each row */
    int *ncolor;
    orc_crs *ilu;        /* ILU: rows ordered by (colour, column), L and U values */
    int **ilu_diag;      /* ILU: position of the diagonal in each row */
    double **sc, **sd, **st;
    orc_lu lu;
    orc_crs *Arap;       /* rap: owned level operators (coarse levels), else NULL */
    double damp_prol, damp_res; /* StdTransfer prolongation / restriction damping (1 after init) */
} orc_gmg;

/* M = R A P (Galerkin coarse operator), AddMultiplyOf(M, R, A, P) with M
   empty (lib_algebra/algebra_common/sparsematrix_util.h:167-241): per row i
   the products R_ik A_kl P_lj in the order k (R's row), l (A's row), j (P's
   row), zero entries skipped, each product rounded before it is added;
   every column reached is stored (sorted), also when its sum is 0. */
int orc_rap(const orc_crs *R, const orc_crs *A, const orc_crs *P, orc_crs *M);
/* rap != 0: the levels below the top are R A P of the level above
   (AssembledMultiGridCycle::init_rap_operator, mg_solver_impl.hpp:830-1012,
   for a fully refined hierarchy); levA[top] is used as given, the coarse
   operators are owned by the multigrid (G->Arap). */
int orc_gmg_init(orc_gmg *G, const orc_hier *H, orc_crs *levA, int smoother, double damp,
                 int nu1, int nu2, int cycle, int base, int rap);
/* a post-smoother other than the pre-smoother (after orc_gmg_init) */
int orc_gmg_set_postsmoother(orc_gmg *G, int smoother, double damp);
/* base_steps > 0: the base solver is base_steps steps of the pre-smoother
   (base_kind 1) instead of the dense LU */
int orc_gmg_init_ex(orc_gmg *G, const orc_hier *H, orc_crs *levA, int smoother, double damp,
                    int nu1, int nu2, int cycle, int base, int rap, int base_steps);
void orc_gmg_apply(orc_gmg *G, double *c, const double *d);
void orc_gmg_free(orc_gmg *G);

/* Krylov with StdConvCheck(maxit, minDefect, relReduction) */
typedef struct {
    int maxit;
    double min_defect, rel_red;
    int steps;
    double initial_defect, final_defect;
    double *history;     /* optional, capacity hist_cap */
    int hist_cap;
    int converged;
    int restart;         /* BiCGStab: restart when step % restart == 0 (0: off) */
    double min_ortho;    /* BiCGStab: restart when |(r,r0)| <= min_ortho |r| |r0| */
} orc_conv;

int orc_cg(const orc_crs *A, orc_gmg *M, double *x, double *b, orc_conv *C);
void orc_conv_start(orc_conv *C, double d);
void orc_conv_update(orc_conv *C, double d);
int orc_conv_ended(const orc_conv *C);
int orc_conv_post(orc_conv *C);
double orc_vnorm(int n, const double *a);
int orc_bicgstab(const orc_crs *A, orc_gmg *M, double *x, double *b, orc_conv *C);

/* full forward problem helper used by the tests */
typedef struct {
    int elem_type, mx, my, mz, nref;
    uint64_t seed;
    int coef_kind;          /* 0: K=1, 1: K=exp(2g) lognormal field, 2: K=exp(m) per element given */
    int coef_modes; double coef_kmax;
    const double *m_top;    /* coef_kind 2: log-coefficient per top element */
    int vel_kind;           /* 0: none, 1: curl field */
    int vel_modes; double vel_kmax; double diffusion; double peclet;
    int solver;             /* 0 CG, 1 BiCGStab */
    int smoother; double damp; int nu1, nu2, cycle, base;
    int maxit; double rel_red;
    const double *f_top;    /* optional source override (nv top) */
} orc_problem;

/* coefficient per element on every level (coarse levels: mean of children's log K) */
int orc_problem_coefficients(const orc_problem *P, const orc_hier *H, double **Klev);

#ifdef __cplusplus
}
#endif

/* ------------------------------------------------------------ problems -- */
/* Parameters of one assemble-and-solve problem (oracle.py Params mirrors
   this layout). */
typedef struct {
    int elem_type, mx, my, mz, nref;
    uint64_t seed;
    int coef_kind;      /* 0: K=1, 1: exp(2g) field, 2: exp(m) given, 3: constant `diffusion` */
    int coef_modes;
    double coef_kmax;
    int vel_kind;       /* 0: none, 1: curl of a random vector potential */
    int vel_modes;
    double vel_kmax, diffusion, peclet;
    int solver;         /* 0: CG, 1: BiCGStab */
    int smoother;       /* 0: Jacobi, 1: multicolour GS */
    double damp;
    int nu1, nu2, cycle, base;
    int maxit;
    double rel_red, min_defect;
    int rap;            /* 1: Galerkin coarse operators R A P instead of re-assembly */
    int bicg_restart;   /* BiCGStab::set_restart (0: off) */
    double bicg_min_ortho; /* BiCGStab::set_min_orthogonality */
    double damp_prol, damp_res; /* StdTransfer damping (both 1 = none) */
    int post_smoother;  /* set_postsmoother: -1 = the pre-smoother */
    double post_damp;
    int base_steps;     /* set_base_solver: 0 = dense LU, k > 0 = k pre-smoother steps */
} orc_params;
typedef struct orc_prob orc_prob;
orc_prob *orc_prob_create(const orc_params *p, const double *m_top, const double *f_top);
int orc_prob_num_levels(const orc_prob *P);
int orc_prob_level_nv(const orc_prob *P, int l);
int orc_prob_level_ne(const orc_prob *P, int l);
void orc_prob_level_elems(const orc_prob *P, int l, int *elems, double *coords, unsigned char *bnd);
int orc_prob_defect(const orc_prob *P, double theta, double dt, const double *u_old, const double *u, double *d);
int orc_prob_scaled_defect(const orc_prob *P, double sm0, double sa0, double sm1, double sa1, const double *u_old,
                           const double *u, double *d);
int orc_prob_scaled_system(const orc_prob *P, double sm0, double sa0, double sm1, double sa1, const double *u_old,
                           int *rowptr, int *col, double *val, double *b);
int64_t orc_prob_level_nnz(const orc_prob *P, int l);
void orc_prob_level_matrix(const orc_prob *P, int l, int *rowptr, int *col, double *val);
int orc_prob_newton_gmg(orc_prob *P, double theta, double dt, orc_gmg *G, orc_crs *J);
void orc_prob_newton_gmg_free(orc_prob *P, orc_gmg *G, orc_crs *J);
void orc_prob_free(orc_prob *P);

#endif

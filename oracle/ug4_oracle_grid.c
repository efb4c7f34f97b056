/*
 * ug4_oracle_grid.c -- oracle: seeded data, structured hierarchies, CRS helpers.
 *
 * TEST INFRASTRUCTURE ONLY (see ug4_oracle.h).
 *
 * Reference counterparts:
 *   - GlobalMultiGridRefiner::perform_refinement
 *     (lib_grid/refinement/global_multi_grid_refiner.cpp:135) builds the level
 *     hierarchy; here the hierarchy is generated directly on structured boxes.
 *     Fine vertices are children of coarse vertices, edges, faces or volumes,
 *     exactly as the refiner's parent relation (hex -> 8, quad -> 4).  Tets
 *     use the Kuhn (Freudenthal) split, whose regular refinement nests.
 *   - DoFDistribution::reinit (lib_disc/dof_manager/dof_distribution.cpp:1339)
 *     numbers vertices in element-list order; this oracle fixes the
 *     lexicographic order i + nx*(j + ny*k) on every level, and the GPU path
 *     uses the same convention, so CRS arrays compare bit for bit.
 *   - LognormalRandomField::eval_K
 *     (lib_disc/spatial_disc/user_data/common_user_data/lognormal_random_field_impl.h)
 *     is the form of the coefficient field: sqrt(2/N) * sum cos(k.x + alpha);
 *     the modes come from a counter-based splitmix64 stream instead of rand().
 *   - SparseMatrix<T>::set_as_transpose_of / set_as_transpose_of2
 *     (lib_algebra/cpu_algebra/sparsematrix_impl.h:149,186): transpose that
 *     keeps / drops explicit zeros.
 *   - SparseMatrix<T>::axpy, apply_ignore_zero_rows, matmul_minus
 *     (lib_algebra/cpu_algebra/sparsematrix_impl.h:273,294;
 *      lib_algebra/cpu_algebra/sparsematrix.h:203).
 */
#include "ug4_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- RNG ---- */
/* splitmix64 (Steele, Lea, Flood 2014): state += golden gamma, then mix. */
uint64_t orc_splitmix64(uint64_t *state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

double orc_hash_uniform(uint64_t seed, uint64_t i)
{
    uint64_t s = seed ^ (i * 0xD1B54A32D192ED03ULL);
    uint64_t z = orc_splitmix64(&s);
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

void orc_source_uniform(uint64_t seed, int n, double *f)
{
    for (int i = 0; i < n; ++i) f[i] = 2.0 * orc_hash_uniform(seed, (uint64_t)i) - 1.0;
}

static double rng_u01(uint64_t *st) { return (double)(orc_splitmix64(st) >> 11) * (1.0 / 9007199254740992.0); }

static double rng_gauss(uint64_t *st)
{
    /* Box-Muller on two uniforms from the stream; u1 in (0,1]. */
    double u1 = 1.0 - rng_u01(st);
    double u2 = rng_u01(st);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

/* wavevector kappa uniform in the ball |kappa| <= kmax (cycles per unit
   length, rejection from the cube); returned k = 2*pi*kappa */
static void rng_wavevector(uint64_t *st, int dim, double kmax, double *k)
{
    for (;;) {
        double r2 = 0.0, kap[3] = {0, 0, 0};
        for (int d = 0; d < dim; ++d) { kap[d] = kmax * (2.0 * rng_u01(st) - 1.0); r2 += kap[d] * kap[d]; }
        if (r2 <= kmax * kmax && r2 > 0.0) {
            for (int d = 0; d < dim; ++d) k[d] = 6.283185307179586 * kap[d];
            return;
        }
    }
}

int orc_field_scalar_init(orc_field *F, int dim, int nmodes, double kmax, uint64_t seed)
{
    memset(F, 0, sizeof(*F));
    F->nmodes = nmodes; F->dim = dim;
    F->amp = sqrt(2.0 / (double)nmodes);
    F->k = (double *)calloc((size_t)nmodes * dim, sizeof(double));
    F->phase = (double *)calloc((size_t)nmodes, sizeof(double));
    if (!F->k || !F->phase) return -1;
    uint64_t st = seed;
    for (int m = 0; m < nmodes; ++m) {
        rng_wavevector(&st, dim, kmax, F->k + (size_t)m * dim);
        F->phase[m] = 6.283185307179586 * rng_u01(&st);
    }
    F->scale = 1.0;
    return 0;
}

double orc_field_scalar_eval(const orc_field *F, const double *x)
{
    double s = 0.0;
    for (int m = 0; m < F->nmodes; ++m) {
        double th = F->phase[m];
        for (int d = 0; d < F->dim; ++d) th += F->k[m * F->dim + d] * x[d];
        s += cos(th);
    }
    return F->amp * s;
}

int orc_field_curl_init(orc_field *F, int nmodes, double kmax, uint64_t seed)
{
    memset(F, 0, sizeof(*F));
    F->nmodes = nmodes; F->dim = 3;
    F->amp = 1.0;
    F->k = (double *)calloc((size_t)nmodes * 3, sizeof(double));
    F->phase = (double *)calloc((size_t)nmodes, sizeof(double));
    F->a = (double *)calloc((size_t)nmodes * 3, sizeof(double));
    if (!F->k || !F->phase || !F->a) return -1;
    uint64_t st = seed;
    double bound = 0.0;
    for (int m = 0; m < nmodes; ++m) {
        double *k = F->k + 3 * m, *a = F->a + 3 * m;
        rng_wavevector(&st, 3, kmax, k);
        F->phase[m] = 6.283185307179586 * rng_u01(&st);
        for (int d = 0; d < 3; ++d) a[d] = rng_gauss(&st);
        /* store c_m = k x a (curl of a cos(k.x+phi) is -sin(.) k x a) */
        double c0 = k[1] * a[2] - k[2] * a[1];
        double c1 = k[2] * a[0] - k[0] * a[2];
        double c2 = k[0] * a[1] - k[1] * a[0];
        a[0] = c0; a[1] = c1; a[2] = c2;
        bound += sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    }
    F->scale = (bound > 0.0) ? 1.0 / bound : 1.0;   /* |v| <= 1 before the Peclet scaling */
    return 0;
}

void orc_field_curl_eval(const orc_field *F, const double *x, double *v)
{
    v[0] = v[1] = v[2] = 0.0;
    for (int m = 0; m < F->nmodes; ++m) {
        const double *k = F->k + 3 * m, *c = F->a + 3 * m;
        double s = -sin(F->phase[m] + k[0] * x[0] + k[1] * x[1] + k[2] * x[2]);
        v[0] += s * c[0]; v[1] += s * c[1]; v[2] += s * c[2];
    }
    v[0] *= F->scale; v[1] *= F->scale; v[2] *= F->scale;
}

void orc_field_free(orc_field *F)
{
    free(F->k); free(F->phase); free(F->a);
    memset(F, 0, sizeof(*F));
}

/* ---------------------------------------------------------- hierarchy ---- */
static const int kuhn_perm[6][3] = {{0,1,2},{0,2,1},{1,0,2},{1,2,0},{2,0,1},{2,1,0}};

static int level_build(orc_level *L, int elem_type, int cx, int cy, int cz)
{
    memset(L, 0, sizeof(*L));
    L->elem_type = elem_type;
    L->dim = (elem_type == ORC_QUAD) ? 2 : 3;
    L->k = (elem_type == ORC_QUAD) ? 4 : (elem_type == ORC_HEX ? 8 : 4);
    L->nx = cx + 1; L->ny = cy + 1; L->nz = (L->dim == 3) ? cz + 1 : 1;
    L->nv = L->nx * L->ny * L->nz;
    int ncell = cx * cy * ((L->dim == 3) ? cz : 1);
    L->ne = (elem_type == ORC_TET) ? 6 * ncell : ncell;
    L->coords = (double *)malloc(sizeof(double) * (size_t)L->nv * L->dim);
    L->elems = (int *)malloc(sizeof(int) * (size_t)L->ne * L->k);
    L->bnd = (unsigned char *)calloc((size_t)L->nv, 1);
    L->npar = (int *)calloc((size_t)L->nv, sizeof(int));
    L->par = (int *)calloc((size_t)L->nv * 8, sizeof(int));
    if (!L->coords || !L->elems || !L->bnd || !L->npar || !L->par) return -1;
    const int nx = L->nx, ny = L->ny, nz = L->nz;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int v = i + nx * (j + ny * k);
                double *x = L->coords + (size_t)v * L->dim;
                x[0] = (double)i / (double)(nx - 1);
                x[1] = (double)j / (double)(ny - 1);
                if (L->dim == 3) x[2] = (double)k / (double)(nz - 1);
                int b = (i == 0 || i == nx - 1 || j == 0 || j == ny - 1);
                if (L->dim == 3) b = b || (k == 0 || k == nz - 1);
                L->bnd[v] = (unsigned char)b;
            }
    if (elem_type == ORC_QUAD) {
        for (int j = 0; j < cy; ++j)
            for (int i = 0; i < cx; ++i) {
                int *e = L->elems + 4 * (size_t)(i + cx * j);
                int v0 = i + nx * j;
                e[0] = v0; e[1] = v0 + 1; e[2] = v0 + 1 + nx; e[3] = v0 + nx;
            }
    } else {
        for (int k = 0; k < cz; ++k)
            for (int j = 0; j < cy; ++j)
                for (int i = 0; i < cx; ++i) {
                    int h = i + cx * (j + cy * k);
                    int v0 = i + nx * (j + ny * k);
                    int sx = 1, sy = nx, sz = nx * ny;
                    if (elem_type == ORC_HEX) {
                        int *e = L->elems + 8 * (size_t)h;
                        e[0] = v0; e[1] = v0 + sx; e[2] = v0 + sx + sy; e[3] = v0 + sy;
                        e[4] = v0 + sz; e[5] = v0 + sx + sz; e[6] = v0 + sx + sy + sz; e[7] = v0 + sy + sz;
                    } else {
                        int step[3] = {sx, sy, sz};
                        for (int p = 0; p < 6; ++p) {
                            int *e = L->elems + 4 * (size_t)(6 * h + p);
                            int a = kuhn_perm[p][0], b = kuhn_perm[p][1];
                            int v1 = v0 + step[a], v2 = v1 + step[b], v3 = v0 + sx + sy + sz;
                            /* permutations 1,2,5 are odd: swap v1,v2 for positive orientation */
                            int odd = (p == 1 || p == 2 || p == 5);
                            e[0] = v0; e[1] = odd ? v2 : v1; e[2] = odd ? v1 : v2; e[3] = v3;
                        }
                    }
                }
    }
    return 0;
}

static void level_parents(orc_level *F, const orc_level *C)
{
    const int nx = F->nx, ny = F->ny, nz = F->nz;
    for (int k = 0; k < nz; ++k)
        for (int j = 0; j < ny; ++j)
            for (int i = 0; i < nx; ++i) {
                int v = i + nx * (j + ny * k);
                int p[3] = {i & 1, j & 1, k & 1};
                int b[3] = {i >> 1, j >> 1, k >> 1};
                int *par = F->par + 8 * (size_t)v;
                int n = 0;
                if (F->elem_type == ORC_TET) {
                    par[n++] = b[0] + C->nx * (b[1] + C->ny * b[2]);
                    if (p[0] | p[1] | p[2])
                        par[n++] = (b[0] + p[0]) + C->nx * ((b[1] + p[1]) + C->ny * (b[2] + p[2]));
                } else {
                    for (int dk = 0; dk <= p[2]; ++dk)
                        for (int dj = 0; dj <= p[1]; ++dj)
                            for (int di = 0; di <= p[0]; ++di)
                                par[n++] = (b[0] + di) + C->nx * ((b[1] + dj) + C->ny * (b[2] + dk));
                }
                F->npar[v] = n;
            }
}

int orc_hier_create(orc_hier *H, int elem_type, int mx, int my, int mz, int nref)
{
    H->nlev = nref + 1;
    H->lev = (orc_level *)calloc((size_t)H->nlev, sizeof(orc_level));
    if (!H->lev) return -1;
    for (int l = 0; l <= nref; ++l) {
        int f = 1 << l;
        if (level_build(&H->lev[l], elem_type, mx * f, my * f, mz * f)) return -1;
        if (l > 0) level_parents(&H->lev[l], &H->lev[l - 1]);
    }
    return 0;
}

void orc_hier_free(orc_hier *H)
{
    for (int l = 0; l < H->nlev; ++l) {
        orc_level *L = &H->lev[l];
        free(L->coords); free(L->elems); free(L->bnd); free(L->npar); free(L->par);
    }
    free(H->lev);
    H->lev = NULL; H->nlev = 0;
}

/* hierarchy from given levels (an unstructured hierarchy exported by the
   library under test): the arrays are copied; par is nv x 8 per level >= 1 */
int orc_hier_from_arrays(orc_hier *H, int elem_type, int nlev, const int *nv, const int *ne,
                         const double *const *coords, const int *const *elems, const unsigned char *const *bnd,
                         const int *const *npar, const int *const *par)
{
    H->nlev = nlev;
    H->lev = (orc_level *)calloc((size_t)nlev, sizeof(orc_level));
    if (!H->lev) return -1;
    for (int l = 0; l < nlev; ++l) {
        orc_level *L = &H->lev[l];
        L->elem_type = elem_type;
        L->dim = (elem_type == ORC_QUAD || elem_type == ORC_TRI) ? 2 : 3;
        L->k = (elem_type == ORC_HEX) ? 8 : (elem_type == ORC_TRI ? 3 : 4);
        L->nx = L->ny = L->nz = 0;
        L->nv = nv[l];
        L->ne = ne[l];
        L->coords = (double *)malloc(sizeof(double) * (size_t)L->nv * L->dim);
        L->elems = (int *)malloc(sizeof(int) * (size_t)L->ne * L->k);
        L->bnd = (unsigned char *)malloc((size_t)L->nv);
        if (!L->coords || !L->elems || !L->bnd) return -1;
        memcpy(L->coords, coords[l], sizeof(double) * (size_t)L->nv * L->dim);
        memcpy(L->elems, elems[l], sizeof(int) * (size_t)L->ne * L->k);
        memcpy(L->bnd, bnd[l], (size_t)L->nv);
        if (l > 0) {
            L->npar = (int *)malloc(sizeof(int) * (size_t)L->nv);
            L->par = (int *)malloc(sizeof(int) * (size_t)L->nv * 8);
            if (!L->npar || !L->par) return -1;
            memcpy(L->npar, npar[l], sizeof(int) * (size_t)L->nv);
            memcpy(L->par, par[l], sizeof(int) * (size_t)L->nv * 8);
        }
    }
    return 0;
}

void orc_level_centroids(const orc_level *L, double *c)
{
    for (int e = 0; e < L->ne; ++e) {
        double s[3] = {0, 0, 0};
        const int *ev = L->elems + (size_t)e * L->k;
        for (int i = 0; i < L->k; ++i)
            for (int d = 0; d < L->dim; ++d) s[d] += L->coords[(size_t)ev[i] * L->dim + d];
        for (int d = 0; d < L->dim; ++d) c[(size_t)e * L->dim + d] = s[d] * (1.0 / (double)L->k);
    }
}

/* ---------------------------------------------------------------- CRS ---- */
void orc_crs_free(orc_crs *A)
{
    free(A->rowptr); free(A->col); free(A->val);
    memset(A, 0, sizeof(*A));
}

static int cmp_int(const void *a, const void *b)
{
    int x = *(const int *)a, y = *(const int *)b;
    return (x > y) - (x < y);
}

/* Pattern = union of all element couplings, columns sorted per row, values 0.
   (The reference grows the same set through SparseMatrix::operator() /
   get_index while assembling, sparsematrix_impl.h:553-701.) */
int orc_crs_pattern_from_elems(const orc_level *L, orc_crs *A)
{
    const int nv = L->nv, ne = L->ne, k = L->k;
    int *cnt = (int *)calloc((size_t)nv + 1, sizeof(int));
    if (!cnt) return -1;
    for (int e = 0; e < ne; ++e)
        for (int i = 0; i < k; ++i) cnt[L->elems[(size_t)e * k + i] + 1]++;
    for (int v = 0; v < nv; ++v) cnt[v + 1] += cnt[v];
    int *adj = (int *)malloc(sizeof(int) * (size_t)cnt[nv]);
    int *pos = (int *)malloc(sizeof(int) * (size_t)nv);
    if (!adj || !pos) return -1;
    memcpy(pos, cnt, sizeof(int) * (size_t)nv);
    for (int e = 0; e < ne; ++e)
        for (int i = 0; i < k; ++i) adj[pos[L->elems[(size_t)e * k + i]]++] = e;
    A->n_rows = A->n_cols = nv;
    A->rowptr = (int *)calloc((size_t)nv + 1, sizeof(int));
    int cap = 64 * 8;
    int *buf = (int *)malloc(sizeof(int) * (size_t)cap);
    int64_t total = 0;
    /* pass 1: count */
    for (int pass = 0; pass < 2; ++pass) {
        for (int v = 0; v < nv; ++v) {
            int n = 0;
            for (int a = cnt[v]; a < cnt[v + 1]; ++a) {
                const int *ev = L->elems + (size_t)adj[a] * k;
                for (int i = 0; i < k; ++i) {
                    if (n >= cap) { cap *= 2; buf = (int *)realloc(buf, sizeof(int) * (size_t)cap); }
                    buf[n++] = ev[i];
                }
            }
            qsort(buf, (size_t)n, sizeof(int), cmp_int);
            int u = 0;
            for (int t = 0; t < n; ++t)
                if (t == 0 || buf[t] != buf[t - 1]) buf[u++] = buf[t];
            if (pass == 0) A->rowptr[v + 1] = u;
            else memcpy(A->col + A->rowptr[v], buf, sizeof(int) * (size_t)u);
        }
        if (pass == 0) {
            for (int v = 0; v < nv; ++v) A->rowptr[v + 1] += A->rowptr[v];
            total = A->rowptr[nv];
            A->nnz = total;
            A->col = (int *)malloc(sizeof(int) * (size_t)total);
            A->val = (double *)calloc((size_t)total, sizeof(double));
        }
    }
    free(buf); free(adj); free(pos); free(cnt);
    return 0;
}

int orc_crs_find(const orc_crs *A, int r, int c)
{
    int lo = A->rowptr[r], hi = A->rowptr[r + 1] - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int cm = A->col[mid];
        if (cm == c) return mid;
        if (cm < c) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

/* B^T; keep_zeros = 1 follows set_as_transpose_of (every stored entry is
   inserted), keep_zeros = 0 follows set_as_transpose_of2 (zeros dropped). */
int orc_crs_transpose(const orc_crs *B, int keep_zeros, orc_crs *T)
{
    memset(T, 0, sizeof(*T));
    T->n_rows = B->n_cols; T->n_cols = B->n_rows;
    T->rowptr = (int *)calloc((size_t)T->n_rows + 1, sizeof(int));
    if (!T->rowptr) return -1;
    for (int r = 0; r < B->n_rows; ++r)
        for (int a = B->rowptr[r]; a < B->rowptr[r + 1]; ++a)
            if (keep_zeros || B->val[a] != 0.0) T->rowptr[B->col[a] + 1]++;
    for (int r = 0; r < T->n_rows; ++r) T->rowptr[r + 1] += T->rowptr[r];
    T->nnz = T->rowptr[T->n_rows];
    T->col = (int *)malloc(sizeof(int) * (size_t)(T->nnz ? T->nnz : 1));
    T->val = (double *)malloc(sizeof(double) * (size_t)(T->nnz ? T->nnz : 1));
    int *pos = (int *)malloc(sizeof(int) * (size_t)(T->n_rows ? T->n_rows : 1));
    if (!T->col || !T->val || !pos) return -1;
    memcpy(pos, T->rowptr, sizeof(int) * (size_t)T->n_rows);
    /* rows of B visited in increasing order -> columns of T come out sorted */
    for (int r = 0; r < B->n_rows; ++r)
        for (int a = B->rowptr[r]; a < B->rowptr[r + 1]; ++a)
            if (keep_zeros || B->val[a] != 0.0) {
                int t = pos[B->col[a]]++;
                T->col[t] = r;
                T->val[t] = B->val[a];
            }
    free(pos);
    return 0;
}

/* dest = alpha1*v1 + beta1*A*w1, row by row (sparsematrix_impl.h:294-342) */
void orc_crs_axpy(const orc_crs *A, double *dest, double alpha1, const double *v1,
                  double beta1, const double *w1)
{
    for (int i = 0; i < A->n_rows; ++i) {
        int a = A->rowptr[i], e = A->rowptr[i + 1];
        double d;
        if (alpha1 == 0.0) {
            if (a == e) { dest[i] = 0.0; continue; }
            d = beta1 * A->val[a] * w1[A->col[a]];
            for (++a; a < e; ++a) d = d + beta1 * A->val[a] * w1[A->col[a]];
        } else {
            d = (dest == v1 && alpha1 == 1.0) ? dest[i] : alpha1 * v1[i];
            for (; a < e; ++a) d += beta1 * A->val[a] * w1[A->col[a]];
        }
        dest[i] = d;
    }
}

void orc_crs_matmul_minus(const orc_crs *A, double *res, const double *x)
{
    orc_crs_axpy(A, res, 1.0, res, -1.0, x);
}

/* sparsematrix_impl.h:273-288: empty rows leave dest untouched */
void orc_crs_apply_ignore_zero_rows(const orc_crs *A, double *dest, double beta, const double *w)
{
    for (int i = 0; i < A->n_rows; ++i) {
        int a = A->rowptr[i], e = A->rowptr[i + 1];
        if (a == e) continue;
        double d = beta * A->val[a] * w[A->col[a]];
        for (++a; a < e; ++a) d = d + beta * A->val[a] * w[A->col[a]];
        dest[i] = d;
    }
}

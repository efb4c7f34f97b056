/*
 * ug4_oracle_fv1.c -- oracle: FV1 (vertex-centred box) geometry and assembly.
 *
 * TEST INFRASTRUCTURE ONLY (see ug4_oracle.h).
 *
 * Geometry follows FV1Geometry_gen<TElem,dim>::update_local_data / update
 * (lib_disc/spatial_disc/disc_util/fv1_geom.cpp:259-464):
 *   - mid points of edges/faces/element = average of their corners
 *     (ComputeMidPoints, fv1_geom.cpp:53-77);
 *   - one SCVF per element edge, from/to = edge corners
 *     (fv1_traits_most_common::scvf_from_to, fv_util.h:88-95); patch corners
 *     [edge mid, elem centre] in 2D and [edge mid, side-0 centre, elem centre,
 *     side-1 centre] in 3D (ComputeSCVFMidID, fv1_geom.cpp:118-139);
 *   - integration point = average of the patch corners (local and global);
 *   - normal: 2D ElementNormal<ReferenceEdge,2> (geometry_util.h:499-509),
 *     3D ElementNormal<ReferenceQuadrilateral,3> = 0.5 (p2-p0) x (p3-p1)
 *     (geometry_util.h:578-589);
 *   - SCV i = [corner, edge, centre, edge] (2D) or the 8-corner hexahedron of
 *     ComputeSCVMidID (fv1_geom.cpp:156-186); volume by ElementSize of the
 *     quadrilateral / hexahedron (geometry_util.h:156-161,294-323);
 *   - global shape gradients = JtInv(ip) * local gradients of the Lagrange P1
 *     shapes; JtInv per ip for multilinear elements, once for the tetrahedron
 *     (fv1_geom.cpp:406-446).
 * Reference-element tables (corner, edge, face numbering) are those of
 * lib_disc/reference_element/reference_element.cpp (triangle :320-420,
 * quadrilateral :428, tetrahedron :547, hexahedron :1327).
 *
 * The element discretisation itself lives in the external ConvectionDiffusion
 * plugin (not part of ugcore).  It is restated here from the box-method
 * mathematics: for SCVF (from -> to) with area normal n,
 *   diffusion:   F_sh = -(K grad phi_sh) . n ;  J(from,sh) += F_sh,
 *                J(to,sh) -= F_sh;
 *   full upwind: flux = v(ip) . n ; up = flux >= 0 ? from : to
 *                (ConvectionShapesFullUpwind::update, conv_shape.h:277-345);
 *                J(from,up) += flux, J(to,up) -= flux;
 *   source:      rhs(i) += f_i * |SCV_i|.
 * Dirichlet rows: all values 0, diagonal 1, pattern kept, rhs 0
 * (SetDirichletRow, lib_algebra/algebra_common/sparsematrix_util.h:850-862).
 */
#include "ug4_oracle.h"
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------ reference elements ---- */
static const double quad_corner[4][2] = {{0,0},{1,0},{1,1},{0,1}};
static const int quad_edge[4][2] = {{0,1},{1,2},{2,3},{3,0}};
static const int quad_pt_edge[4][2] = {{3,0},{0,1},{1,2},{2,3}};

static const double hex_corner[8][3] = {{0,0,0},{1,0,0},{1,1,0},{0,1,0},{0,0,1},{1,0,1},{1,1,1},{0,1,1}};
static const int hex_edge[12][2] = {{0,1},{1,2},{2,3},{3,0},{0,4},{1,5},{2,6},{3,7},{4,5},{5,6},{6,7},{7,4}};
static const int hex_face[6][4] = {{0,3,2,1},{0,1,5,4},{1,2,6,5},{2,3,7,6},{3,0,4,7},{4,5,6,7}};
static const int hex_edge_face[12][2] = {{0,1},{0,2},{0,3},{0,4},{1,4},{2,1},{3,2},{4,3},{1,5},{2,5},{3,5},{4,5}};
static const int hex_pt_edge[8][3] = {{3,0,4},{0,1,5},{1,2,6},{2,3,7},{4,8,11},{5,9,8},{6,10,9},{7,11,10}};
static const int hex_pt_face[8][3] = {{0,4,1},{0,1,2},{0,2,3},{0,3,4},{1,4,5},{2,1,5},{3,2,5},{4,3,5}};

/* triangle (reference_element.cpp, ReferenceTriangle): corners (0,0),(1,0),(0,1),
   edges (0,1),(1,2),(2,0), edges at corner {2,0},{0,1},{1,2} */
static const double tri_corner[3][2] = {{0,0},{1,0},{0,1}};
static const int tri_edge[3][2] = {{0,1},{1,2},{2,0}};
static const int tri_pt_edge[3][2] = {{2,0},{0,1},{1,2}};

static const double tet_corner[4][3] = {{0,0,0},{1,0,0},{0,1,0},{0,0,1}};
static const int tet_edge[6][2] = {{0,1},{1,2},{2,0},{0,3},{1,3},{2,3}};
static const int tet_face[4][3] = {{0,2,1},{1,2,3},{0,3,2},{0,1,3}};
static const int tet_edge_face[6][2] = {{0,3},{0,1},{0,2},{3,2},{1,3},{2,1}};
static const int tet_pt_edge[4][3] = {{2,0,3},{0,1,4},{1,2,5},{3,4,5}};
static const int tet_pt_face[4][3] = {{0,2,3},{0,3,1},{0,1,2},{3,2,1}};

/* local gradients of the P1 Lagrange shapes at local position x */
static void local_grads(int type, const double *x, double g[8][3])
{
    if (type == ORC_TRI) {
        g[0][0] = -1; g[0][1] = -1;
        g[1][0] = 1;  g[1][1] = 0;
        g[2][0] = 0;  g[2][1] = 1;
    } else if (type == ORC_QUAD) {
        g[0][0] = -(1.0 - x[1]); g[0][1] = -(1.0 - x[0]);
        g[1][0] =  (1.0 - x[1]); g[1][1] = -x[0];
        g[2][0] =  x[1];         g[2][1] =  x[0];
        g[3][0] = -x[1];         g[3][1] =  (1.0 - x[0]);
    } else if (type == ORC_HEX) {
        for (int i = 0; i < 8; ++i) {
            const double *c = hex_corner[i];
            double fx = c[0] ? x[0] : 1.0 - x[0], dx = c[0] ? 1.0 : -1.0;
            double fy = c[1] ? x[1] : 1.0 - x[1], dy = c[1] ? 1.0 : -1.0;
            double fz = c[2] ? x[2] : 1.0 - x[2], dz = c[2] ? 1.0 : -1.0;
            g[i][0] = dx * fy * fz;
            g[i][1] = fx * dy * fz;
            g[i][2] = fx * fy * dz;
        }
    } else {
        g[0][0] = -1; g[0][1] = -1; g[0][2] = -1;
        g[1][0] = 1;  g[1][1] = 0;  g[1][2] = 0;
        g[2][0] = 0;  g[2][1] = 1;  g[2][2] = 0;
        g[3][0] = 0;  g[3][1] = 0;  g[3][2] = 1;
    }
}

/* JtInv = (J^T)^{-1} with J_ab = d x_a / d xi_b */
static void jt_inverse(int dim, int k, const double *corner, const double lg[8][3], double Ji[3][3])
{
    double J[3][3] = {{0}};
    for (int i = 0; i < k; ++i)
        for (int a = 0; a < dim; ++a)
            for (int b = 0; b < dim; ++b) J[a][b] += corner[i * dim + a] * lg[i][b];
    if (dim == 2) {
        double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        double inv = 1.0 / det;
        /* (J^T)^{-1} = (J^{-1})^T */
        Ji[0][0] =  J[1][1] * inv; Ji[0][1] = -J[1][0] * inv;
        Ji[1][0] = -J[0][1] * inv; Ji[1][1] =  J[0][0] * inv;
    } else {
        double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
        double inv = 1.0 / det;
        double Jinv[3][3];
        Jinv[0][0] = c00 * inv;
        Jinv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * inv;
        Jinv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * inv;
        Jinv[1][0] = c01 * inv;
        Jinv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * inv;
        Jinv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * inv;
        Jinv[2][0] = c02 * inv;
        Jinv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * inv;
        Jinv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * inv;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) Ji[a][b] = Jinv[b][a];
    }
}

static void avg(int dim, int n, const double *const *p, double *out)
{
    for (int d = 0; d < dim; ++d) out[d] = p[0][d];
    for (int j = 1; j < n; ++j)
        for (int d = 0; d < dim; ++d) out[d] += p[j][d];
    for (int d = 0; d < dim; ++d) out[d] *= 1.0 / (double)n;
}

static double quad_size2d(const double q[4][3])
{
    return 0.5 * fabs((q[3][1] - q[1][1]) * (q[2][0] - q[0][0]) - (q[3][0] - q[1][0]) * (q[2][1] - q[0][1]));
}

static void sub3(double *o, const double *a, const double *b) { o[0] = a[0]-b[0]; o[1] = a[1]-b[1]; o[2] = a[2]-b[2]; }
static void cross3(double *o, const double *a, const double *b)
{
    o[0] = a[1]*b[2] - a[2]*b[1]; o[1] = a[2]*b[0] - a[0]*b[2]; o[2] = a[0]*b[1] - a[1]*b[0];
}
static double dot3(const double *a, const double *b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }

/* ElementSize<ReferenceHexahedron,3> (geometry_util.h:294-323) */
static double hex_size(const double c[8][3])
{
    double x50[3], x14[3], x10[3], x20[3], x60[3], m1[3], n1[3];
    double x24[3], x30[3], x70[3], m2[3], n2[3];
    sub3(x50, c[5], c[0]); sub3(x14, c[1], c[4]); sub3(x10, c[1], c[0]);
    sub3(x20, c[2], c[0]); sub3(x60, c[6], c[0]);
    cross3(m1, x50, x14); cross3(n1, x10, x20);
    n1[0] += m1[0]; n1[1] += m1[1]; n1[2] += m1[2];
    sub3(x24, c[2], c[4]); sub3(x30, c[3], c[0]); sub3(x70, c[7], c[0]);
    cross3(m2, x60, x24); cross3(n2, x20, x30);
    n2[0] += m2[0]; n2[1] += m2[1]; n2[2] += m2[2];
    return (1.0 / 6.0) * (dot3(n1, x60) + dot3(n2, x70));
}

/* Computes the FV1 geometry of one element from its global corner coords.
   Local ip positions are recomputed from the local reference corners the
   same way (they are constants of the element type). */
int orc_fv1_geometry(int type, const double *corner, orc_fv1geom *G)
{
    memset(G, 0, sizeof(*G));
    const int dim = (type == ORC_QUAD || type == ORC_TRI) ? 2 : 3;
    const int k = (type == ORC_HEX) ? 8 : (type == ORC_TRI ? 3 : 4);
    const int ne = (type == ORC_QUAD) ? 4 : (type == ORC_HEX ? 12 : (type == ORC_TRI ? 3 : 6));
    const int nf = (type == ORC_HEX) ? 6 : (type == ORC_TET ? 4 : 0);
    const int (*edge)[2] = (type == ORC_QUAD) ? quad_edge
                           : (type == ORC_HEX ? hex_edge : (type == ORC_TRI ? tri_edge : tet_edge));
    G->nscv = k; G->nscvf = ne;

    /* loc/glob mids: [0] corners, [1] edges, [2] faces, [3] centre */
    double lc[8][3], gc[8][3], le[12][3], ge[12][3], lf[6][3], gf[6][3], lm[3], gm[3];
    for (int i = 0; i < k; ++i)
        for (int d = 0; d < dim; ++d) {
            lc[i][d] = (type == ORC_QUAD) ? quad_corner[i][d]
                       : (type == ORC_HEX ? hex_corner[i][d] : (type == ORC_TRI ? tri_corner[i][d] : tet_corner[i][d]));
            gc[i][d] = corner[i * dim + d];
        }
    for (int e = 0; e < ne; ++e) {
        const double *pl[2] = {lc[edge[e][0]], lc[edge[e][1]]};
        const double *pg[2] = {gc[edge[e][0]], gc[edge[e][1]]};
        avg(dim, 2, pl, le[e]); avg(dim, 2, pg, ge[e]);
    }
    for (int f = 0; f < nf; ++f) {
        int nfc = (type == ORC_HEX) ? 4 : 3;
        const double *pl[4], *pg[4];
        for (int j = 0; j < nfc; ++j) {
            int c = (type == ORC_HEX) ? hex_face[f][j] : tet_face[f][j];
            pl[j] = lc[c]; pg[j] = gc[c];
        }
        avg(dim, nfc, pl, lf[f]); avg(dim, nfc, pg, gf[f]);
    }
    {
        const double *pl[8], *pg[8];
        for (int i = 0; i < k; ++i) { pl[i] = lc[i]; pg[i] = gc[i]; }
        avg(dim, k, pl, lm); avg(dim, k, pg, gm);
    }

    /* SCVF: patch, ip, normal */
    double lip[12][3];
    for (int e = 0; e < ne; ++e) {
        G->from[e] = edge[e][0]; G->to[e] = edge[e][1];
        if (dim == 2) {
            const double *pl[2] = {le[e], lm}, *pg[2] = {ge[e], gm};
            avg(2, 2, pl, lip[e]); avg(2, 2, pg, G->gip[e]);
            double dx = gm[0] - ge[e][0], dy = gm[1] - ge[e][1];
            G->normal[e][0] = dy; G->normal[e][1] = -dx;
        } else {
            int s0 = (type == ORC_HEX) ? hex_edge_face[e][0] : tet_edge_face[e][0];
            int s1 = (type == ORC_HEX) ? hex_edge_face[e][1] : tet_edge_face[e][1];
            const double *pl[4] = {le[e], lf[s0], lm, lf[s1]};
            const double *pg[4] = {ge[e], gf[s0], gm, gf[s1]};
            avg(3, 4, pl, lip[e]); avg(3, 4, pg, G->gip[e]);
            double a[3], b[3], n[3];
            sub3(a, pg[2], pg[0]); sub3(b, pg[3], pg[1]);
            cross3(n, a, b);
            G->normal[e][0] = 0.5 * n[0]; G->normal[e][1] = 0.5 * n[1]; G->normal[e][2] = 0.5 * n[2];
        }
    }

    /* SCV volumes */
    for (int i = 0; i < k; ++i) {
        if (dim == 2) {
            double q[4][3] = {{0}};
            const int (*pe)[2] = (type == ORC_TRI) ? tri_pt_edge : quad_pt_edge;
            const double *p[4] = {gc[i], ge[pe[i][0]], gm, ge[pe[i][1]]};
            for (int j = 0; j < 4; ++j) { q[j][0] = p[j][0]; q[j][1] = p[j][1]; }
            G->vol[i] = quad_size2d(q);
        } else {
            const int *pe = (type == ORC_HEX) ? hex_pt_edge[i] : tet_pt_edge[i];
            const int *pf = (type == ORC_HEX) ? hex_pt_face[i] : tet_pt_face[i];
            const double *p[8] = {gc[i], ge[pe[1]], gf[pf[0]], ge[pe[0]], ge[pe[2]], gf[pf[2]], gm, gf[pf[1]]};
            double h[8][3];
            for (int j = 0; j < 8; ++j) { h[j][0] = p[j][0]; h[j][1] = p[j][1]; h[j][2] = p[j][2]; }
            G->vol[i] = hex_size(h);
        }
    }

    /* gradients */
    double Ji[3][3], lg[8][3];
    const int affine = (type == ORC_TET || type == ORC_TRI);
    if (affine) {
        local_grads(type, lip[0], lg);
        jt_inverse(dim, k, corner, lg, Ji);
    }
    for (int e = 0; e < ne; ++e) {
        local_grads(type, lip[e], lg);
        if (!affine) jt_inverse(dim, k, corner, lg, Ji);
        for (int sh = 0; sh < k; ++sh)
            for (int a = 0; a < dim; ++a) {
                double s = 0.0;
                for (int b = 0; b < dim; ++b) s += Ji[a][b] * lg[sh][b];
                G->grad[e][sh][a] = s;
            }
    }
    return 0;
}

/* element matrix of -div(K grad u) + div(v u) and SCV volumes */
static void element_matrix(int type, const orc_fv1geom *G, int dim, int k, double K,
                           const double *vel /* nscvf*dim or NULL */, int upwind, double Aloc[8][8])
{
    memset(Aloc, 0, sizeof(double) * 64);
    for (int ip = 0; ip < G->nscvf; ++ip) {
        const int from = G->from[ip], to = G->to[ip];
        for (int sh = 0; sh < k; ++sh) {
            double gn = 0.0;
            for (int d = 0; d < dim; ++d) gn += G->grad[ip][sh][d] * G->normal[ip][d];
            double F = -K * gn;
            Aloc[from][sh] += F;
            Aloc[to][sh] -= F;
        }
        if (upwind && vel) {
            double flux = 0.0;
            for (int d = 0; d < dim; ++d) flux += G->normal[ip][d] * vel[ip * dim + d];
            int up = (flux >= 0.0) ? from : to;
            Aloc[from][up] += flux;
            Aloc[to][up] -= flux;
        }
    }
    (void)type;
}

static void element_corners(const orc_level *L, int e, double *corner)
{
    const int *ev = L->elems + (size_t)e * L->k;
    for (int i = 0; i < L->k; ++i)
        for (int d = 0; d < L->dim; ++d) corner[i * L->dim + d] = L->coords[(size_t)ev[i] * L->dim + d];
}

int orc_assemble(const orc_level *L, const orc_disc *D, orc_crs *A, double *b)
{
    if (orc_crs_pattern_from_elems(L, A)) return -1;
    const int k = L->k, dim = L->dim;
    if (b) memset(b, 0, sizeof(double) * (size_t)L->nv);
    double corner[24], vel[36];
    orc_fv1geom G;
    double Aloc[8][8];
    for (int e = 0; e < L->ne; ++e) {
        element_corners(L, e, corner);
        orc_fv1_geometry(L->elem_type, corner, &G);
        const double *v = NULL;
        if (D->upwind) {
            if (D->vel) v = D->vel + (size_t)e * G.nscvf * dim;
            else if (D->vfield) {
                for (int ip = 0; ip < G.nscvf; ++ip) orc_field_curl_eval(D->vfield, G.gip[ip], vel + ip * dim);
                v = vel;
            }
        }
        double K = D->K ? D->K[e] : 1.0;
        element_matrix(L->elem_type, &G, dim, k, K, v, D->upwind, Aloc);
        const int *ev = L->elems + (size_t)e * k;
        if (D->inst) {
            /* rhs of the element first (it uses the stiffness A_e), then
               locA = sm0 M_e + sa0 A_e; every scaled term rounded before it is added */
            double rhs[8];
            if (b) {
                for (int i = 0; i < k; ++i) {
                    const double fv = (D->f ? D->f[ev[i]] : 0.0) * G.vol[i];
                    double r = 0.0;
                    if (D->sa0 != 0.0) r = D->sa0 * fv;
                    r = r + (-D->sm1) * (G.vol[i] * D->u_old[ev[i]]);
                    if (D->sa1 != 0.0) {
                        double au = 0.0;
                        for (int j = 0; j < k; ++j) au = au + Aloc[i][j] * D->u_old[ev[j]];
                        r = r + (-D->sa1) * au;
                        r = r + D->sa1 * fv;
                    }
                    rhs[i] = r;
                }
            }
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j) {
                    const double m = (i == j) ? D->sm0 * G.vol[i] : 0.0;
                    const int s = orc_crs_find(A, ev[i], ev[j]);
                    A->val[s] += m + D->sa0 * Aloc[i][j];
                }
            if (b)
                for (int i = 0; i < k; ++i) b[ev[i]] += rhs[i];
            continue;
        }
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) {
                int s = orc_crs_find(A, ev[i], ev[j]);
                A->val[s] += Aloc[i][j];
            }
        if (b && D->f)
            for (int i = 0; i < k; ++i) b[ev[i]] += D->f[ev[i]] * G.vol[i];
    }
    if (D->dirichlet) {
        for (int v = 0; v < L->nv; ++v) {
            if (!L->bnd[v]) continue;
            for (int a = A->rowptr[v]; a < A->rowptr[v + 1]; ++a) A->val[a] = 0.0;
            A->val[orc_crs_find(A, v, v)] = 1.0;
            if (b) b[v] = 0.0;
        }
    }
    return 0;
}

/* Defect d = A(u) u - f of the level (DomainDiscretization::assemble_defect,
   lib_disc/spatial_disc/domain_disc_impl.h:648; StdGlobAssembler::
   AssembleDefect, elem_disc_assemble_util.h:578-690): per element
   locD = A_e u_e (add_def_A_elem, restated as the element operator applied to
   the local solution), locD += (-1) rhs_e (add_rhs_elem, scale_append), added
   to d in element order; Dirichlet vertices get d = 0
   (DirichletBoundary::adjust_defect, lagrange_dirichlet_boundary_impl.h:
   972-1033).  With D->inst the instationary AssembleDefect
   (elem_disc_assemble_util.h:713-860) for the time points (u, u_old) with
   s_m = (sm0, sm1), s_a = (sa0, sa1): per time point t,
   locD += s_m[t] M_e u_t, then (s_a[t] != 0) locD += s_a[t] A_e u_t and
   locD += (-s_a[t]) rhs_e; M_e = diag(|SCV_i|). */
int orc_assemble_defect(const orc_level *L, const orc_disc *D, const double *u, double *d)
{
    const int k = L->k, dim = L->dim;
    memset(d, 0, sizeof(double) * (size_t)L->nv);
    double corner[24], vel[36];
    orc_fv1geom G;
    double Aloc[8][8];
    for (int e = 0; e < L->ne; ++e) {
        element_corners(L, e, corner);
        orc_fv1_geometry(L->elem_type, corner, &G);
        const double *v = NULL;
        if (D->upwind) {
            if (D->vel) v = D->vel + (size_t)e * G.nscvf * dim;
            else if (D->vfield) {
                for (int ip = 0; ip < G.nscvf; ++ip) orc_field_curl_eval(D->vfield, G.gip[ip], vel + ip * dim);
                v = vel;
            }
        }
        const double K = D->K ? D->K[e] : 1.0;
        element_matrix(L->elem_type, &G, dim, k, K, v, D->upwind, Aloc);
        const int *ev = L->elems + (size_t)e * k;
        for (int i = 0; i < k; ++i) {
            const double fv = (D->f ? D->f[ev[i]] : 0.0) * G.vol[i];
            double au = 0.0;
            for (int j = 0; j < k; ++j) au = au + Aloc[i][j] * u[ev[j]];
            double r;
            if (!D->inst) {
                r = au + (-1.0) * fv;
            } else {
                r = 0.0 + D->sm0 * (G.vol[i] * u[ev[i]]);
                if (D->sa0 != 0.0) {
                    r = r + D->sa0 * au;
                    r = r + (-D->sa0) * fv;
                }
                r = r + D->sm1 * (G.vol[i] * D->u_old[ev[i]]);
                if (D->sa1 != 0.0) {
                    double ao = 0.0;
                    for (int j = 0; j < k; ++j) ao = ao + Aloc[i][j] * D->u_old[ev[j]];
                    r = r + D->sa1 * ao;
                    r = r + (-D->sa1) * fv;
                }
            }
            d[ev[i]] += r;
        }
    }
    if (D->dirichlet)
        for (int v = 0; v < L->nv; ++v)
            if (L->bnd[v]) d[v] = 0.0;
    return 0;
}

/* sum over elements of the SCV volume of each vertex: d rhs_i / d f_i */
void orc_scv_volume_sum(const orc_level *L, double *vol)
{
    memset(vol, 0, sizeof(double) * (size_t)L->nv);
    double corner[24];
    orc_fv1geom G;
    for (int e = 0; e < L->ne; ++e) {
        element_corners(L, e, corner);
        orc_fv1_geometry(L->elem_type, corner, &G);
        const int *ev = L->elems + (size_t)e * L->k;
        for (int i = 0; i < L->k; ++i) vol[ev[i]] += G.vol[i];
    }
}

/* element-local adjoint gradient for K_e = exp(m_e):
   dJ/dm_e = -K_e * sum_{i not Dirichlet} lambda_i (A1_e u_e)_i  */
int orc_grad_logk(const orc_level *L, const double *K, const double *u, const double *lam, double *g)
{
    double corner[24];
    orc_fv1geom G;
    double A1[8][8];
    for (int e = 0; e < L->ne; ++e) {
        element_corners(L, e, corner);
        orc_fv1_geometry(L->elem_type, corner, &G);
        element_matrix(L->elem_type, &G, L->dim, L->k, 1.0, NULL, 0, A1);
        const int *ev = L->elems + (size_t)e * L->k;
        double s = 0.0;
        for (int i = 0; i < L->k; ++i) {
            if (L->bnd[ev[i]]) continue;
            double r = 0.0;
            for (int j = 0; j < L->k; ++j) r += A1[i][j] * u[ev[j]];
            s += lam[ev[i]] * r;
        }
        g[e] = -K[e] * s;
    }
    return 0;
}

/* element matrix (row-major k x k) and SCV volumes of element e of level L,
   exported for the reference-algebra driver (oracle/ref_driver.cpp) */
int orc_element_matrix(const orc_level *L, int e, double K, const orc_field *vf, int upwind,
                       double *Aloc, double *vol)
{
    double corner[24], vel[36], A8[8][8];
    orc_fv1geom G;
    element_corners(L, e, corner);
    orc_fv1_geometry(L->elem_type, corner, &G);
    const double *v = NULL;
    if (upwind && vf) {
        for (int ip = 0; ip < G.nscvf; ++ip) orc_field_curl_eval(vf, G.gip[ip], vel + ip * L->dim);
        v = vel;
    }
    element_matrix(L->elem_type, &G, L->dim, L->k, K, v, upwind, A8);
    for (int i = 0; i < L->k; ++i) {
        for (int j = 0; j < L->k; ++j) Aloc[i * L->k + j] = A8[i][j];
        if (vol) vol[i] = G.vol[i];
    }
    return L->k;
}

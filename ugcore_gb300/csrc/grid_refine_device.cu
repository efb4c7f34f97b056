// grid_refine_device.cu -- one regular refinement step of an unstructured
// level on the device.
//
// The same rules and the same numbering as the host refinement in
// grid_unstructured.cu (which stays as the host-side reference and serves the
// host-only ug4gb_io_ugx_level): edges are numbered by their sorted (smaller,
// larger) vertex keys, quadrilateral faces of hexahedra by their sorted corner
// quadruples; new vertices are the averages of their parents (corners taken
// in increasing index, explicitly rounded in that order); children in
// element order with the reference child tables, the tetrahedron's inner
// octahedron cut along its shortest diagonal (first of (01,23), (12,03),
// (02,13) on ties), every child stored with positive orientation; the
// Dirichlet edges / faces / elements carried to the children and to the edges
// and faces created inside Dirichlet faces and elements.  Keys are sorted and
// de-duplicated with CUB's radix sort and selection (set-up only).
#include <cub/cub.cuh>

#include <vector>

#include "grid_refine.cuh"

namespace ug4gb {

namespace {

constexpr u64 kNoKey = ~0ULL;

__device__ __forceinline__ u64 ekey(int a, int b)
{
    return a < b ? ((u64)a << 32) | (u64)(unsigned)b : ((u64)b << 32) | (u64)(unsigned)a;
}

__device__ __forceinline__ void sort4(int *s)
{
    for (int i = 1; i < 4; ++i) {
        int v = s[i], j = i - 1;
        while (j >= 0 && s[j] > v) {
            s[j + 1] = s[j];
            --j;
        }
        s[j + 1] = v;
    }
}

__device__ __forceinline__ int find_u64(const u64 *arr, int n, u64 key)
{
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const u64 v = arr[mid];
        if (v == key) return mid;
        if (v < key) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

__device__ __forceinline__ int find_face(const u64 *fh, const u64 *fl, int n, u64 h, u64 l)
{
    int lo = 0, hi = n - 1;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const u64 vh = fh[mid], vl = fl[mid];
        if (vh == h && vl == l) return mid;
        if (vh < h || (vh == h && vl < l)) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// reference tables (reference_element.cpp)
__constant__ int c_tri_edges[3][2] = {{0, 1}, {1, 2}, {2, 0}};
__constant__ int c_quad_edges[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
__constant__ int c_tet_edges[6][2] = {{0, 1}, {1, 2}, {2, 0}, {0, 3}, {1, 3}, {2, 3}};
__constant__ int c_hex_edges[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {0, 4}, {1, 5},
                                       {2, 6}, {3, 7}, {4, 5}, {5, 6}, {6, 7}, {7, 4}};
__constant__ int c_hex_faces[6][4] = {{0, 3, 2, 1}, {0, 1, 5, 4}, {1, 2, 6, 5}, {2, 3, 7, 6}, {3, 0, 4, 7}, {4, 5, 6, 7}};
__constant__ int c_quad_ref[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
__constant__ int c_hex_ref[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                    {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

__device__ __forceinline__ int n_edges_of(int t) { return t == UG4GB_TRI ? 3 : (t == UG4GB_QUAD ? 4 : (t == UG4GB_TET ? 6 : 12)); }
__device__ __forceinline__ int edge_corner(int t, int j, int q)
{
    return t == UG4GB_TRI ? c_tri_edges[j][q]
                          : (t == UG4GB_QUAD ? c_quad_edges[j][q] : (t == UG4GB_TET ? c_tet_edges[j][q] : c_hex_edges[j][q]));
}

__global__ void k_edge_keys(const int *elems, int ne, int k, int t, u64 *keys)
{
    const int ned = n_edges_of(t);
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)ne * ned) return;
    const int e = (int)(i / ned), j = (int)(i % ned);
    keys[i] = ekey(elems[(size_t)e * k + edge_corner(t, j, 0)], elems[(size_t)e * k + edge_corner(t, j, 1)]);
}

__global__ void k_hex_face_keys(const int *elems, int ne, u64 *hi, u64 *lo, int *idx)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (int64_t)ne * 6) return;
    const int e = (int)(i / 6), f = (int)(i % 6);
    int s[4];
    for (int j = 0; j < 4; ++j) s[j] = elems[(size_t)e * 8 + c_hex_faces[f][j]];
    sort4(s);
    hi[i] = ((u64)s[0] << 32) | (u64)(unsigned)s[1];
    lo[i] = ((u64)s[2] << 32) | (u64)(unsigned)s[3];
    idx[i] = (int)i;
}

// vertex v = average of the (sorted) corners; parents = those corners
__device__ __forceinline__ void set_vertex(const double *cc, int dim, int *corners, int n, int v, double *fc,
                                          int *npar, int *par)
{
    for (int i = 1; i < n; ++i) {
        int x = corners[i], j = i - 1;
        while (j >= 0 && corners[j] > x) {
            corners[j + 1] = corners[j];
            --j;
        }
        corners[j + 1] = x;
    }
    const double inv = 1.0 / n;
    for (int d = 0; d < dim; ++d) {
        double acc = 0.0;
        for (int j = 0; j < n; ++j) acc = __dadd_rn(acc, cc[(size_t)corners[j] * dim + d]);
        fc[(size_t)v * dim + d] = __dmul_rn(acc, inv);
    }
    npar[v] = n;
    for (int j = 0; j < 8; ++j) par[(size_t)v * 8 + j] = j < n ? corners[j] : -1;
}

__global__ void k_old_vertices(const double *cc, const unsigned char *cb, int nv, int dim, double *fc,
                               unsigned char *fb, int *npar, int *par)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv) return;
    int c1[1] = {v};
    set_vertex(cc, dim, c1, 1, v, fc, npar, par);
    fb[v] = cb[v];
}

__global__ void k_edge_vertices(const u64 *E, int nedge, const double *cc, int nv, int dim, double *fc,
                                unsigned char *fb, int *npar, int *par)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nedge) return;
    int c2[2] = {(int)(E[i] >> 32), (int)(E[i] & 0xffffffffULL)};
    set_vertex(cc, dim, c2, 2, nv + i, fc, npar, par);
    fb[nv + i] = 0;
}

__global__ void k_face_vertices(const u64 *fh, const u64 *fl, int nqf, const double *cc, int base, double *fc,
                                unsigned char *fb, int *npar, int *par)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nqf) return;
    int c4[4] = {(int)(fh[i] >> 32), (int)(fh[i] & 0xffffffffULL), (int)(fl[i] >> 32), (int)(fl[i] & 0xffffffffULL)};
    set_vertex(cc, 3, c4, 4, base + i, fc, npar, par);
    fb[base + i] = 0;
}

// centres of 2D quadrilaterals (4 corners) or of hexahedra (8 corners)
__global__ void k_elem_centres(const int *elems, int ne, int k, const double *cc, int dim, int base, double *fc,
                               unsigned char *fb, int *npar, int *par)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int cs[8];
    for (int j = 0; j < k; ++j) cs[j] = elems[(size_t)e * k + j];
    set_vertex(cc, dim, cs, k, base + e, fc, npar, par);
    fb[base + e] = 0;
}

__global__ void k_mark_dir_edges(const u64 *dir, int n, const u64 *E, int nedge, int nv, unsigned char *fb, int *err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int m = find_u64(E, nedge, dir[i]);
    if (m < 0) {
        atomicExch(err, 1);
        return;
    }
    fb[nv + m] = 1;
}

struct Lookup {
    const u64 *E;
    int nedge;
    const u64 *fh, *fl;
    int nqf;
    int nv;
    int *err;
    __device__ int mid(int a, int b) const
    {
        const int i = find_u64(E, nedge, ekey(a, b));
        if (i < 0) {
            atomicExch(err, 1);
            return 0;
        }
        return nv + i;
    }
    __device__ int qcentre(const int *q) const
    {
        int s[4] = {q[0], q[1], q[2], q[3]};
        sort4(s);
        const int i = find_face(fh, fl, nqf, ((u64)s[0] << 32) | (u64)(unsigned)s[1],
                                ((u64)s[2] << 32) | (u64)(unsigned)s[3]);
        if (i < 0) {
            atomicExch(err, 1);
            return 0;
        }
        return nv + nedge + i;
    }
};

// 2D: twice the signed area of (0, 1, 2); 3D: six times the signed volume of
// (0, 1, 2, 3), in the host's evaluation order without contraction
__device__ double signed_measure(const double *x, int dim, const int *ev)
{
    const double *x0 = x + (size_t)ev[0] * dim, *x1 = x + (size_t)ev[1] * dim, *x2 = x + (size_t)ev[2] * dim;
    if (dim == 2)
        return __dsub_rn(__dmul_rn(__dsub_rn(x1[0], x0[0]), __dsub_rn(x2[1], x0[1])),
                         __dmul_rn(__dsub_rn(x1[1], x0[1]), __dsub_rn(x2[0], x0[0])));
    const double *x3 = x + (size_t)ev[3] * dim;
    double a[3], b[3], c[3];
    for (int d = 0; d < 3; ++d) {
        a[d] = __dsub_rn(x1[d], x0[d]);
        b[d] = __dsub_rn(x2[d], x0[d]);
        c[d] = __dsub_rn(x3[d], x0[d]);
    }
    const double t0 = __dmul_rn(a[0], __dsub_rn(__dmul_rn(b[1], c[2]), __dmul_rn(b[2], c[1])));
    const double t1 = __dmul_rn(a[1], __dsub_rn(__dmul_rn(b[0], c[2]), __dmul_rn(b[2], c[0])));
    const double t2 = __dmul_rn(a[2], __dsub_rn(__dmul_rn(b[0], c[1]), __dmul_rn(b[1], c[0])));
    return __dadd_rn(__dsub_rn(t0, t1), t2);
}

__device__ void orient_child(const double *x, int dim, int t, int *ev)
{
    if (t == UG4GB_HEX) {
        const int f[4] = {ev[0], ev[1], ev[3], ev[4]};
        if (signed_measure(x, dim, f) >= 0.0) return;
        int s = ev[1]; ev[1] = ev[3]; ev[3] = s;
        s = ev[5]; ev[5] = ev[7]; ev[7] = s;
    } else if (t == UG4GB_QUAD) {
        if (signed_measure(x, dim, ev) >= 0.0) return;
        int s = ev[1]; ev[1] = ev[3]; ev[3] = s;
    } else {
        if (signed_measure(x, dim, ev) >= 0.0) return;
        int s = ev[1]; ev[1] = ev[2]; ev[2] = s;
    }
}

__device__ __forceinline__ int tet_best_diagonal(const double *fc, const int (*diag)[2])
{
    int best = 0;
    double bl = 0.0;
    for (int d = 0; d < 3; ++d) {
        double l2 = 0.0;
        for (int x = 0; x < 3; ++x) {
            const double dd = __dsub_rn(fc[(size_t)diag[d][0] * 3 + x], fc[(size_t)diag[d][1] * 3 + x]);
            l2 = __dadd_rn(l2, __dmul_rn(dd, dd));
        }
        if (d == 0 || l2 < bl) {
            bl = l2;
            best = d;
        }
    }
    return best;
}

// Children of element e (then oriented), and for elements of Dirichlet
// subsets the edges / faces created inside them (at pe[e] / pf[e], the
// exclusive scans of their counts) with their vertices marked.
template <int T>
__global__ void k_children(const int *celems, int ne, const unsigned char *cedir, Lookup lk, int nqf_base,
                           int cen_base, const double *fc, int *felems, unsigned char *fedir, const int *pe,
                           const int *pf, u64 *oute, int4 *outf, unsigned char *fb)
{
    constexpr int K = (T == UG4GB_HEX) ? 8 : (T == UG4GB_TRI ? 3 : 4);
    constexpr int DIM = (T == UG4GB_QUAD || T == UG4GB_TRI) ? 2 : 3;
    constexpr int NCH = (DIM == 2) ? 4 : 8;
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int ev[K];
    for (int j = 0; j < K; ++j) ev[j] = celems[(size_t)e * K + j];
    const bool ed = cedir[e] != 0;
    u64 *IE = oute + (ed ? pe[e] : 0);
    int4 *IF = outf + (ed ? pf[e] : 0);
    int ch[NCH][K];
    if constexpr (T == UG4GB_TRI) {
        const int m0 = lk.mid(ev[0], ev[1]), m1 = lk.mid(ev[1], ev[2]), m2 = lk.mid(ev[2], ev[0]);
        const int t[4][3] = {{ev[0], m0, m2}, {m0, ev[1], m1}, {m2, m1, ev[2]}, {m0, m1, m2}};
        for (int q = 0; q < 4; ++q)
            for (int j = 0; j < 3; ++j) ch[q][j] = t[q][j];
        if (ed) {
            IE[0] = ekey(m0, m1);
            IE[1] = ekey(m1, m2);
            IE[2] = ekey(m2, m0);
            fb[m0] = fb[m1] = fb[m2] = 1;
        }
    } else if constexpr (T == UG4GB_TET) {
        const int m01 = lk.mid(ev[0], ev[1]), m12 = lk.mid(ev[1], ev[2]), m02 = lk.mid(ev[0], ev[2]);
        const int m03 = lk.mid(ev[0], ev[3]), m13 = lk.mid(ev[1], ev[3]), m23 = lk.mid(ev[2], ev[3]);
        const int corner[4][4] = {{ev[0], m01, m02, m03}, {m01, ev[1], m12, m13}, {m02, m12, ev[2], m23},
                                  {m03, m13, m23, ev[3]}};
        for (int q = 0; q < 4; ++q)
            for (int j = 0; j < 4; ++j) ch[q][j] = corner[q][j];
        // the inner octahedron, cut along its shortest diagonal
        const int diag[3][2] = {{m01, m23}, {m12, m03}, {m02, m13}};
        const int ring[3][4] = {{m12, m13, m03, m02}, {m01, m13, m23, m02}, {m01, m12, m23, m03}};
        const int best = tet_best_diagonal(fc, diag);
        for (int q = 0; q < 4; ++q) {
            ch[4 + q][0] = diag[best][0];
            ch[4 + q][1] = diag[best][1];
            ch[4 + q][2] = ring[best][q];
            ch[4 + q][3] = ring[best][(q + 1) % 4];
        }
        if (ed) {
            IE[0] = ekey(diag[best][0], diag[best][1]);
            for (int q = 0; q < 4; ++q) {
                IF[2 * q] = make_int4(diag[best][0], diag[best][1], ring[best][q], -1);
                int fm[3], n = 0;
                for (int j = 0; j < 4; ++j)
                    if (corner[q][j] != ev[q]) fm[n++] = corner[q][j];
                IF[2 * q + 1] = make_int4(fm[0], fm[1], fm[2], -1);
            }
            fb[m01] = fb[m12] = fb[m02] = fb[m03] = fb[m13] = fb[m23] = 1;
        }
    } else {
        // tensor sub-boxes: the point of child corner j is the parent object
        // spanned by the coordinates that are 1/2 in half units
        for (int q = 0; q < NCH; ++q)
            for (int j = 0; j < K; ++j) {
                int h[3];
                for (int d = 0; d < DIM; ++d) {
                    const int r = (DIM == 2) ? c_quad_ref[j][d] : c_hex_ref[j][d];
                    h[d] = ((q >> d) & 1) + r;
                }
                int cs[8], n = 0;
                for (int i = 0; i < K; ++i) {
                    bool in = true;
                    for (int d = 0; d < DIM; ++d) {
                        const int r = 2 * ((DIM == 2) ? c_quad_ref[i][d] : c_hex_ref[i][d]);
                        if (h[d] != 1 && h[d] != r) in = false;
                    }
                    if (in) cs[n++] = ev[i];
                }
                int v;
                if (n == 1) v = cs[0];
                else if (n == 2) v = lk.mid(cs[0], cs[1]);
                else if (n == 4) v = (T == UG4GB_QUAD) ? nqf_base + e : lk.qcentre(cs);
                else v = cen_base + e;
                ch[q][j] = v;
            }
        if constexpr (T == UG4GB_QUAD) {
            if (ed) {
                const int z = nqf_base + e;
                fb[z] = 1;
                for (int j = 0; j < 4; ++j) {
                    const int m = lk.mid(ev[c_quad_edges[j][0]], ev[c_quad_edges[j][1]]);
                    fb[m] = 1;
                    IE[j] = ekey(z, m);
                }
            }
        } else if (ed) {
            const int z = cen_base + e;
            fb[z] = 1;
            for (int j = 0; j < 12; ++j) fb[lk.mid(ev[c_hex_edges[j][0]], ev[c_hex_edges[j][1]])] = 1;
            for (int f = 0; f < 6; ++f) {
                int qf[4];
                for (int j = 0; j < 4; ++j) qf[j] = ev[c_hex_faces[f][j]];
                const int fcen = lk.qcentre(qf);
                fb[fcen] = 1;
                IE[f] = ekey(z, fcen);
            }
            // the 12 inner faces: edge mid point, face centre, centre, face centre
            for (int j = 0; j < 12; ++j) {
                const int a = c_hex_edges[j][0], b = c_hex_edges[j][1];
                const int m = lk.mid(ev[a], ev[b]);
                int fcs[2] = {0, 0}, n = 0;
                for (int f = 0; f < 6 && n < 2; ++f) {
                    int has = 0;
                    for (int x = 0; x < 4; ++x) has += (c_hex_faces[f][x] == a || c_hex_faces[f][x] == b);
                    if (has == 2) {
                        int qf[4];
                        for (int x = 0; x < 4; ++x) qf[x] = ev[c_hex_faces[f][x]];
                        fcs[n++] = lk.qcentre(qf);
                    }
                }
                IF[j] = make_int4(m, fcs[0], z, fcs[1]);
            }
        }
    }
    for (int q = 0; q < NCH; ++q) {
        orient_child(fc, DIM, T, ch[q]);
        int *out = felems + ((size_t)e * NCH + q) * K;
        for (int j = 0; j < K; ++j) out[j] = ch[q][j];
        fedir[(size_t)e * NCH + q] = cedir[e];
    }
}

// children of the Dirichlet edges: (a, m), (m, b)
__global__ void k_dir_edge_children(const u64 *dir, int n, Lookup lk, u64 *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int a = (int)(dir[i] >> 32), b = (int)(dir[i] & 0xffffffffULL);
    const int m = lk.mid(a, b);
    out[2 * (size_t)i] = ekey(a, m);
    out[2 * (size_t)i + 1] = ekey(m, b);
}

// children and inner edges of the Dirichlet faces (4 edge slots, 4 faces each)
__global__ void k_dir_face_children(const int4 *dir, int n, Lookup lk, unsigned char *fb, u64 *oute, int4 *outf)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int4 f = dir[i];
    u64 *e = oute + 4 * (size_t)i;
    int4 *g = outf + 4 * (size_t)i;
    if (f.w < 0) {
        const int a = f.x, b = f.y, c = f.z;
        const int mab = lk.mid(a, b), mbc = lk.mid(b, c), mca = lk.mid(c, a);
        fb[mab] = fb[mbc] = fb[mca] = 1;
        e[0] = ekey(mab, mbc);
        e[1] = ekey(mbc, mca);
        e[2] = ekey(mca, mab);
        e[3] = kNoKey;
        g[0] = make_int4(a, mab, mca, -1);
        g[1] = make_int4(mab, b, mbc, -1);
        g[2] = make_int4(mca, mbc, c, -1);
        g[3] = make_int4(mab, mbc, mca, -1);
    } else {
        const int q[4] = {f.x, f.y, f.z, f.w};
        const int z = lk.qcentre(q);
        int m[4];
        for (int j = 0; j < 4; ++j) m[j] = lk.mid(q[j], q[(j + 1) % 4]);
        fb[z] = 1;
        for (int j = 0; j < 4; ++j) {
            fb[m[j]] = 1;
            e[j] = ekey(z, m[j]);
        }
        g[0] = make_int4(q[0], m[0], z, m[3]);
        g[1] = make_int4(m[0], q[1], m[1], z);
        g[2] = make_int4(z, m[1], q[2], m[2]);
        g[3] = make_int4(m[3], z, m[2], q[3]);
    }
}

__global__ void k_elem_obj_counts(const unsigned char *edir, int ne, int t, int *ce, int *cf)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int on = edir[e] ? 1 : 0;
    const int ned = t == UG4GB_TRI ? 3 : (t == UG4GB_QUAD ? 4 : (t == UG4GB_TET ? 1 : 6));
    const int nf = t == UG4GB_TET ? 8 : (t == UG4GB_HEX ? 12 : 0);
    ce[e] = on * ned;
    cf[e] = on * nf;
}

// sorted-key (hi, lo) of a face
__global__ void k_face_sortkeys(const int4 *f, int n, u64 *hi, u64 *lo, int *idx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int s[4] = {f[i].x, f[i].y, f[i].z, f[i].w};
    sort4(s);   // -1 (triangle) first; stored shifted by one
    hi[i] = ((u64)(unsigned)(s[0] + 1) << 32) | (u64)(unsigned)(s[1] + 1);
    lo[i] = ((u64)(unsigned)(s[2] + 1) << 32) | (u64)(unsigned)(s[3] + 1);
    idx[i] = i;
}

__global__ void k_first_of_run(const u64 *hi, const u64 *lo, int n, unsigned char *flag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (i == 0 || hi[i] != hi[i - 1] || lo[i] != lo[i - 1]) ? 1 : 0;
}

__global__ void k_iota(int *p, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = i;
}

__global__ void k_gather_faces(const int4 *in, const int *idx, int n, int4 *out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[idx[i]];
}

__global__ void k_gather_pairs(const u64 *hi, const u64 *lo, const int *idx, int n, u64 *ho, u64 *lo_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        ho[i] = hi[idx[i]];
        lo_out[i] = lo[idx[i]];
    }
}

int grid1(int64_t n) { return (int)div_up(n > 0 ? n : 1, 256); }

// keys sorted and made unique; kNoKey entries dropped; returns the count
int sort_unique_keys(Ctx &c, DevBuf<u64> &keys, int n, DevBuf<u64> &out)
{
    out.alloc(n > 0 ? n : 1);
    if (n == 0) return 0;
    DevBuf<u64> sorted;
    sorted.alloc(n);
    DevBuf<int> cnt;
    cnt.alloc(1);
    size_t b1 = 0, b2 = 0;
    UG_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, b1, keys.p, sorted.p, n, 0, 64, c.stream));
    UG_CUDA(cub::DeviceSelect::Unique(nullptr, b2, sorted.p, out.p, cnt.p, n, c.stream));
    DevBuf<unsigned char> tmp;
    tmp.alloc(std::max(b1, b2) + 1);
    UG_CUDA(cub::DeviceRadixSort::SortKeys(tmp.p, b1, keys.p, sorted.p, n, 0, 64, c.stream));
    UG_CUDA(cub::DeviceSelect::Unique(tmp.p, b2, sorted.p, out.p, cnt.p, n, c.stream));
    int m = 0;
    UG_CUDA(cudaMemcpyAsync(&m, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    if (m > 0) {
        u64 last = 0;
        UG_CUDA(cudaMemcpyAsync(&last, out.p + m - 1, sizeof(u64), cudaMemcpyDeviceToHost, c.stream));
        UG_CUDA(cudaStreamSynchronize(c.stream));
        if (last == kNoKey) --m;
    }
    return m;
}

// (hi, lo) pairs stably sorted by (hi, lo); idx = their original positions
void sort_pairs128(Ctx &c, DevBuf<u64> &hi, DevBuf<u64> &lo, DevBuf<int> &idx, int n)
{
    if (n == 0) return;
    DevBuf<u64> k2;
    DevBuf<int> i2;
    k2.alloc(n);
    i2.alloc(n);
    size_t b = 0;
    UG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, b, lo.p, k2.p, idx.p, i2.p, n, 0, 64, c.stream));
    DevBuf<unsigned char> tmp;
    tmp.alloc(b + 1);
    // by lo, then stably by hi
    UG_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, b, lo.p, k2.p, idx.p, i2.p, n, 0, 64, c.stream));
    DevBuf<u64> h2;
    h2.alloc(n);
    UG_LAUNCH(c, k_gather_pairs, grid1(n), 256, 0, hi.p, lo.p, i2.p, n, h2.p, k2.p);
    DevBuf<u64> h3;
    h3.alloc(n);
    UG_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, b, h2.p, h3.p, i2.p, idx.p, n, 0, 64, c.stream));
    UG_LAUNCH(c, k_gather_pairs, grid1(n), 256, 0, hi.p, lo.p, idx.p, n, h2.p, k2.p);
    UG_CUDA(cudaMemcpyAsync(hi.p, h2.p, sizeof(u64) * (size_t)n, cudaMemcpyDeviceToDevice, c.stream));
    UG_CUDA(cudaMemcpyAsync(lo.p, k2.p, sizeof(u64) * (size_t)n, cudaMemcpyDeviceToDevice, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));   // before the temporaries are freed
}

// indices of the first entry of each run of equal (hi, lo); returns the count
int first_of_runs(Ctx &c, const DevBuf<u64> &hi, const DevBuf<u64> &lo, const DevBuf<int> &idx, int n,
                  DevBuf<int> &sel)
{
    sel.alloc(n > 0 ? n : 1);
    if (n == 0) return 0;
    DevBuf<unsigned char> flag;
    flag.alloc(n);
    DevBuf<int> cnt;
    cnt.alloc(1);
    UG_LAUNCH(c, k_first_of_run, grid1(n), 256, 0, hi.p, lo.p, n, flag.p);
    size_t b = 0;
    UG_CUDA(cub::DeviceSelect::Flagged(nullptr, b, idx.p, flag.p, sel.p, cnt.p, n, c.stream));
    DevBuf<unsigned char> tmp;
    tmp.alloc(b + 1);
    UG_CUDA(cub::DeviceSelect::Flagged(tmp.p, b, idx.p, flag.p, sel.p, cnt.p, n, c.stream));
    int m = 0;
    UG_CUDA(cudaMemcpyAsync(&m, cnt.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    return m;
}

void check_flag(Ctx &c, const DevBuf<int> &err, const char *what)
{
    int h = 0;
    UG_CUDA(cudaMemcpyAsync(&h, err.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    UG_REQUIRE(!h, UG4GB_ERR_INVALID, what);
}

}  // namespace

void refine_device(Ctx &c, const Level &C, const DevDir &Cd, Level &F, DevDir &Fd)
{
    const int t = C.elem_type, k = C.k, dim = C.dim, ne = C.ne, nv = C.nv;
    const int ned = (t == UG4GB_TRI) ? 3 : (t == UG4GB_QUAD ? 4 : (t == UG4GB_TET ? 6 : 12));
    DevBuf<int> err;
    err.alloc(1);
    UG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), c.stream));
    // edges, numbered in (smaller, larger) vertex order
    DevBuf<u64> E;
    const int64_t nk = (int64_t)ne * ned;
    UG_REQUIRE(nk < ((int64_t)1 << 31), UG4GB_ERR_INVALID, "refinement: too many element edges");
    int nedge = 0;
    {
        DevBuf<u64> keys;
        keys.alloc(nk);
        UG_LAUNCH(c, k_edge_keys, grid1(nk), 256, 0, C.elems.p, ne, k, t, keys.p);
        nedge = sort_unique_keys(c, keys, (int)nk, E);
    }
    // quadrilateral faces of hexahedra, numbered in sorted-corner order
    DevBuf<u64> FH, FL;
    int nqf = 0, nqf_keys = 0;
    if (t == UG4GB_HEX) {
        const int nf = ne * 6;
        DevBuf<u64> hi, lo;
        DevBuf<int> idx, pos, sel;
        hi.alloc(nf);
        lo.alloc(nf);
        idx.alloc(nf);
        pos.alloc(nf);
        UG_LAUNCH(c, k_hex_face_keys, grid1(nf), 256, 0, C.elems.p, ne, hi.p, lo.p, idx.p);
        sort_pairs128(c, hi, lo, idx, nf);
        UG_LAUNCH(c, k_iota, grid1(nf), 256, 0, pos.p, nf);
        nqf = nqf_keys = first_of_runs(c, hi, lo, pos, nf, sel);
        FH.alloc(nqf > 0 ? nqf : 1);
        FL.alloc(nqf > 0 ? nqf : 1);
        UG_LAUNCH(c, k_gather_pairs, grid1(nqf), 256, 0, hi.p, lo.p, sel.p, nqf, FH.p, FL.p);
        UG_CUDA(cudaStreamSynchronize(c.stream));   // before the temporaries are freed
    } else if (t == UG4GB_QUAD) {
        nqf = ne;
    }
    const int ncen = (t == UG4GB_HEX) ? ne : 0;
    const int64_t nv64 = (int64_t)nv + nedge + nqf + ncen;
    UG_REQUIRE(nv64 < ((int64_t)1 << 31), UG4GB_ERR_INVALID, "refinement: too many vertices for 32-bit indices");
    const int nch = (dim == 2) ? 4 : 8;
    const int64_t ne64 = (int64_t)ne * nch;
    UG_REQUIRE(ne64 * k < ((int64_t)1 << 31), UG4GB_ERR_INVALID, "refinement: too many elements for 32-bit indices");
    F.elem_type = t;
    F.dim = dim;
    F.k = k;
    F.nv = (int)nv64;
    F.ne = (int)ne64;
    F.nx = F.ny = F.nz = 0;
    F.structured = false;
    F.coords.alloc((size_t)F.nv * dim);
    F.elems.alloc((size_t)F.ne * k);
    F.bnd.alloc(F.nv);
    F.npar.alloc(F.nv);
    F.par.alloc((size_t)F.nv * 8);
    // vertices: old ones, edge mid points, face centres, element centres
    UG_LAUNCH(c, k_old_vertices, grid1(nv), 256, 0, C.coords.p, C.bnd.p, nv, dim, F.coords.p, F.bnd.p, F.npar.p,
              F.par.p);
    if (nedge > 0)
        UG_LAUNCH(c, k_edge_vertices, grid1(nedge), 256, 0, E.p, nedge, C.coords.p, nv, dim, F.coords.p, F.bnd.p,
                  F.npar.p, F.par.p);
    if (t == UG4GB_HEX) {
        if (nqf > 0)
            UG_LAUNCH(c, k_face_vertices, grid1(nqf), 256, 0, FH.p, FL.p, nqf, C.coords.p, nv + nedge, F.coords.p,
                      F.bnd.p, F.npar.p, F.par.p);
        UG_LAUNCH(c, k_elem_centres, grid1(ne), 256, 0, C.elems.p, ne, 8, C.coords.p, 3, nv + nedge + nqf,
                  F.coords.p, F.bnd.p, F.npar.p, F.par.p);
    } else if (t == UG4GB_QUAD) {
        UG_LAUNCH(c, k_elem_centres, grid1(ne), 256, 0, C.elems.p, ne, 4, C.coords.p, 2, nv + nedge, F.coords.p,
                  F.bnd.p, F.npar.p, F.par.p);
    }
    Lookup lk{E.p, nedge, FH.p, FL.p, nqf_keys, nv, err.p};
    // Dirichlet vertices: mid points of the Dirichlet edges
    if (Cd.n_edges > 0)
        UG_LAUNCH(c, k_mark_dir_edges, grid1(Cd.n_edges), 256, 0, Cd.edges.p, Cd.n_edges, E.p, nedge, nv, F.bnd.p,
                  err.p);
    // Dirichlet objects of the fine level: children of the Dirichlet edges and
    // faces, then the objects created inside Dirichlet elements (element order)
    DevBuf<int> ce, cf, pe, pf;
    ce.alloc(ne + 1);
    cf.alloc(ne + 1);
    pe.alloc(ne + 1);
    pf.alloc(ne + 1);
    UG_CUDA(cudaMemsetAsync(ce.p + ne, 0, sizeof(int), c.stream));
    UG_CUDA(cudaMemsetAsync(cf.p + ne, 0, sizeof(int), c.stream));
    UG_LAUNCH(c, k_elem_obj_counts, grid1(ne), 256, 0, Cd.edir.p, ne, t, ce.p, cf.p);
    int64_t n_ie = 0, n_if = 0;
    exclusive_scan_int(c, ce.p, pe.p, ne + 1, &n_ie);
    exclusive_scan_int(c, cf.p, pf.p, ne + 1, &n_if);
    const int n_de = 2 * Cd.n_edges, n_fe = 4 * Cd.n_faces, n_ff = 4 * Cd.n_faces;
    const int64_t n_all_e = (int64_t)n_de + n_fe + n_ie, n_all_f = (int64_t)n_ff + n_if;
    UG_REQUIRE(n_all_e < ((int64_t)1 << 31) && n_all_f < ((int64_t)1 << 31), UG4GB_ERR_INVALID,
               "refinement: too many Dirichlet objects");
    DevBuf<u64> ekeys;
    DevBuf<int4> faces;
    ekeys.alloc(n_all_e > 0 ? n_all_e : 1);
    faces.alloc(n_all_f > 0 ? n_all_f : 1);
    if (Cd.n_edges > 0)
        UG_LAUNCH(c, k_dir_edge_children, grid1(Cd.n_edges), 256, 0, Cd.edges.p, Cd.n_edges, lk, ekeys.p);
    if (Cd.n_faces > 0)
        UG_LAUNCH(c, k_dir_face_children, grid1(Cd.n_faces), 256, 0, Cd.faces.p, Cd.n_faces, lk, F.bnd.p,
                  ekeys.p + n_de, faces.p);
    // children (the inner Dirichlet objects before orientation, as the cut was made)
    Fd.edir.alloc(F.ne);
    const int qbase = nv + nedge, cbase = nv + nedge + nqf;
    u64 *oe = ekeys.p + n_de + n_fe;
    int4 *of = faces.p + n_ff;
#define UG_CHILDREN(TT)                                                                                            \
    UG_LAUNCH(c, k_children<TT>, (int)div_up(ne, 128), 128, 0, C.elems.p, ne, Cd.edir.p, lk, qbase, cbase, F.coords.p,       \
              F.elems.p, Fd.edir.p, pe.p, pf.p, oe, of, F.bnd.p)
    switch (t) {
        case UG4GB_TRI: UG_CHILDREN(UG4GB_TRI); break;
        case UG4GB_QUAD: UG_CHILDREN(UG4GB_QUAD); break;
        case UG4GB_TET: UG_CHILDREN(UG4GB_TET); break;
        default: UG_CHILDREN(UG4GB_HEX); break;
    }
#undef UG_CHILDREN
    check_flag(c, err, "refinement: an edge or face of the grid was not found (non-conforming input)");
    Fd.n_edges = sort_unique_keys(c, ekeys, (int)n_all_e, Fd.edges);
    // faces: unique by their sorted corners, the first occurrence kept
    if (n_all_f > 0) {
        const int n = (int)n_all_f;
        DevBuf<u64> hi, lo;
        DevBuf<int> idx, sel;
        hi.alloc(n);
        lo.alloc(n);
        idx.alloc(n);
        UG_LAUNCH(c, k_face_sortkeys, grid1(n), 256, 0, faces.p, n, hi.p, lo.p, idx.p);
        sort_pairs128(c, hi, lo, idx, n);
        Fd.n_faces = first_of_runs(c, hi, lo, idx, n, sel);
        Fd.faces.alloc(Fd.n_faces > 0 ? Fd.n_faces : 1);
        UG_LAUNCH(c, k_gather_faces, grid1(Fd.n_faces), 256, 0, faces.p, sel.p, Fd.n_faces, Fd.faces.p);
        UG_CUDA(cudaStreamSynchronize(c.stream));   // before the temporaries are freed
    } else {
        Fd.n_faces = 0;
        Fd.faces.alloc(1);
    }
    UG_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace ug4gb

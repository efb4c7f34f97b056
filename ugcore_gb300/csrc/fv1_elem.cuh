// fv1_elem.cuh -- per-element FV1 geometry and element matrix (device code).
//
// Reference-element tables (lib_disc/reference_element/reference_element.cpp:
// triangle :320-420, quadrilateral :428, tetrahedron :547, hexahedron :1327)
// are packed as 4-bit nibbles in 64-bit literals so that, with every element
// loop unrolled, each table lookup is a compile-time constant and the element
// matrix stays in registers (a dynamic index would spill it to local memory).
#pragma once

#include "common.cuh"

namespace ug4gb {

__host__ __device__ constexpr int nib(unsigned long long w, int i) { return (int)((w >> (4 * i)) & 15ULL); }
__host__ __device__ constexpr int nib2(unsigned long long lo, unsigned long long hi, int i)
{
    return i < 16 ? nib(lo, i) : nib(hi, i - 16);
}

template <int T>
struct Elem;

// quadrilateral: corners (0,0),(1,0),(1,1),(0,1); edges (0,1),(1,2),(2,3),(3,0)
template <>
struct Elem<UG4GB_QUAD> {
    static constexpr int DIM = 2, K = 4, NSCVF = 4, NFACE = 0;
    __host__ __device__ static constexpr int from(int e) { return nib(0x3210ULL, e); }
    __host__ __device__ static constexpr int to(int e) { return nib(0x0321ULL, e); }
    // edges at each corner [edge0, edge1]: {3,0},{0,1},{1,2},{2,3}
    __host__ __device__ static constexpr int pt_edge(int i, int q) { return nib(0x32211003ULL, 2 * i + q); }
    __host__ __device__ static constexpr double corner(int i, int d)
    {
        return (double)(((d == 0 ? 0x6 : 0xC) >> i) & 1);
    }
    __host__ __device__ static constexpr int face_n() { return 0; }
    __host__ __device__ static constexpr int face(int, int) { return 0; }
    __host__ __device__ static constexpr int edge_face(int, int) { return 0; }
    __host__ __device__ static constexpr int pt_face(int, int) { return 0; }
};

// triangle: corners (0,0),(1,0),(0,1); edges (0,1),(1,2),(2,0)
// (reference_element.cpp, ReferenceTriangle)
template <>
struct Elem<UG4GB_TRI> {
    static constexpr int DIM = 2, K = 3, NSCVF = 3, NFACE = 0;
    __host__ __device__ static constexpr int from(int e) { return nib(0x210ULL, e); }
    __host__ __device__ static constexpr int to(int e) { return nib(0x021ULL, e); }
    // edges at each corner [edge0, edge1]: {2,0},{0,1},{1,2}
    __host__ __device__ static constexpr int pt_edge(int i, int q) { return nib(0x211002ULL, 2 * i + q); }
    __host__ __device__ static constexpr double corner(int i, int d)
    {
        return (double)(((d == 0 ? 0x2 : 0x4) >> i) & 1);
    }
    __host__ __device__ static constexpr int face_n() { return 0; }
    __host__ __device__ static constexpr int face(int, int) { return 0; }
    __host__ __device__ static constexpr int edge_face(int, int) { return 0; }
    __host__ __device__ static constexpr int pt_face(int, int) { return 0; }
};

// hexahedron: reference corners 0..7; edges 0..11; faces 0..5
template <>
struct Elem<UG4GB_HEX> {
    static constexpr int DIM = 3, K = 8, NSCVF = 12, NFACE = 6;
    // from: 0,1,2,3,0,1,2,3,4,5,6,7   to: 1,2,3,0,4,5,6,7,5,6,7,4
    __host__ __device__ static constexpr int from(int e) { return nib(0x765432103210ULL, e); }
    __host__ __device__ static constexpr int to(int e) { return nib(0x476576540321ULL, e); }
    // sides of edge e: s0 = 0,0,0,0,1,2,3,4,1,2,3,4  s1 = 1,2,3,4,4,1,2,3,5,5,5,5
    __host__ __device__ static constexpr int edge_face(int e, int q)
    {
        return q == 0 ? nib(0x432143210000ULL, e) : nib(0x555532144321ULL, e);
    }
    // faces: (0,3,2,1)(0,1,5,4)(1,2,6,5)(2,3,7,6)(3,0,4,7)(4,5,6,7)
    __host__ __device__ static constexpr int face(int f, int j)
    {
        return nib2(0x6732562145101230ULL, 0x76547403ULL, 4 * f + j);
    }
    __host__ __device__ static constexpr int face_n() { return 4; }
    // edges at corner i: {3,0,4},{0,1,5},{1,2,6},{2,3,7},{4,8,11},{5,9,8},{6,10,9},{7,11,10}
    __host__ __device__ static constexpr int pt_edge(int i, int q)
    {
        return nib2(0x5B84732621510403ULL, 0xAB79A689ULL, 3 * i + q);
    }
    // faces at corner i: {0,4,1},{0,1,2},{0,2,3},{0,3,4},{1,4,5},{2,1,5},{3,2,5},{4,3,5}
    __host__ __device__ static constexpr int pt_face(int i, int q)
    {
        return nib2(0x2541430320210140ULL, 0x53452351ULL, 3 * i + q);
    }
    __host__ __device__ static constexpr double corner(int i, int d)
    {
        return (double)(((d == 0 ? 0x66 : (d == 1 ? 0xCC : 0xF0)) >> i) & 1);
    }
};

// tetrahedron: corners (0,0,0),(1,0,0),(0,1,0),(0,0,1)
template <>
struct Elem<UG4GB_TET> {
    static constexpr int DIM = 3, K = 4, NSCVF = 6, NFACE = 4;
    // edges (0,1),(1,2),(2,0),(0,3),(1,3),(2,3)
    __host__ __device__ static constexpr int from(int e) { return nib(0x210210ULL, e); }
    __host__ __device__ static constexpr int to(int e) { return nib(0x333021ULL, e); }
    // sides of edge e: s0 = 0,0,0,3,1,2  s1 = 3,1,2,2,3,1
    __host__ __device__ static constexpr int edge_face(int e, int q)
    {
        return q == 0 ? nib(0x213000ULL, e) : nib(0x132213ULL, e);
    }
    // faces (0,2,1),(1,2,3),(0,3,2),(0,1,3)
    __host__ __device__ static constexpr int face(int f, int j) { return nib(0x310230321120ULL, 3 * f + j); }
    __host__ __device__ static constexpr int face_n() { return 3; }
    // edges at corner: {2,0,3},{0,1,4},{1,2,5},{3,4,5}
    __host__ __device__ static constexpr int pt_edge(int i, int q) { return nib(0x543521410302ULL, 3 * i + q); }
    // faces at corner: {0,2,3},{0,3,1},{0,1,2},{3,2,1}
    __host__ __device__ static constexpr int pt_face(int i, int q) { return nib(0x123210130320ULL, 3 * i + q); }
    __host__ __device__ static constexpr double corner(int i, int d) { return (i == d + 1) ? 1.0 : 0.0; }
};

// local gradient of P1 shape sh at local position xi
template <int T>
__host__ __device__ __forceinline__ void local_grad(const double *xi, int sh, double *g)
{
    if constexpr (T == UG4GB_TRI) {
        g[0] = (sh == 0) ? -1.0 : (sh == 1 ? 1.0 : 0.0);
        g[1] = (sh == 0) ? -1.0 : (sh == 2 ? 1.0 : 0.0);
    } else if constexpr (T == UG4GB_QUAD) {
        double cx = Elem<T>::corner(sh, 0), cy = Elem<T>::corner(sh, 1);
        double fx = cx ? xi[0] : 1.0 - xi[0], fy = cy ? xi[1] : 1.0 - xi[1];
        g[0] = (cx ? 1.0 : -1.0) * fy;
        g[1] = fx * (cy ? 1.0 : -1.0);
    } else if constexpr (T == UG4GB_HEX) {
        double cx = Elem<T>::corner(sh, 0), cy = Elem<T>::corner(sh, 1), cz = Elem<T>::corner(sh, 2);
        double fx = cx ? xi[0] : 1.0 - xi[0], fy = cy ? xi[1] : 1.0 - xi[1], fz = cz ? xi[2] : 1.0 - xi[2];
        double dx = cx ? 1.0 : -1.0, dy = cy ? 1.0 : -1.0, dz = cz ? 1.0 : -1.0;
        g[0] = dx * fy * fz;
        g[1] = fx * dy * fz;
        g[2] = fx * fy * dz;
    } else {
        g[0] = (sh == 0) ? -1.0 : (sh == 1 ? 1.0 : 0.0);
        g[1] = (sh == 0) ? -1.0 : (sh == 2 ? 1.0 : 0.0);
        g[2] = (sh == 0) ? -1.0 : (sh == 3 ? 1.0 : 0.0);
    }
}

// local SCVF integration point (patch average in reference coordinates)
template <int T>
__host__ __device__ __forceinline__ void local_ip(int e, double *xi)
{
    using E = Elem<T>;
    const int a = E::from(e), b = E::to(e);
    double mid[3], cen[3];
    for (int d = 0; d < E::DIM; ++d) {
        mid[d] = (E::corner(a, d) + E::corner(b, d)) * 0.5;
        double s = 0.0;
        for (int i = 0; i < E::K; ++i) s += E::corner(i, d);
        cen[d] = s * (1.0 / E::K);
    }
    if constexpr (E::DIM == 2) {
        for (int d = 0; d < 2; ++d) xi[d] = (mid[d] + cen[d]) * 0.5;
    } else {
        const int f0 = E::edge_face(e, 0), f1 = E::edge_face(e, 1), nf = E::face_n();
        for (int d = 0; d < 3; ++d) {
            double s0 = 0.0, s1 = 0.0;
            for (int j = 0; j < nf; ++j) {
                s0 += E::corner(E::face(f0, j), d);
                s1 += E::corner(E::face(f1, j), d);
            }
            xi[d] = (mid[d] + s0 * (1.0 / nf) + cen[d] + s1 * (1.0 / nf)) * 0.25;
        }
    }
}

struct VelField {
    int nmodes;
    const double *k, *c, *phase;
    double scale;
    __device__ __forceinline__ void eval(const double *x, double *v) const
    {
        v[0] = v[1] = v[2] = 0.0;
        for (int m = 0; m < nmodes; ++m) {
            double s = -sin(__ldg(phase + m) + __ldg(k + 3 * m) * x[0] + __ldg(k + 3 * m + 1) * x[1] +
                            __ldg(k + 3 * m + 2) * x[2]);
            v[0] += s * __ldg(c + 3 * m);
            v[1] += s * __ldg(c + 3 * m + 1);
            v[2] += s * __ldg(c + 3 * m + 2);
        }
        v[0] *= scale;
        v[1] *= scale;
        v[2] *= scale;
    }
};

// (J^T)^{-1} from corner coordinates and local gradients at one point
template <int T>
__device__ __forceinline__ void jt_inverse(const double (&X)[Elem<T>::K][Elem<T>::DIM], const double *xi,
                                           double (&Ji)[3][3])
{
    using E = Elem<T>;
    double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        double lg[3];
        local_grad<T>(xi, i, lg);
#pragma unroll
        for (int a = 0; a < E::DIM; ++a)
#pragma unroll
            for (int b = 0; b < E::DIM; ++b) J[a][b] += X[i][a] * lg[b];
    }
    if constexpr (E::DIM == 2) {
        double inv = 1.0 / (J[0][0] * J[1][1] - J[0][1] * J[1][0]);
        Ji[0][0] = J[1][1] * inv;
        Ji[0][1] = -J[1][0] * inv;
        Ji[1][0] = -J[0][1] * inv;
        Ji[1][1] = J[0][0] * inv;
    } else {
        double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        double inv = 1.0 / (J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02);
        // Ji = (J^{-1})^T
        Ji[0][0] = c00 * inv;
        Ji[1][0] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * inv;
        Ji[2][0] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * inv;
        Ji[0][1] = c01 * inv;
        Ji[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * inv;
        Ji[2][1] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * inv;
        Ji[0][2] = c02 * inv;
        Ji[1][2] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * inv;
        Ji[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * inv;
    }
}

template <int T>
__device__ __forceinline__ void edge_mid(const double (&X)[Elem<T>::K][Elem<T>::DIM], int e, double *m)
{
    using E = Elem<T>;
#pragma unroll
    for (int d = 0; d < E::DIM; ++d) m[d] = (X[E::from(e)][d] + X[E::to(e)][d]) * 0.5;
}

template <int T>
__device__ __forceinline__ void face_mid(const double (&X)[Elem<T>::K][Elem<T>::DIM], int f, double *m)
{
    using E = Elem<T>;
    constexpr int nf = E::face_n();
#pragma unroll
    for (int d = 0; d < E::DIM; ++d) {
        double s = X[E::face(f, 0)][d];
#pragma unroll
        for (int j = 1; j < nf; ++j) s += X[E::face(f, j)][d];
        m[d] = s * (1.0 / nf);
    }
}

template <int T>
__device__ __forceinline__ void elem_centre(const double (&X)[Elem<T>::K][Elem<T>::DIM], double *m)
{
    using E = Elem<T>;
#pragma unroll
    for (int d = 0; d < E::DIM; ++d) {
        double s = X[0][d];
#pragma unroll
        for (int i = 1; i < E::K; ++i) s += X[i][d];
        m[d] = s * (1.0 / E::K);
    }
}

__device__ __forceinline__ double hex_size(const double (&c)[8][3])
{
    double x50[3], x14[3], x10[3], x20[3], x60[3], x24[3], x30[3], x70[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        x50[d] = c[5][d] - c[0][d]; x14[d] = c[1][d] - c[4][d]; x10[d] = c[1][d] - c[0][d];
        x20[d] = c[2][d] - c[0][d]; x60[d] = c[6][d] - c[0][d]; x24[d] = c[2][d] - c[4][d];
        x30[d] = c[3][d] - c[0][d]; x70[d] = c[7][d] - c[0][d];
    }
    double n1[3], n2[3];
    n1[0] = (x10[1] * x20[2] - x10[2] * x20[1]) + (x50[1] * x14[2] - x50[2] * x14[1]);
    n1[1] = (x10[2] * x20[0] - x10[0] * x20[2]) + (x50[2] * x14[0] - x50[0] * x14[2]);
    n1[2] = (x10[0] * x20[1] - x10[1] * x20[0]) + (x50[0] * x14[1] - x50[1] * x14[0]);
    n2[0] = (x20[1] * x30[2] - x20[2] * x30[1]) + (x60[1] * x24[2] - x60[2] * x24[1]);
    n2[1] = (x20[2] * x30[0] - x20[0] * x30[2]) + (x60[2] * x24[0] - x60[0] * x24[2]);
    n2[2] = (x20[0] * x30[1] - x20[1] * x30[0]) + (x60[0] * x24[1] - x60[1] * x24[0]);
    return (1.0 / 6.0) * ((n1[0] * x60[0] + n1[1] * x60[1] + n1[2] * x60[2]) +
                          (n2[0] * x70[0] + n2[1] * x70[1] + n2[2] * x70[2]));
}

// SCV volumes (ElementSize of the SCV quadrilateral / hexahedron)
template <int T>
__device__ __forceinline__ void scv_volumes(const double (&X)[Elem<T>::K][Elem<T>::DIM], double *vol)
{
    using E = Elem<T>;
    double gm[3];
    elem_centre<T>(X, gm);
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        if constexpr (E::DIM == 2) {
            double e0[3], e1[3];
            edge_mid<T>(X, E::pt_edge(i, 0), e0);
            edge_mid<T>(X, E::pt_edge(i, 1), e1);
            // q = [corner, e0, centre, e1]
            vol[i] = 0.5 * fabs((e1[1] - e0[1]) * (gm[0] - X[i][0]) - (e1[0] - e0[0]) * (gm[1] - X[i][1]));
        } else {
            double c[8][3];
            double t[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) c[0][d] = X[i][d];
            edge_mid<T>(X, E::pt_edge(i, 1), t); for (int d = 0; d < 3; ++d) c[1][d] = t[d];
            face_mid<T>(X, E::pt_face(i, 0), t); for (int d = 0; d < 3; ++d) c[2][d] = t[d];
            edge_mid<T>(X, E::pt_edge(i, 0), t); for (int d = 0; d < 3; ++d) c[3][d] = t[d];
            edge_mid<T>(X, E::pt_edge(i, 2), t); for (int d = 0; d < 3; ++d) c[4][d] = t[d];
            face_mid<T>(X, E::pt_face(i, 2), t); for (int d = 0; d < 3; ++d) c[5][d] = t[d];
            for (int d = 0; d < 3; ++d) c[6][d] = gm[d];
            face_mid<T>(X, E::pt_face(i, 1), t); for (int d = 0; d < 3; ++d) c[7][d] = t[d];
            vol[i] = hex_size(c);
        }
    }
}

// element matrix of -div(K grad u) + div(v u) (full upwind), FP64
template <int T>
__device__ __forceinline__ void elem_matrix(const double (&X)[Elem<T>::K][Elem<T>::DIM], double Kv,
                                            const VelField *vf, double (&A)[Elem<T>::K][Elem<T>::K], double *vol)
{
    using E = Elem<T>;
#pragma unroll
    for (int i = 0; i < E::K; ++i)
#pragma unroll
        for (int j = 0; j < E::K; ++j) A[i][j] = 0.0;
    double gm[3];
    elem_centre<T>(X, gm);
    double Ji[3][3];
    // simplices: affine map, one (J^T)^{-1} for the element
    constexpr bool affine = (T == UG4GB_TET || T == UG4GB_TRI);
    if constexpr (affine) {
        double xi[3] = {0.25, 0.25, 0.25};
        jt_inverse<T>(X, xi, Ji);
    }
#pragma unroll
    for (int ip = 0; ip < E::NSCVF; ++ip) {
        const int from = E::from(ip), to = E::to(ip);
        double n[3] = {0, 0, 0}, gip[3] = {0, 0, 0};
        double em[3];
        edge_mid<T>(X, ip, em);
        if constexpr (E::DIM == 2) {
            double dx = gm[0] - em[0], dy = gm[1] - em[1];
            n[0] = dy;
            n[1] = -dx;
            gip[0] = (em[0] + gm[0]) * 0.5;
            gip[1] = (em[1] + gm[1]) * 0.5;
        } else {
            double f0[3], f1[3];
            face_mid<T>(X, E::edge_face(ip, 0), f0);
            face_mid<T>(X, E::edge_face(ip, 1), f1);
            double a[3], b[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                a[d] = gm[d] - em[d];
                b[d] = f1[d] - f0[d];
                gip[d] = (em[d] + f0[d] + gm[d] + f1[d]) * 0.25;
            }
            n[0] = 0.5 * (a[1] * b[2] - a[2] * b[1]);
            n[1] = 0.5 * (a[2] * b[0] - a[0] * b[2]);
            n[2] = 0.5 * (a[0] * b[1] - a[1] * b[0]);
        }
        double xi[3];
        local_ip<T>(ip, xi);
        if constexpr (!affine) jt_inverse<T>(X, xi, Ji);
#pragma unroll
        for (int sh = 0; sh < E::K; ++sh) {
            double lg[3];
            local_grad<T>(xi, sh, lg);
            double gn = 0.0;
#pragma unroll
            for (int a = 0; a < E::DIM; ++a) {
                double g = 0.0;
#pragma unroll
                for (int b = 0; b < E::DIM; ++b) g += Ji[a][b] * lg[b];
                gn += g * n[a];
            }
            double F = -Kv * gn;
            A[from][sh] += F;
            A[to][sh] -= F;
        }
        if (vf) {
            double v[3];
            vf->eval(gip, v);
            double flux = 0.0;
#pragma unroll
            for (int d = 0; d < E::DIM; ++d) flux += n[d] * v[d];
            if (flux >= 0.0) {
                A[from][from] += flux;
                A[to][from] -= flux;
            } else {
                A[from][to] += flux;
                A[to][to] -= flux;
            }
        }
    }
    if (vol) scv_volumes<T>(X, vol);
}

}  // namespace ug4gb

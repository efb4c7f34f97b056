// k_fv1_rows.cu -- FV1 assembly of a structured level row by row.
//
// On a structured level every cell is the same box (spacing hx, hy, hz), so
// the FV1 geometry of an element depends only on its class: the hexahedron
// or quadrilateral of a cell, or one of the 6 Kuhn tetrahedra of a cell.  The
// element matrix of unit coefficient A1_c, the SCV volumes vol_c, the SCVF
// area normals and the integration-point offsets from the cell origin are
// computed once per class (k_class_data, with the same device code as the
// element kernel of k_fv1.cu) and passed to the row kernel as a kernel
// parameter, so that every table lookup is a constant-bank operand.  The
// element matrix of an element e of class c is then K_e A1_c (the box-method
// stencil F_sh = -(K grad phi_sh).n is linear in K).
//
// One thread per interior row gathers the contributions of the elements
// around its vertex (8 cells in 3D, 4 in 2D; for Kuhn cells the tets that
// contain the vertex) in increasing cell order, the order in which the
// element-wise reference adds them, and writes every value of the row and
// its right-hand side once: no read-modify-write of the matrix, no colour
// passes, no atomics.  The right-hand side of an interior row is
// f_i * sum_e |SCV_i^e|, the volumes summed once per level in the gather
// order (the element-wise reference adds the products f_i |SCV_i^e|; the two
// agree to rounding).  Convection (full upwind, ConvectionShapesFullUpwind,
// conv_shape.h:277-345) enters through the SCVF fluxes v(ip).n of each
// element, computed once per element and SCVF by k_scvf_flux.
// Rows on the box boundary (Dirichlet rows) get the identity row and a zero
// right-hand side (SetDirichletRow, sparsematrix_util.h:850-862); a boundary
// row without the Dirichlet flag is assembled by the general path.
//
// The element kernel of k_fv1.cu stays the path of unstructured levels and of
// the time-discrete assembly.  Values agree with it (and with the oracle,
// which computes every element's geometry from its own corner coordinates)
// to rounding: the cells of a structured level are congruent up to the
// rounding of their corner coordinates i / (n - 1).
#include <cstring>
#include <type_traits>

#include "common.cuh"
#include "disc.cuh"
#include "fv1_elem.cuh"

namespace ug4gb {

namespace {

// ------------------------------------------------------ class geometry ----
// Corner bits (x | y << 1 | z << 2) of the cell for corner q of element class
// p, as k_gen_elements (k_grid.cu) numbers them.
template <int T>
__host__ __device__ constexpr int class_corner_bits(int p, int q)
{
    if constexpr (T == UG4GB_QUAD) {
        // (0,0),(1,0),(1,1),(0,1)
        return q == 0 ? 0 : (q == 1 ? 1 : (q == 2 ? 3 : 2));
    } else if constexpr (T == UG4GB_HEX) {
        // bottom (0,0,0),(1,0,0),(1,1,0),(0,1,0), then the top
        return (q & 4) | (q == 0 || q == 4 ? 0 : (q == 1 || q == 5 ? 1 : (q == 2 || q == 6 ? 3 : 2)));
    } else {
        // Kuhn tet p: v0, v0 + e_a, v0 + e_a + e_b, v0 + (1,1,1) with
        // (a, b) = (0,1),(0,2),(1,0),(1,2),(2,0),(2,1); corners 1 and 2
        // swapped for p = 1, 2, 5 (positive orientation)
        const int a = (p < 2) ? 0 : (p < 4 ? 1 : 2);
        const int b = (p == 0) ? 1 : (p == 1 ? 2 : (p == 2 ? 0 : (p == 3 ? 2 : (p == 4 ? 0 : 1))));
        const int one = 1 << a, two = one | (1 << b);
        const bool odd = (p == 1 || p == 2 || p == 5);
        return q == 0 ? 0 : (q == 3 ? 7 : ((q == 1) != odd ? one : two));
    }
}

template <int T>
struct ClassTraits {
    using E = Elem<T>;
    static constexpr int NC = (T == UG4GB_TET) ? 6 : 1;   // element classes per cell
    static constexpr int K = E::K, NF = E::NSCVF, DIM = E::DIM;
    static constexpr int NCELL = (DIM == 3) ? 8 : 4;       // cells around a vertex
};

// per-class data passed by value to the row kernel
template <int T>
struct ClassData {
    double A[ClassTraits<T>::NC][ClassTraits<T>::K][ClassTraits<T>::K];   // unit-coefficient element matrix
    double vol[ClassTraits<T>::NC][ClassTraits<T>::K];                    // SCV volumes
};

// one thread per class: geometry of the classes of cell 0 from its actual
// corner coordinates (X), element matrix with K = 1 and no convection, SCV
// volumes, SCVF normals and integration points relative to the cell origin
template <int T>
__global__ void k_class_data(const double *coords, const int *elems, double *A, double *vol, double *normal,
                             double *ipoff, int *corner_ok)
{
    using E = Elem<T>;
    using CT = ClassTraits<T>;
    const int p = threadIdx.x;
    if (p >= CT::NC) return;
    double X[E::K][E::DIM];
    const int *ev = elems + (size_t)p * E::K;   // cell 0: elements 0 .. NC-1
    int ok = 1;
#pragma unroll
    for (int q = 0; q < E::K; ++q) {
        const int bits = class_corner_bits<T>(p, q);
#pragma unroll
        for (int d = 0; d < E::DIM; ++d) {
            X[q][d] = coords[(size_t)ev[q] * E::DIM + d];
            // the corner must sit where the class table says (cell 0 at the origin)
            const bool upper = (bits >> d) & 1;
            if ((X[q][d] > 0.0) != upper) ok = 0;
        }
    }
    double Aloc[E::K][E::K], v[E::K];
    elem_matrix<T>(X, 1.0, nullptr, Aloc, v);
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        vol[p * E::K + i] = v[i];
#pragma unroll
        for (int j = 0; j < E::K; ++j) A[(p * E::K + i) * E::K + j] = Aloc[i][j];
    }
    // SCVF normals and integration points (as elem_matrix forms them)
    double gm[3];
    elem_centre<T>(X, gm);
#pragma unroll
    for (int ip = 0; ip < E::NSCVF; ++ip) {
        double n[3] = {0, 0, 0}, gip[3] = {0, 0, 0}, em[3];
        edge_mid<T>(X, ip, em);
        if constexpr (E::DIM == 2) {
            n[0] = gm[1] - em[1];
            n[1] = -(gm[0] - em[0]);
            gip[0] = (em[0] + gm[0]) * 0.5;
            gip[1] = (em[1] + gm[1]) * 0.5;
        } else {
            double f0[3], f1[3], a[3], b[3];
            face_mid<T>(X, E::edge_face(ip, 0), f0);
            face_mid<T>(X, E::edge_face(ip, 1), f1);
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
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            normal[(p * E::NSCVF + ip) * 3 + d] = n[d];
            ipoff[(p * E::NSCVF + ip) * 3 + d] = gip[d];
        }
    }
    // corner ordering of the classes as k_gen_elements builds them
    if (!ok) atomicExch(corner_ok, 0);
}

// SCVF fluxes v(ip).n of the convection velocity v = curl of the random
// vector potential (VelField: v = scale sum_m -sin(phase_m + k_m.x) c_m) at
// the integration points x = o + d of every element: cell origin o plus the
// class's offset d.  The phase splits, sin(a + b) = sin a cos b + cos a sin b
// with a = phase_m + k_m.o per cell and mode and b = k_m.d per class, SCVF
// and mode, so one sine and cosine per cell and mode serve all SCVFs of the
// cell (GB300 evaluates FP64 sines on its slow FP64 pipe).  Table per class,
// SCVF and mode: cos b, sin b and w = c_m.n (the SCVF's area normal n).
template <int T>
__global__ void k_flux_table(int nmodes, const double *__restrict__ kv, const double *__restrict__ cv,
                             const double *__restrict__ normal, const double *__restrict__ ipoff,
                             double *__restrict__ tab)
{
    using CT = ClassTraits<T>;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= CT::NC * CT::NF * nmodes) return;
    const int m = t % nmodes, pf = t / nmodes;
    double b = 0.0, w = 0.0;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        b += kv[3 * m + d] * ipoff[pf * 3 + d];
        w += cv[3 * m + d] * normal[pf * 3 + d];
    }
    double sb, cb;
    sincos(b, &sb, &cb);
    tab[3 * t] = cb;
    tab[3 * t + 1] = sb;
    tab[3 * t + 2] = w;
}

template <int T>
__global__ void __launch_bounds__(128) k_scvf_flux(int cx, int cy, int ncell, double hx, double hy, double hz,
                                                   int nmodes, const double *__restrict__ kv,
                                                   const double *__restrict__ phase, double scale,
                                                   const double *__restrict__ tab, double *__restrict__ flux)
{
    using CT = ClassTraits<T>;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ncell * CT::NC) return;
    const int cell = t / CT::NC, p = t % CT::NC;
    const int i = cell % cx, j = (cell / cx) % cy, k = cell / (cx * cy);
    const double o[3] = {i * hx, j * hy, k * hz};
    double acc[CT::NF];
#pragma unroll
    for (int f = 0; f < CT::NF; ++f) acc[f] = 0.0;
    for (int m = 0; m < nmodes; ++m) {
        const double a = __ldg(phase + m) + __ldg(kv + 3 * m) * o[0] + __ldg(kv + 3 * m + 1) * o[1] +
                         __ldg(kv + 3 * m + 2) * o[2];
        double sa, ca;
        sincos(a, &sa, &ca);
#pragma unroll
        for (int f = 0; f < CT::NF; ++f) {
            const double *e = tab + 3 * ((p * CT::NF + f) * nmodes + m);
            const double s = sa * __ldg(e) + ca * __ldg(e + 1);
            acc[f] -= s * __ldg(e + 2);
        }
    }
#pragma unroll
    for (int f = 0; f < CT::NF; ++f) flux[(size_t)t * CT::NF + f] = scale * acc[f];
}

// ------------------------------------------------------------- stencil ----
// Offsets of the stencil of an interior row, in the order of the sorted
// columns (increasing dz, then dy, then dx).  Quadrilaterals 9, hexahedra
// 27, Kuhn tetrahedra 15 (0 and the +-offsets with components of one sign).
template <int T>
struct Stencil {
    static constexpr int DIM = Elem<T>::DIM;
    static constexpr int N = (T == UG4GB_QUAD) ? 9 : (T == UG4GB_HEX ? 27 : 15);
    __host__ __device__ static constexpr bool member(int dx, int dy, int dz)
    {
        if (DIM == 2 && dz != 0) return false;
        if (T != UG4GB_TET) return true;
        const bool pos = dx > 0 || dy > 0 || dz > 0, neg = dx < 0 || dy < 0 || dz < 0;
        return !(pos && neg);
    }
    // position of offset (dx, dy, dz) among the members
    __host__ __device__ static constexpr int slot(int dx, int dy, int dz)
    {
        int s = 0;
        for (int z = -1; z <= 1; ++z)
            for (int y = -1; y <= 1; ++y)
                for (int x = -1; x <= 1; ++x) {
                    if (z == dz && y == dy && x == dx) return s;
                    if (member(x, y, z)) ++s;
                }
        return -1;
    }
};

// Contributions of the elements around vertex (i, j, k) to its row: calls
// add(slot, value) for every element entry in increasing cell order (and
// class order inside a cell), and rhs(vol) for the SCV volumes.  kconst >= 0:
// every element's coefficient is kconst (the values a.K holds then), so no
// coefficient is loaded.
template <int T, class FA, class FV>
__device__ __forceinline__ void gather_row(const ClassData<T> &cd, const AsmArgs &a, int i, int j, int k,
                                           const double *__restrict__ flux, FA &&add, FV &&rhs,
                                           double kconst = -1.0)
{
    using CT = ClassTraits<T>;
    using E = Elem<T>;
    using S = Stencil<T>;
#pragma unroll
    for (int cz = (CT::DIM == 3 ? -1 : 0); cz <= 0; ++cz)
#pragma unroll
        for (int cy = -1; cy <= 0; ++cy)
#pragma unroll
            for (int cxo = -1; cxo <= 0; ++cxo) {
                // the vertex is corner (-cxo, -cy, -cz) of this cell
                const int lb = (-cxo) | ((-cy) << 1) | ((-cz) << 2);
                const int cell = (i + cxo) + a.cx * ((j + cy) + a.cy * (k + cz));
#pragma unroll
                for (int p = 0; p < CT::NC; ++p) {
                    // local index of the vertex in class p (or none)
                    int li = -1;
#pragma unroll
                    for (int q = 0; q < E::K; ++q)
                        if (class_corner_bits<T>(p, q) == lb) li = q;
                    if (li < 0) continue;
                    const int e = cell * CT::NC + p;
                    const double Ke = kconst >= 0.0 ? kconst : __ldg(a.K + e);
#pragma unroll
                    for (int q = 0; q < E::K; ++q) {
                        const int bq = class_corner_bits<T>(p, q);
                        const int s = S::slot(cxo + (bq & 1), cy + ((bq >> 1) & 1), cz + ((bq >> 2) & 1));
                        add(s, Ke * cd.A[p][li][q]);
                    }
                    if (flux) {
                        // full upwind: row li of SCVF f (from -> to, flux fl)
#pragma unroll
                        for (int f = 0; f < E::NSCVF; ++f) {
                            const int fr = E::from(f), to = E::to(f);
                            if (fr != li && to != li) continue;
                            const double fl = flux[(size_t)e * E::NSCVF + f];
                            const int bf = class_corner_bits<T>(p, fr), bt = class_corner_bits<T>(p, to);
                            const int sf = S::slot(cxo + (bf & 1), cy + ((bf >> 1) & 1), cz + ((bf >> 2) & 1));
                            const int st = S::slot(cxo + (bt & 1), cy + ((bt >> 1) & 1), cz + ((bt >> 2) & 1));
                            if (fr == li) {
                                // A[from][up] += flux
                                if (fl >= 0.0) add(sf, fl);
                                else add(st, fl);
                            } else {
                                // A[to][up] -= flux
                                if (fl >= 0.0) add(sf, -fl);
                                else add(st, -fl);
                            }
                        }
                    }
                    rhs(cd.vol[p][li]);
                }
            }
}

__device__ __forceinline__ double source_at(const AsmArgs &a, int r)
{
    return a.f ? a.f[r] : (a.use_seed ? 2.0 * hash_uniform(a.f_seed, (uint64_t)r) - 1.0 : 0.0);
}

// every interior row must hold exactly the stencil's entries (the pattern of
// csr_from_elements); ok is cleared otherwise (checked once per level)
template <int T>
__global__ void k_check_row_lengths(int cx, int cy, int cz, const int *__restrict__ rowptr, int *ok)
{
    using S = Stencil<T>;
    const int nix = cx - 1, niy = cy - 1, niz = (S::DIM == 3) ? cz - 1 : 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nix * niy * niz) return;
    const int i = 1 + t % nix, j = 1 + (t / nix) % niy, k = (S::DIM == 3) ? 1 + t / (nix * niy) : 0;
    const int r = i + (cx + 1) * (j + (cy + 1) * k);
    if (rowptr[r + 1] - rowptr[r] != S::N) atomicExch(ok, 0);
}

// the sum of an interior vertex's SCV volumes in the order of gather_row
template <int T>
__global__ void k_row_volsum(AsmArgs a, ClassData<T> cd, double *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s = 0.0;
    gather_row<T>(cd, a, 1, 1, (Stencil<T>::DIM == 3) ? 1 : 0, nullptr, [](int, double) {}, [&](double v) { s += v; });
    out[0] = s;
}

// interior rows: one thread per row, every value written once
template <int T>
__global__ void __launch_bounds__(128) k_assemble_rows(AsmArgs a, ClassData<T> cd, const double *__restrict__ flux,
                                                       double volsum)
{
    PDL_ENTRY();
    using S = Stencil<T>;
    const int nix = a.cx - 1, niy = a.cy - 1, niz = (S::DIM == 3) ? a.cz - 1 : 1;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nix * niy * niz) return;
    const int i = 1 + t % nix, j = 1 + (t / nix) % niy, k = (S::DIM == 3) ? 1 + t / (nix * niy) : 0;
    const int nx = a.cx + 1, ny = a.cy + 1;
    const int r = i + nx * (j + ny * k);
    double acc[S::N];
#pragma unroll
    for (int s = 0; s < S::N; ++s) acc[s] = 0.0;
    gather_row<T>(cd, a, i, j, k, flux, [&](int s, double v) { acc[s] += v; }, [](double) {});
    double *row = a.val + __ldg(a.rowptr + r);
#pragma unroll
    for (int s = 0; s < S::N; ++s) row[s] = acc[s];
    if (a.b) a.b[r] = source_at(a, r) * volsum;
}


// rows on the box boundary: the identity row and b = 0 at Dirichlet
// vertices; otherwise the elements that exist, entries found by search
// a boundary row without the Dirichlet flag: the elements that exist, entries
// found by binary search in the row (rare; kept out of line)
template <int T>
__device__ __noinline__ void boundary_row_general(const AsmArgs &a, const ClassData<T> &cd,
                                                  const double *__restrict__ flux, int r, int r0, int r1)
{
    using CT = ClassTraits<T>;
    using E = Elem<T>;
    const int nx = a.cx + 1, ny = a.cy + 1;
    const int i = r % nx, j = (r / nx) % ny, k = r / (nx * ny);
    for (int q = r0; q < r1; ++q) a.val[q] = 0.0;
    double vsum = 0.0;
    const double fr = a.b ? source_at(a, r) : 0.0;
    for (int cz = (CT::DIM == 3 ? -1 : 0); cz <= 0; ++cz)
        for (int cy = -1; cy <= 0; ++cy)
            for (int cxo = -1; cxo <= 0; ++cxo) {
                if (i + cxo < 0 || i + cxo >= a.cx || j + cy < 0 || j + cy >= a.cy ||
                    (CT::DIM == 3 && (k + cz < 0 || k + cz >= a.cz)))
                    continue;
                const int lb = (-cxo) | ((-cy) << 1) | ((-cz) << 2);
                const int cell = (i + cxo) + a.cx * ((j + cy) + a.cy * (k + cz));
                for (int p = 0; p < CT::NC; ++p) {
                    int li = -1;
                    for (int q = 0; q < E::K; ++q)
                        if (class_corner_bits<T>(p, q) == lb) li = q;
                    if (li < 0) continue;
                    const int e = cell * CT::NC + p;
                    auto col_of = [&](int q) {
                        const int bq = class_corner_bits<T>(p, q);
                        return (i + cxo + (bq & 1)) + nx * ((j + cy + ((bq >> 1) & 1)) + ny * (k + cz + ((bq >> 2) & 1)));
                    };
                    auto slot = [&](int c) {
                        int lo = r0, hi = r1 - 1;
                        while (lo <= hi) {
                            const int mid = (lo + hi) >> 1;
                            if (a.col[mid] == c) return mid;
                            if (a.col[mid] < c) lo = mid + 1; else hi = mid - 1;
                        }
                        return -1;
                    };
                    for (int q = 0; q < E::K; ++q) {
                        const int s = slot(col_of(q));
                        if (s >= 0) a.val[s] += a.K[e] * cd.A[p][li][q];
                    }
                    if (flux) {
                        for (int f = 0; f < E::NSCVF; ++f) {
                            const int fr2 = E::from(f), to = E::to(f);
                            if (fr2 != li && to != li) continue;
                            const double fl = flux[(size_t)e * E::NSCVF + f];
                            const int up = (fl >= 0.0) ? fr2 : to;
                            const int s = slot(col_of(up));
                            if (s >= 0) a.val[s] += (fr2 == li) ? fl : -fl;
                        }
                    }
                    vsum += fr * cd.vol[p][li];
                }
            }
    if (a.b) a.b[r] = vsum;
}

// one boundary row by nlanes threads (lane 0..nlanes-1; a warp, or one
// thread with nlanes = 1): a Dirichlet row is the identity row with b = 0,
// any other row is assembled by lane 0
template <int T>
__device__ __forceinline__ void boundary_row(const AsmArgs &a, const ClassData<T> &cd, const double *__restrict__ flux,
                                             const unsigned char *__restrict__ bnd, int r, int lane, int nlanes = 32)
{
    const int r0 = a.rowptr[r], r1 = a.rowptr[r + 1];
    if (bnd[r]) {
        for (int q = r0 + lane; q < r1; q += nlanes) a.val[q] = (a.col[q] == r) ? 1.0 : 0.0;
        if (a.b && lane == 0) a.b[r] = 0.0;
        return;
    }
    if (lane == 0) boundary_row_general<T>(a, cd, flux, r, r0, r1);
}

// small levels (launch-bound): every row of the level in one launch, one
// thread per row, interior rows as k_assemble_rows, boundary rows as
// k_assemble_boundary_rows
template <int T>
__global__ void __launch_bounds__(128) k_assemble_rows_all(AsmArgs a, ClassData<T> cd, const double *__restrict__ flux,
                                                           double volsum, const unsigned char *__restrict__ bnd)
{
    PDL_ENTRY();
    using S = Stencil<T>;
    const int nx = a.cx + 1, ny = a.cy + 1, nz = (S::DIM == 3) ? a.cz + 1 : 1;
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nx * ny * nz) return;
    const int i = r % nx, j = (r / nx) % ny, k = r / (nx * ny);
    if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || (S::DIM == 3 && (k == 0 || k == nz - 1))) {
        boundary_row<T>(a, cd, flux, bnd, r, 0, 1);
        return;
    }
    double acc[S::N];
#pragma unroll
    for (int s = 0; s < S::N; ++s) acc[s] = 0.0;
    gather_row<T>(cd, a, i, j, k, flux, [&](int s, double v) { acc[s] += v; }, [](double) {});
    double *row = a.val + __ldg(a.rowptr + r);
#pragma unroll
    for (int s = 0; s < S::N; ++s) row[s] = acc[s];
    if (a.b) a.b[r] = source_at(a, r) * volsum;
}

// the rows of a list (the box surface), one warp per row
template <int T>
__global__ void __launch_bounds__(256) k_assemble_boundary_rows(AsmArgs a, ClassData<T> cd,
                                                                const double *__restrict__ flux,
                                                                const unsigned char *__restrict__ bnd,
                                                                const int *__restrict__ brows, int nbrows)
{
    PDL_ENTRY();
    const int t = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    if (t >= nbrows) return;
    boundary_row<T>(a, cd, flux, bnd, brows[t], threadIdx.x & 31);
}

// One coefficient K for all elements and no convection: every interior row
// holds the same stencil.  A block takes kLinesPerBlock consecutive grid lines
// (fixed j, k) of the level (one: more lines per block serialise their
// latencies and were slower); the rows (and values) of a line are contiguous
// in the CRS.  Thread 0 first gathers the stencil of the interior row
// (1, 1, 1) with the arithmetic of k_assemble_rows (so the values are the
// same; the coefficient, a.K's value everywhere, comes as a parameter).  On a
// line inside the box, warps 1 and 2 write the line's two end rows on the
// boundary, all threads the right-hand side and then the interior values,
// consecutive threads on consecutive values.  A line on the box surface
// consists of boundary rows: the block sweeps the line's values with
// consecutive threads (the row of a value from the line's row pointers in
// shared memory), writing the identity rows of Dirichlet vertices; any other
// row of the line is assembled by one lane afterwards.  Dynamic shared
// memory: nx + 1 row pointers.
constexpr int kLinesPerBlock = 1;

template <int T>
__global__ void __launch_bounds__(128) k_assemble_lines_uniform(AsmArgs a, ClassData<T> cd, double volsum, double kval,
                                                                const unsigned char *__restrict__ bnd, int nlines)
{
    PDL_ENTRY();
    using S = Stencil<T>;
    __shared__ double st[S::N];
    extern __shared__ int srp[];
    const int nx = a.cx + 1, ny = a.cy + 1, nz = (S::DIM == 3) ? a.cz + 1 : 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int nix = a.cx - 1;
    if (threadIdx.x == 0) {
        double acc[S::N];
#pragma unroll
        for (int s = 0; s < S::N; ++s) acc[s] = 0.0;
        gather_row<T>(cd, a, 1, 1, (S::DIM == 3) ? 1 : 0, nullptr, [&](int s, double v) { acc[s] += v; },
                      [](double) {}, kval);
#pragma unroll
        for (int s = 0; s < S::N; ++s) st[s] = acc[s];
    }
    __syncthreads();
    // the lines on the box surface come first (they take longer: started
    // first, they overlap the stream of interior lines instead of trailing
    // it), then the interior lines
    const int nsurf = (S::DIM == 3) ? 2 * ny + 2 * (nz - 2) : 2;
    for (int ln = 0; ln < kLinesPerBlock; ++ln) {
        const int line_id = blockIdx.x * kLinesPerBlock + ln;
        if (line_id >= nlines) return;
        int j, k;
        if (line_id < nsurf) {
            if (S::DIM != 3) {
                j = line_id == 0 ? 0 : ny - 1;
                k = 0;
            } else if (line_id < 2 * ny) {
                j = line_id % ny;
                k = line_id < ny ? 0 : nz - 1;
            } else {
                const int t = line_id - 2 * ny;
                j = (t & 1) ? ny - 1 : 0;
                k = 1 + (t >> 1);
            }
        } else {
            const int t = line_id - nsurf, ni = ny - 2;
            j = 1 + t % ni;
            k = (S::DIM == 3) ? 1 + t / ni : 0;
        }
        const int rl = nx * (j + ny * k);   // row of (0, j, k)
        if (j == 0 || j == ny - 1 || (S::DIM == 3 && (k == 0 || k == nz - 1))) {
            __syncthreads();   // srp of the previous surface line is read
            for (int i = threadIdx.x; i <= nx; i += blockDim.x) srp[i] = __ldg(a.rowptr + rl + i);
            __syncthreads();
            const int q0 = srp[0], q1 = srp[nx];
            for (int q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
                // the row of value q: the last row pointer <= q
                int lo = 0, hi = nx - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (srp[mid] <= q) lo = mid; else hi = mid - 1;
                }
                const int r = rl + lo;
                if (bnd[r]) a.val[q] = (__ldg(a.col + q) == r) ? 1.0 : 0.0;
            }
            for (int i = threadIdx.x; i < nx; i += blockDim.x)
                if (a.b && bnd[rl + i]) a.b[rl + i] = 0.0;
            // rows without the Dirichlet flag (none where the whole boundary
            // is Dirichlet)
            for (int i = warp; i < nx; i += nwarps)
                if (!bnd[rl + i] && lane == 0) boundary_row_general<T>(a, cd, nullptr, rl + i, srp[i], srp[i + 1]);
            continue;
        }
        const int r0 = rl + 1;
        if (warp == 1) boundary_row<T>(a, cd, nullptr, bnd, rl, lane);
        else if (warp == 2) boundary_row<T>(a, cd, nullptr, bnd, rl + nx - 1, lane);
        double *line = a.val + __ldg(a.rowptr + r0);
        if (a.b)
            for (int i = threadIdx.x; i < nix; i += blockDim.x) a.b[r0 + i] = source_at(a, r0 + i) * volsum;
        const int len = S::N * nix;
        for (int q = threadIdx.x; q < len; q += blockDim.x) line[q] = st[q % S::N];
    }
}

}  // namespace

// levels up to this size are assembled in one launch (k_assemble_rows_all):
// their assembly is bound by the launches, not by the rows
constexpr int kSmallLevelRows = 1 << 16;

// Assembles level L row by row when it is a structured level and the
// assembly is stationary; returns false (nothing launched) otherwise.
bool launch_assemble_rows(Ctx &c, const Level &L, const AsmArgs &a_in, RowAsmCache &cache)
{
    if (!L.structured || a_in.inst || L.nx < 3 || L.ny < 3 || (L.dim == 3 && L.nz < 3)) return false;
    bool done = false;
    auto run = [&](auto tag) {
        constexpr int T = decltype(tag)::value;
        using CT = ClassTraits<T>;
        using E = Elem<T>;
        const int cx = L.nx - 1, cy = L.ny - 1, cz = (L.dim == 3) ? L.nz - 1 : 1;
        const int nint = (cx - 1) * (cy - 1) * ((L.dim == 3) ? cz - 1 : 1);
        if (!cache.ready) {
            DevBuf<double> A, vol, nrm, ipo;
            DevBuf<int> ok;
            A.alloc(CT::NC * E::K * E::K);
            vol.alloc(CT::NC * E::K);
            nrm.alloc(CT::NC * E::NSCVF * 3);
            ipo.alloc(CT::NC * E::NSCVF * 3);
            ok.alloc(1);
            const int one = 1;
            copy_in(c, ok.p, &one, sizeof(int));
            UG_LAUNCH(c, k_class_data<T>, 1, 32, 0, L.coords.p, L.elems.p, A.p, vol.p, nrm.p, ipo.p, ok.p);
            UG_LAUNCH(c, k_check_row_lengths<T>, div_up(nint, 256), 256, 0, cx, cy, cz, a_in.rowptr, ok.p);
            cache.A.resize(CT::NC * E::K * E::K);
            cache.vol.resize(CT::NC * E::K);
            copy_out(c, cache.A.data(), A.p, sizeof(double) * cache.A.size());
            copy_out(c, cache.vol.data(), vol.p, sizeof(double) * cache.vol.size());
            int okh = 0;
            copy_out(c, &okh, ok.p, sizeof(int));
            cache.normal = std::move(nrm);
            cache.ipoff = std::move(ipo);
            cache.usable = (okh == 1);
            cache.ready = true;
        }
        if (!cache.usable) return;
        ClassData<T> cd;
        std::memcpy(&cd.A[0][0][0], cache.A.data(), sizeof(cd.A));
        std::memcpy(&cd.vol[0][0], cache.vol.data(), sizeof(cd.vol));
        AsmArgs a = a_in;
        a.cx = cx;
        a.cy = cy;
        a.cz = cz;
        if (cache.nbrows == 0) {
            // once per level: the interior rows' SCV volume sum and the list of
            // the rows on the box boundary
            DevBuf<double> vs;
            vs.alloc(1);
            UG_LAUNCH(c, k_row_volsum<T>, 1, 32, 0, a, cd, vs.p);
            copy_out(c, &cache.volsum, vs.p, sizeof(double));
            const int nx = L.nx, ny = L.ny, nz = (L.dim == 3) ? L.nz : 1;
            std::vector<int> rows;
            for (int k = 0; k < nz; ++k)
                for (int j = 0; j < ny; ++j)
                    for (int i = 0; i < nx; ++i)
                        if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || (L.dim == 3 && (k == 0 || k == nz - 1)))
                            rows.push_back(i + nx * (j + ny * k));
            cache.brows.alloc(rows.size());
            copy_in(c, cache.brows.p, rows.data(), sizeof(int) * rows.size());
            UG_CUDA(cudaStreamSynchronize(c.stream));
            cache.nbrows = (int)rows.size();
        }
        const double *flux = nullptr;
        if (a.vmodes > 0) {
            if constexpr (E::DIM == 3) {
                const int ncell = a.cx * a.cy * a.cz;
                const size_t nf = (size_t)ncell * CT::NC * E::NSCVF;
                // the fluxes depend on the velocity field and the geometry
                // only: computed again when the field changed
                if (cache.flux.n < nf || cache.flux_version != a.vel_version) {
                    if (cache.flux.n < nf) cache.flux.alloc(nf);
                    const int ntab = CT::NC * CT::NF * a.vmodes;
                    DevBuf<double> tab;
                    tab.alloc(3 * (size_t)ntab);
                    UG_LAUNCH(c, k_flux_table<T>, div_up(ntab, 128), 128, 0, a.vmodes, a.vk, a.vc, cache.normal.p,
                              cache.ipoff.p, tab.p);
                    UG_LAUNCH(c, k_scvf_flux<T>, div_up(ncell * CT::NC, 128), 128, 0, a.cx, a.cy, ncell,
                              1.0 / (double)a.cx, 1.0 / (double)a.cy, 1.0 / (double)a.cz, a.vmodes, a.vk, a.vphase,
                              a.vscale, tab.p, cache.flux.p);
                    // the table is freed on return: its kernel must have read it
                    UG_CUDA(cudaStreamSynchronize(c.stream));
                    cache.flux_version = a.vel_version;
                }
                flux = cache.flux.p;
            } else {
                return;   // no 2D velocity field
            }
        }
        const size_t line_smem = sizeof(int) * (size_t)(L.nx + 1);
        if (a.k_uniform && !flux && line_smem <= 32 * 1024) {
            // every grid line, the boundary rows with it
            const int nlines = L.ny * ((L.dim == 3) ? L.nz : 1);
            UG_LAUNCH_PDL(c, k_assemble_lines_uniform<T>, div_up(nlines, kLinesPerBlock), 128, line_smem, a, cd,
                      cache.volsum, a.k_value, L.bnd.p, nlines);
        } else {
            if (L.nv <= kSmallLevelRows) {
                UG_LAUNCH_PDL(c, k_assemble_rows_all<T>, div_up(L.nv, 128), 128, 0, a, cd, flux, cache.volsum, L.bnd.p);
            } else {
                UG_LAUNCH_PDL(c, k_assemble_rows<T>, div_up(nint, 128), 128, 0, a, cd, flux, cache.volsum);
                UG_LAUNCH_PDL(c, k_assemble_boundary_rows<T>, div_up(cache.nbrows, 8), 256, 0, a, cd, flux, L.bnd.p,
                          cache.brows.p, cache.nbrows);
            }
        }
        done = true;
    };
    switch (L.elem_type) {
        case UG4GB_QUAD: run(std::integral_constant<int, UG4GB_QUAD>()); break;
        case UG4GB_HEX: run(std::integral_constant<int, UG4GB_HEX>()); break;
        case UG4GB_TET: run(std::integral_constant<int, UG4GB_TET>()); break;
        default: break;
    }
    return done;
}

}  // namespace ug4gb

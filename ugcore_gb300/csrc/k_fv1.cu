// k_fv1.cu -- FV1 (vertex-centred box) element assembly on the GPU, FP64.
//
// One thread per element.  The element geometry follows FV1Geometry_gen::
// update (lib_disc/spatial_disc/disc_util/fv1_geom.cpp:331-464): mid points
// as corner averages, one SCVF per element edge with patch [edge mid, centre]
// (2D) or [edge mid, side-0 centre, centre, side-1 centre] (3D), area normal
// by ElementNormal (lib_disc/common/geometry_util.h:499-589), integration
// point = patch average, global gradients JtInv * local P1 gradients (per ip
// for quad/hex, once for tet), SCV volumes by ElementSize of the SCV
// quadrilateral / hexahedron (geometry_util.h:156-161,294-323).
// The stencil is the box-method one of the (external) ConvectionDiffusion
// FV1 element disc: F_sh = -(K grad phi_sh).n added to (from, sh) and
// subtracted from (to, sh); full upwind adds flux = v(ip).n to the upwind
// column (ConvectionShapesFullUpwind::update, conv_shape.h:277-345); the
// right-hand side gets f_i |SCV_i|.  Element matrices are scattered with FP64
// atomics into the level CRS, found by binary search in the sorted row.
// Reference-element numbering: lib_disc/reference_element/reference_element.cpp
// (quadrilateral :428, tetrahedron :547, hexahedron :1327).
#include "common.cuh"
#include "fv1_elem.cuh"
#include "disc.cuh"

namespace ug4gb {

__device__ __forceinline__ int find_slot(const int *__restrict__ rowptr, const int *__restrict__ col, int r, int c)
{
    int lo = rowptr[r], hi = rowptr[r + 1] - 1;
    while (lo <= hi) {
        int mid = (lo + hi) >> 1;
        int cm = col[mid];
        if (cm == c) return mid;
        if (cm < c) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}



template <int T>
__global__ void __launch_bounds__(128) k_assemble(AsmArgs a)
{
    using E = Elem<T>;
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= a.ne) return;
    int ev[E::K];
    double X[E::K][E::DIM];
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        ev[i] = a.elems[(size_t)e * E::K + i];
#pragma unroll
        for (int d = 0; d < E::DIM; ++d) X[i][d] = a.coords[(size_t)ev[i] * E::DIM + d];
    }
    double Aloc[E::K][E::K];
    double vol[E::K];
    VelField vf{a.vmodes, a.vk, a.vc, a.vphase, a.vscale};
    elem_matrix<T>(X, a.K[e], a.vmodes > 0 ? &vf : nullptr, Aloc, a.b ? vol : nullptr);
#pragma unroll
    for (int i = 0; i < E::K; ++i)
#pragma unroll
        for (int j = 0; j < E::K; ++j) {
            int s = find_slot(a.rowptr, a.col, ev[i], ev[j]);
            if (s >= 0) atomicAdd(a.val + s, Aloc[i][j]);
        }
    if (a.b) {
#pragma unroll
        for (int i = 0; i < E::K; ++i) {
            double fi = a.f ? a.f[ev[i]] : (a.use_seed ? 2.0 * hash_uniform(a.f_seed, (uint64_t)ev[i]) - 1.0 : 0.0);
            atomicAdd(a.b + ev[i], fi * vol[i]);
        }
    }
}

// Dirichlet rows: values 0, diagonal 1, pattern kept, rhs 0
// (SetDirichletRow, lib_algebra/algebra_common/sparsematrix_util.h:850-862)
__global__ void k_dirichlet_rows(const unsigned char *bnd, int nv, const int *rowptr, const int *col, double *val,
                                 double *b)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nv || !bnd[v]) return;
    for (int a = rowptr[v]; a < rowptr[v + 1]; ++a) val[a] = (col[a] == v) ? 1.0 : 0.0;
    if (b) b[v] = 0.0;
}

void launch_assemble(Ctx &c, const Level &L, const AsmArgs &a)
{
    unsigned g = div_up(L.ne, 128);
    if (L.elem_type == UG4GB_QUAD) UG_LAUNCH(c, k_assemble<UG4GB_QUAD>, g, 128, 0, a);
    else if (L.elem_type == UG4GB_HEX) UG_LAUNCH(c, k_assemble<UG4GB_HEX>, g, 128, 0, a);
    else UG_LAUNCH(c, k_assemble<UG4GB_TET>, g, 128, 0, a);
}

void launch_dirichlet(Ctx &c, const Level &L, Csr &A, double *b)
{
    UG_LAUNCH(c, k_dirichlet_rows, div_up(L.nv, 256), 256, 0, L.bnd.p, L.nv, A.rowptr.p, A.col.p, A.val.p, b);
}

// ------------------------------------------------------ coefficients -----
// K_e = exp(factor * amp * sum_m cos(k_m . c_e + phase_m)), c_e = centroid
template <int T>
__global__ void k_coef_fourier(const double *coords, const int *elems, int ne, int nmodes, const double *k,
                               const double *phase, double amp, double factor, double *K)
{
    using E = Elem<T>;
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    double cc[E::DIM];
#pragma unroll
    for (int d = 0; d < E::DIM; ++d) cc[d] = 0.0;
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        int v = elems[(size_t)e * E::K + i];
#pragma unroll
        for (int d = 0; d < E::DIM; ++d) cc[d] += coords[(size_t)v * E::DIM + d];
    }
#pragma unroll
    for (int d = 0; d < E::DIM; ++d) cc[d] *= 1.0 / (double)E::K;
    double s = 0.0;
    for (int m = 0; m < nmodes; ++m) {
        double th = phase[m];
#pragma unroll
        for (int d = 0; d < E::DIM; ++d) th += k[m * E::DIM + d] * cc[d];
        s += cos(th);
    }
    K[e] = exp(factor * (amp * s));
}

void launch_coef_fourier(Ctx &c, const Level &L, int nmodes, const double *k, const double *phase, double amp,
                         double factor, double *K)
{
    unsigned g = div_up(L.ne, 256);
    if (L.elem_type == UG4GB_QUAD)
        UG_LAUNCH(c, k_coef_fourier<UG4GB_QUAD>, g, 256, 0, L.coords.p, L.elems.p, L.ne, nmodes, k, phase, amp, factor, K);
    else if (L.elem_type == UG4GB_HEX)
        UG_LAUNCH(c, k_coef_fourier<UG4GB_HEX>, g, 256, 0, L.coords.p, L.elems.p, L.ne, nmodes, k, phase, amp, factor, K);
    else
        UG_LAUNCH(c, k_coef_fourier<UG4GB_TET>, g, 256, 0, L.coords.p, L.elems.p, L.ne, nmodes, k, phase, amp, factor, K);
}

// coarse log K = mean of the children's log K (structured children)
__global__ void k_coarsen_log(int elem_type, const double *fcoords, const int *felems, int fne, int fnx, int fny,
                              int fnz, int cnx, int cny, const double *logf, double *sumc, int *cntc)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= fne) return;
    int fx = fnx - 1, fy = fny - 1;
    int cx = cnx - 1, cy = cny - 1;
    int ce;
    if (elem_type == UG4GB_QUAD) {
        int i = e % fx, j = e / fx;
        ce = (i >> 1) + cx * (j >> 1);
    } else if (elem_type == UG4GB_HEX) {
        int i = e % fx, j = (e / fx) % fy, k = e / (fx * fy);
        ce = (i >> 1) + cx * ((j >> 1) + cy * (k >> 1));
    } else {
        int h = e / 6;
        int i = h % fx, j = (h / fx) % fy, k = h / (fx * fy);
        double cc[3] = {0, 0, 0};
        for (int a = 0; a < 4; ++a) {
            int v = felems[4 * (size_t)e + a];
            for (int d = 0; d < 3; ++d) cc[d] += fcoords[3 * (size_t)v + d];
        }
        int ci[3] = {i >> 1, j >> 1, k >> 1};
        double off[3];
        for (int d = 0; d < 3; ++d) off[d] = cc[d] * 0.25 * (double)(cnx - 1) - (double)ci[d];
        int p;
        if (off[0] >= off[1] && off[1] >= off[2]) p = 0;
        else if (off[0] >= off[2] && off[2] >= off[1]) p = 1;
        else if (off[1] >= off[0] && off[0] >= off[2]) p = 2;
        else if (off[1] >= off[2] && off[2] >= off[0]) p = 3;
        else if (off[2] >= off[0] && off[0] >= off[1]) p = 4;
        else p = 5;
        ce = 6 * (ci[0] + cx * (ci[1] + cy * ci[2])) + p;
    }
    (void)fnz;
    atomicAdd(sumc + ce, logf[e]);
    atomicAdd(cntc + ce, 1);
}

__global__ void k_finish_coarse_log(const double *sumc, const int *cntc, int ne, double *logc)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < ne) logc[e] = sumc[e] / (double)(cntc[e] ? cntc[e] : 1);
}

__global__ void k_exp(const double *m, int n, double *K)
{
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) K[e] = exp(m[e]);
}

void coarsen_log(Ctx &c, const Level &F, const Level &Cl, const double *logf, double *logc)
{
    DevBuf<double> sum;
    DevBuf<int> cnt;
    sum.alloc(Cl.ne);
    cnt.alloc(Cl.ne);
    UG_CUDA(cudaMemsetAsync(sum.p, 0, sum.bytes(), c.stream));
    UG_CUDA(cudaMemsetAsync(cnt.p, 0, cnt.bytes(), c.stream));
    UG_LAUNCH(c, k_coarsen_log, div_up(F.ne, 256), 256, 0, F.elem_type, F.coords.p, F.elems.p, F.ne, F.nx, F.ny, F.nz,
              Cl.nx, Cl.ny, logf, sum.p, cnt.p);
    UG_LAUNCH(c, k_finish_coarse_log, div_up(Cl.ne, 256), 256, 0, sum.p, cnt.p, Cl.ne, logc);
}

void exp_elements(Ctx &c, const double *m, int n, double *K)
{
    UG_LAUNCH(c, k_exp, div_up(n, 256), 256, 0, m, n, K);
}

// ------------------------------------------------------------ adjoint ----
// dJ/dm_e = -K_e * sum_{i not Dirichlet} lambda_i (A1_e u_e)_i
template <int T>
__global__ void __launch_bounds__(128) k_grad_logk(const double *coords, const int *elems, int ne,
                                                   const unsigned char *bnd, const double *K, const double *u,
                                                   const double *lam, double *g)
{
    using E = Elem<T>;
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int ev[E::K];
    double X[E::K][E::DIM];
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        ev[i] = elems[(size_t)e * E::K + i];
#pragma unroll
        for (int d = 0; d < E::DIM; ++d) X[i][d] = coords[(size_t)ev[i] * E::DIM + d];
    }
    double A1[E::K][E::K];
    elem_matrix<T>(X, 1.0, nullptr, A1, nullptr);
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        if (bnd[ev[i]]) continue;
        double r = 0.0;
#pragma unroll
        for (int j = 0; j < E::K; ++j) r += A1[i][j] * u[ev[j]];
        s += lam[ev[i]] * r;
    }
    g[e] = -K[e] * s;
}

void launch_grad_logk(Ctx &c, const Level &L, const double *K, const double *u, const double *lam, double *g)
{
    unsigned gr = div_up(L.ne, 128);
    if (L.elem_type == UG4GB_QUAD)
        UG_LAUNCH(c, k_grad_logk<UG4GB_QUAD>, gr, 128, 0, L.coords.p, L.elems.p, L.ne, L.bnd.p, K, u, lam, g);
    else if (L.elem_type == UG4GB_HEX)
        UG_LAUNCH(c, k_grad_logk<UG4GB_HEX>, gr, 128, 0, L.coords.p, L.elems.p, L.ne, L.bnd.p, K, u, lam, g);
    else
        UG_LAUNCH(c, k_grad_logk<UG4GB_TET>, gr, 128, 0, L.coords.p, L.elems.p, L.ne, L.bnd.p, K, u, lam, g);
}

// sum of SCV volumes per vertex (d rhs_i / d f_i)
template <int T>
__global__ void k_scv_volumes(const double *coords, const int *elems, int ne, double *vol)
{
    using E = Elem<T>;
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    int ev[E::K];
    double X[E::K][E::DIM];
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        ev[i] = elems[(size_t)e * E::K + i];
#pragma unroll
        for (int d = 0; d < E::DIM; ++d) X[i][d] = coords[(size_t)ev[i] * E::DIM + d];
    }
    double v[E::K];
    scv_volumes<T>(X, v);
#pragma unroll
    for (int i = 0; i < E::K; ++i) atomicAdd(vol + ev[i], v[i]);
}

__global__ void k_grad_source(const double *vol, const unsigned char *bnd, const double *lam, int nv, double *g)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nv) g[i] = bnd[i] ? 0.0 : vol[i] * lam[i];
}

void launch_grad_source(Ctx &c, const Level &L, const double *lam, double *g)
{
    DevBuf<double> vol;
    vol.alloc(L.nv);
    UG_CUDA(cudaMemsetAsync(vol.p, 0, vol.bytes(), c.stream));
    unsigned gr = div_up(L.ne, 128);
    if (L.elem_type == UG4GB_QUAD) UG_LAUNCH(c, k_scv_volumes<UG4GB_QUAD>, gr, 128, 0, L.coords.p, L.elems.p, L.ne, vol.p);
    else if (L.elem_type == UG4GB_HEX) UG_LAUNCH(c, k_scv_volumes<UG4GB_HEX>, gr, 128, 0, L.coords.p, L.elems.p, L.ne, vol.p);
    else UG_LAUNCH(c, k_scv_volumes<UG4GB_TET>, gr, 128, 0, L.coords.p, L.elems.p, L.ne, vol.p);
    UG_LAUNCH(c, k_grad_source, div_up(L.nv, 256), 256, 0, vol.p, L.bnd.p, lam, L.nv, g);
    UG_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace ug4gb

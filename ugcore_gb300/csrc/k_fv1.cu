// k_fv1.cu -- FV1 (vertex-centred box) element assembly on the GPU, FP64.
//
// One thread per cell (a quad, a hex, or the 6 Kuhn tets of a hex), launched
// once per parity colour; on unstructured levels one thread per element,
// launched once per element colour.  The element geometry follows FV1Geometry_gen::
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
// right-hand side gets f_i |SCV_i|.  Element matrices are added into the
// level CRS (slots found by binary search in the sorted row) colour by colour,
// without atomics, so every run assembles the same bits.
// Reference-element numbering: lib_disc/reference_element/reference_element.cpp
// (triangle :320-420, quadrilateral :428, tetrahedron :547, hexahedron :1327).
#include <type_traits>

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



// Cells of one parity colour: cell (i,j,k) with (i&1, j&1, k&1) = colour bits.
// No two cells of a colour share a vertex, so their element matrices are
// added with plain read-modify-writes, colour after colour: the assembled
// values are the same bits in every run (an FP64 atomic scatter would sum in
// a run-dependent order).  A tet cell is the hexahedron of its 6 Kuhn tets.
__device__ __forceinline__ int colour_cell(const AsmArgs &a, int t, int colour, int *cell)
{
    const int b0 = colour & 1, b1 = (colour >> 1) & 1, b2 = (colour >> 2) & 1;
    const int n0 = (a.cx - b0 + 1) >> 1, n1 = (a.cy - b1 + 1) >> 1, n2 = (a.cz - b2 + 1) >> 1;
    if (t >= n0 * n1 * n2) return 0;
    const int t0 = t % n0, t1 = (t / n0) % n1, t2 = t / (n0 * n1);
    *cell = (2 * t0 + b0) + a.cx * ((2 * t1 + b1) + a.cy * (2 * t2 + b2));
    return 1;
}

// Calls f(e) for the elements of one colour handled by thread t: on a
// structured level the element(s) of one parity cell (a tet cell holds 6
// Kuhn tets), on an unstructured level one element of the colour's list
// (element colours such that no two elements of a colour share a vertex).
template <int T, class F>
__device__ __forceinline__ void for_colour_elements(const AsmArgs &a, int colour, F &&f)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (a.elist) {
        if (t < a.nlist) f(a.elist[t]);
        return;
    }
    int cell;
    if (!colour_cell(a, t, colour, &cell)) return;
    if (T == UG4GB_TET) {
        for (int p = 0; p < 6; ++p) f(6 * cell + p);
    } else {
        f(cell);
    }
}

// Launches kern(a, colour) once per colour of level L (parity cells of a
// structured level, element lists of an unstructured one), 128 threads a block.
template <class K>
void launch_coloured(Ctx &c, const Level &L, AsmArgs a, K kern)
{
    if (L.structured) {
        a.cx = L.nx - 1;
        a.cy = L.ny - 1;
        a.cz = (L.dim == 3) ? L.nz - 1 : 1;
        a.elist = nullptr;
        const int ncol = (L.dim == 3) ? 8 : 4;
        const int per = ((a.cx + 1) / 2) * ((a.cy + 1) / 2) * ((a.cz + 1) / 2);
        for (int colour = 0; colour < ncol; ++colour) kern(a, colour, div_up(per, 128));
    } else {
        for (int q = 0; q + 1 < (int)L.ecol_off.size(); ++q) {
            a.elist = L.ecol.p + L.ecol_off[q];
            a.nlist = L.ecol_off[q + 1] - L.ecol_off[q];
            if (a.nlist > 0) kern(a, q, div_up(a.nlist, 128));
        }
    }
}

// Calls f(std::integral_constant<int, T>) for the element type of level L.
template <class F>
void dispatch_elem(int elem_type, F &&f)
{
    switch (elem_type) {
        case UG4GB_QUAD: f(std::integral_constant<int, UG4GB_QUAD>()); break;
        case UG4GB_HEX: f(std::integral_constant<int, UG4GB_HEX>()); break;
        case UG4GB_TET: f(std::integral_constant<int, UG4GB_TET>()); break;
        case UG4GB_TRI: f(std::integral_constant<int, UG4GB_TRI>()); break;
        default: throw Error{UG4GB_ERR_INVALID, "unknown element type"};
    }
}

template <int T>
__device__ __forceinline__ void assemble_element(const AsmArgs &a, int e)
{
    using E = Elem<T>;
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
    elem_matrix<T>(X, a.K[e], a.vmodes > 0 ? &vf : nullptr, Aloc, (a.b || a.inst) ? vol : nullptr);
    if (a.inst) {
        // instationary AssembleLinear / AssembleJacobian
        // (lib_disc/spatial_disc/elem_disc/elem_disc_assemble_util.h:1124-1205, :520-535):
        // locA = sm0 M_e + sa0 A_e, each scaled term rounded before the sum
        double rhs[E::K];
        if (a.b) {
#pragma unroll
            for (int i = 0; i < E::K; ++i) {
                const double fi =
                    a.f ? a.f[ev[i]] : (a.use_seed ? 2.0 * hash_uniform(a.f_seed, (uint64_t)ev[i]) - 1.0 : 0.0);
                const double fv = __dmul_rn(fi, vol[i]);
                double r = 0.0, au = 0.0;
                if (a.sa0 != 0.0) r = __dmul_rn(a.sa0, fv);
                // previous time point: -sm1 (M_e u_old), -sa1 (A_e u_old), +sa1 f_e
                r = __dadd_rn(r, __dmul_rn(-a.sm1, __dmul_rn(vol[i], a.u_old[ev[i]])));
                if (a.sa1 != 0.0) {
#pragma unroll
                    for (int j = 0; j < E::K; ++j) au = __dadd_rn(au, __dmul_rn(Aloc[i][j], a.u_old[ev[j]]));
                    r = __dadd_rn(r, __dmul_rn(-a.sa1, au));
                    r = __dadd_rn(r, __dmul_rn(a.sa1, fv));
                }
                rhs[i] = r;
            }
        }
#pragma unroll
        for (int i = 0; i < E::K; ++i)
#pragma unroll
            for (int j = 0; j < E::K; ++j) {
                const double m = (i == j) ? __dmul_rn(a.sm0, vol[i]) : 0.0;
                Aloc[i][j] = __dadd_rn(m, __dmul_rn(a.sa0, Aloc[i][j]));
            }
#pragma unroll
        for (int i = 0; i < E::K; ++i)
#pragma unroll
            for (int j = 0; j < E::K; ++j) {
                int s = find_slot(a.rowptr, a.col, ev[i], ev[j]);
                if (s >= 0) a.val[s] = __dadd_rn(a.val[s], Aloc[i][j]);
            }
        if (a.b) {
#pragma unroll
            for (int i = 0; i < E::K; ++i) a.b[ev[i]] = __dadd_rn(a.b[ev[i]], rhs[i]);
        }
        return;
    }
#pragma unroll
    for (int i = 0; i < E::K; ++i)
#pragma unroll
        for (int j = 0; j < E::K; ++j) {
            int s = find_slot(a.rowptr, a.col, ev[i], ev[j]);
            if (s >= 0) a.val[s] += Aloc[i][j];
        }
    if (a.b) {
#pragma unroll
        for (int i = 0; i < E::K; ++i) {
            double fi = a.f ? a.f[ev[i]] : (a.use_seed ? 2.0 * hash_uniform(a.f_seed, (uint64_t)ev[i]) - 1.0 : 0.0);
            a.b[ev[i]] += fi * vol[i];
        }
    }
}

template <int T>
__global__ void __launch_bounds__(128) k_assemble(AsmArgs a, int colour)
{
    for_colour_elements<T>(a, colour, [&](int e) { assemble_element<T>(a, e); });
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

void launch_assemble(Ctx &c, const Level &L, const AsmArgs &a_in)
{
    dispatch_elem(L.elem_type, [&](auto tag) {
        constexpr int T = decltype(tag)::value;
        launch_coloured(c, L, a_in, [&](const AsmArgs &a, int colour, int g) {
            UG_LAUNCH(c, k_assemble<T>, g, 128, 0, a, colour);
        });
    });
}

void launch_dirichlet(Ctx &c, const Level &L, Csr &A, double *b)
{
    UG_LAUNCH(c, k_dirichlet_rows, div_up(L.nv, 256), 256, 0, L.bnd.p, L.nv, A.rowptr.p, A.col.p, A.val.p, b);
}

// ---------------------------------------------------------------- defect --
// Element defect (StdGlobAssembler::AssembleDefect, lib_disc/spatial_disc/
// elem_disc/elem_disc_assemble_util.h:578-690 stationary, 713-860
// instationary).  add_def_A_elem is the element operator applied to the local
// solution (the same sums the box method forms through the gradients at the
// integration points); add_rhs_elem is f_i |SCV_i|, add_def_M_elem
// |SCV_i| u_i.  Per element and corner i, with explicit rounding in the
// reference's order:
//   stationary:    r = (A_e u)_i + (-1) f_i |SCV_i|
//   instationary:  r = 0 + sm0 |SCV_i| u_i [+ sa0 (A_e u)_i + (-sa0) f_i |SCV_i|]
//                        + sm1 |SCV_i| uo_i [+ sa1 (A_e uo)_i + (-sa1) f_i |SCV_i|]
// then d_i += r (cells of one parity colour per launch: no two threads share
// a vertex).
template <int T>
__device__ __forceinline__ void defect_element(const AsmArgs &a, int e)
{
    using E = Elem<T>;
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
    elem_matrix<T>(X, a.K[e], a.vmodes > 0 ? &vf : nullptr, Aloc, vol);
    double uc[E::K];
#pragma unroll
    for (int j = 0; j < E::K; ++j) uc[j] = a.u[ev[j]];
#pragma unroll
    for (int i = 0; i < E::K; ++i) {
        const double fi = a.f ? a.f[ev[i]] : (a.use_seed ? 2.0 * hash_uniform(a.f_seed, (uint64_t)ev[i]) - 1.0 : 0.0);
        const double fv = __dmul_rn(fi, vol[i]);
        double au = 0.0;
#pragma unroll
        for (int j = 0; j < E::K; ++j) au = __dadd_rn(au, __dmul_rn(Aloc[i][j], uc[j]));
        double r;
        if (!a.inst) {
            r = __dadd_rn(au, __dmul_rn(-1.0, fv));
        } else {
            r = __dadd_rn(0.0, __dmul_rn(a.sm0, __dmul_rn(vol[i], uc[i])));
            if (a.sa0 != 0.0) {
                r = __dadd_rn(r, __dmul_rn(a.sa0, au));
                r = __dadd_rn(r, __dmul_rn(-a.sa0, fv));
            }
            r = __dadd_rn(r, __dmul_rn(a.sm1, __dmul_rn(vol[i], a.u_old[ev[i]])));
            if (a.sa1 != 0.0) {
                double ao = 0.0;
#pragma unroll
                for (int j = 0; j < E::K; ++j) ao = __dadd_rn(ao, __dmul_rn(Aloc[i][j], a.u_old[ev[j]]));
                r = __dadd_rn(r, __dmul_rn(a.sa1, ao));
                r = __dadd_rn(r, __dmul_rn(-a.sa1, fv));
            }
        }
        a.d[ev[i]] = __dadd_rn(a.d[ev[i]], r);
    }
}

template <int T>
__global__ void __launch_bounds__(128) k_defect(AsmArgs a, int colour)
{
    for_colour_elements<T>(a, colour, [&](int e) { defect_element<T>(a, e); });
}

// Dirichlet vertices: defect 0 (DirichletBoundary::adjust_defect,
// lagrange_dirichlet_boundary_impl.h:972-1033) or solution value 0
// (adjust_solution); both set the boundary entries to zero here
__global__ void k_zero_dirichlet(const unsigned char *bnd, int nv, double *x)
{
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v < nv && bnd[v]) x[v] = 0.0;
}

void launch_defect(Ctx &c, const Level &L, const AsmArgs &a_in)
{
    dispatch_elem(L.elem_type, [&](auto tag) {
        constexpr int T = decltype(tag)::value;
        launch_coloured(c, L, a_in, [&](const AsmArgs &a, int colour, int g) {
            UG_LAUNCH(c, k_defect<T>, g, 128, 0, a, colour);
        });
    });
    UG_LAUNCH(c, k_zero_dirichlet, div_up(L.nv, 256), 256, 0, L.bnd.p, L.nv, a_in.d);
}

void launch_dirichlet_values(Ctx &c, const Level &L, double *u)
{
    UG_LAUNCH(c, k_zero_dirichlet, div_up(L.nv, 256), 256, 0, L.bnd.p, L.nv, u);
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
    dispatch_elem(L.elem_type, [&](auto tag) {
        constexpr int T = decltype(tag)::value;
        UG_LAUNCH(c, k_coef_fourier<T>, g, 256, 0, L.coords.p, L.elems.p, L.ne, nmodes, k, phase, amp, factor, K);
    });
}

// coarse log K = mean of the children's log K.  Gather: each coarse element
// sums its structured children in increasing fine-element order (no atomics,
// same order as the oracle).  A fine Kuhn tet belongs to the coarse Kuhn tet
// whose permutation orders its centroid's offsets inside the coarse hex.
__device__ __forceinline__ int kuhn_perm_of(const double *off)
{
    if (off[0] >= off[1] && off[1] >= off[2]) return 0;
    if (off[0] >= off[2] && off[2] >= off[1]) return 1;
    if (off[1] >= off[0] && off[0] >= off[2]) return 2;
    if (off[1] >= off[2] && off[2] >= off[0]) return 3;
    if (off[2] >= off[0] && off[0] >= off[1]) return 4;
    return 5;
}

__global__ void k_coarsen_log(int elem_type, const double *fcoords, const int *felems, int fnx, int fny, int cnx,
                              int cny, int cne, const double *logf, double *logc)
{
    PDL_ENTRY();
    int ce = blockIdx.x * blockDim.x + threadIdx.x;
    if (ce >= cne) return;
    const int fx = fnx - 1, fy = fny - 1, cx = cnx - 1, cy = cny - 1;
    double s = 0.0;
    int n = 0;
    if (elem_type == UG4GB_QUAD) {
        int I = ce % cx, J = ce / cx;
        for (int b = 0; b < 2; ++b)
            for (int a = 0; a < 2; ++a) {
                s += logf[(2 * I + a) + fx * (2 * J + b)];
                ++n;
            }
    } else if (elem_type == UG4GB_HEX) {
        int I = ce % cx, J = (ce / cx) % cy, K = ce / (cx * cy);
        for (int c = 0; c < 2; ++c)
            for (int b = 0; b < 2; ++b)
                for (int a = 0; a < 2; ++a) {
                    s += logf[(2 * I + a) + fx * ((2 * J + b) + fy * (2 * K + c))];
                    ++n;
                }
    } else {
        int hc = ce / 6, pc = ce % 6;
        int I = hc % cx, J = (hc / cx) % cy, K = hc / (cx * cy);
        for (int c = 0; c < 2; ++c)
            for (int b = 0; b < 2; ++b)
                for (int a = 0; a < 2; ++a) {
                    int hf = (2 * I + a) + fx * ((2 * J + b) + fy * (2 * K + c));
                    for (int p = 0; p < 6; ++p) {
                        int e = 6 * hf + p;
                        double cc[3] = {0, 0, 0};
                        for (int q = 0; q < 4; ++q) {
                            int v = felems[4 * (size_t)e + q];
                            for (int d = 0; d < 3; ++d) cc[d] += fcoords[3 * (size_t)v + d];
                        }
                        double off[3];
                        const int ci[3] = {I, J, K};
                        for (int d = 0; d < 3; ++d) off[d] = cc[d] * 0.25 * (double)(cnx - 1) - (double)ci[d];
                        if (kuhn_perm_of(off) == pc) {
                            s += logf[e];
                            ++n;
                        }
                    }
                }
    }
    logc[ce] = s / (double)(n ? n : 1);
}

__global__ void k_exp(const double *m, int n, double *K)
{
    PDL_ENTRY();
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) K[e] = exp(m[e]);
}

void coarsen_log(Ctx &c, const Level &F, const Level &Cl, const double *logf, double *logc)
{
    UG_LAUNCH_PDL(c, k_coarsen_log, div_up(Cl.ne, 128), 128, 0, F.elem_type, F.coords.p, F.elems.p, F.nx, F.ny, Cl.nx,
              Cl.ny, Cl.ne, logf, logc);
}

// unstructured levels: the children of coarse element e are the fine
// elements e*nchild .. e*nchild + nchild - 1 (regular refinement order)
__global__ void k_coarsen_children(const double *logf, int nchild, int cne, double *logc)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= cne) return;
    double s = 0.0;
    for (int q = 0; q < nchild; ++q) s += logf[(size_t)e * nchild + q];
    logc[e] = s / (double)nchild;
}

void coarsen_log_children(Ctx &c, const Level &F, const Level &Cl, const double *logf, double *logc)
{
    UG_REQUIRE((int64_t)Cl.ne * (F.dim == 2 ? 4 : 8) == F.ne, UG4GB_ERR_INVALID,
               "coarse log coefficients: the fine level is not a regular refinement of the coarse one");
    UG_LAUNCH(c, k_coarsen_children, div_up(Cl.ne, 256), 256, 0, logf, F.dim == 2 ? 4 : 8, Cl.ne, logc);
}

void exp_elements(Ctx &c, const double *m, int n, double *K)
{
    UG_LAUNCH_PDL(c, k_exp, div_up(n, 256), 256, 0, m, n, K);
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
    dispatch_elem(L.elem_type, [&](auto tag) {
        constexpr int T = decltype(tag)::value;
        UG_LAUNCH(c, k_grad_logk<T>, gr, 128, 0, L.coords.p, L.elems.p, L.ne, L.bnd.p, K, u, lam, g);
    });
}

// sum of SCV volumes per vertex (d rhs_i / d f_i)
template <int T>
__global__ void k_scv_volumes(AsmArgs a, int colour, double *vol)
{
    using E = Elem<T>;
    for_colour_elements<T>(a, colour, [&](int e) {
        int ev[E::K];
        double X[E::K][E::DIM];
#pragma unroll
        for (int i = 0; i < E::K; ++i) {
            ev[i] = a.elems[(size_t)e * E::K + i];
#pragma unroll
            for (int d = 0; d < E::DIM; ++d) X[i][d] = a.coords[(size_t)ev[i] * E::DIM + d];
        }
        double v[E::K];
        scv_volumes<T>(X, v);
#pragma unroll
        for (int i = 0; i < E::K; ++i) vol[ev[i]] += v[i];
    });
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
    AsmArgs a{};
    a.coords = L.coords.p;
    a.elems = L.elems.p;
    a.ne = L.ne;
    dispatch_elem(L.elem_type, [&](auto tag) {
        constexpr int T = decltype(tag)::value;
        launch_coloured(c, L, a, [&](const AsmArgs &aa, int colour, int g) {
            UG_LAUNCH(c, k_scv_volumes<T>, g, 128, 0, aa, colour, vol.p);
        });
    });
    UG_LAUNCH(c, k_grad_source, div_up(L.nv, 256), 256, 0, vol.p, L.bnd.p, lam, L.nv, g);
    UG_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace ug4gb

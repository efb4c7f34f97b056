// k_sweep2.cu -- two consecutive damped-Jacobi steps of a structured 3D level
// in one pass over the level operator (temporal blocking).
//
// AssembledMultiGridCycle smooths every level with nu1 = nu2 = 2 damped-Jacobi
// steps (presmooth_and_restriction / prolongation_and_postsmooth,
// mg_solver_impl.hpp:1687-1966; Jacobi::step, jacobi.h:222).  Step k+1 reads
// the defect that step k wrote at every neighbour of a row, so kernels that
// apply one step per launch stream the operator once per step.  Here a block
// owns a 32 x TY column of the level's (x, y) plane and a chunk of its z
// planes, and marches through the chunk one plane at a time:
//   step A on plane p, for the block's vertices and a ring of one vertex:
//       d1 = dA - At xA        (xA staged in a ring of 3 shared planes)
//   step B on plane p - dir, for the block's vertices:
//       d2 = d1 - At d1        (d1 kept in a second ring of 3 shared planes)
// The block's operator rows are read from HBM once for both steps (kept in
// registers between the steps for 15 diagonals, re-read from L2 for 27), and
// the defect between the two steps never leaves the SM.  Consecutive z chunks
// march in opposite directions, so the two chunks that both read a plane next
// to their common boundary read it at about the same time (the second read
// comes from L2).
//
// In post-smoothing the structured prolongation (StdTransfer::prolongate,
// std_transfer_impl.h:721) is folded into step A: the staged xA is
// w = (P sc_c) * dfac, formed from the coarse correction while the plane is
// staged, and the block's rows add P sc_c to sc before step A's increment.
//
// The level operator is the column-scaled At = A diag(dinv) in the
// constant-offset layout: diagonal k couples vertex (x, y, z) with
// (x+dx_k, y+dy_k, z+dz_k); an entry whose neighbour lies outside the level is
// stored as 0 and multiplies a staged 0 here.  Each row update runs through
// the explicitly rounded helpers of k_solve.cuh in the diagonal order of the
// one-step kernels, so sc and the defects are bit-identical to theirs.
#include "k_solve.cuh"

namespace ug4gb {

namespace {

template <class V>
struct Sweep2Args {
    const V *__restrict__ val;   // At, constant-offset layout
    int ld;                      // stride between diagonals
    int nx, ny, nz;              // level vertices per direction
    int tz, ntx, nty;            // z planes per block, blocks along x and y
    const V *__restrict__ xA;    // step A's x
    const V *__restrict__ dbA;   // step A's defect; nullptr: same as xA
    const V *__restrict__ dinv;
    V *__restrict__ sc;
    V *__restrict__ dout;        // d2 (nullable)
    int modeA, modeB;
    const int *skip;
    const double *__restrict__ r_rho;
    RedArgs red;
    int rho_kind;
    double *__restrict__ z64;
};

// The stencils of the structured levels, in the order of the constant-offset
// layout (offsets dx + nx*(dy + ny*dz) ascending).  Compile-time, so every
// neighbour access below is one shared-memory load at an immediate offset.
//   27: hexahedra (Q1 coupling, (dz, dy, dx) lexicographic);
//   15: Kuhn tetrahedra around the (1,1,1) diagonal: the vertex, +-e_x, +-e_y,
//       +-e_z, +-(e_x+e_y), +-(e_x+e_z), +-(e_y+e_z), +-(1,1,1).
template <int S>
struct Stencil3;
template <>
struct Stencil3<27> {
    __host__ __device__ static constexpr int dx(int k) { return k % 3 - 1; }
    __host__ __device__ static constexpr int dy(int k) { return (k / 3) % 3 - 1; }
    __host__ __device__ static constexpr int dz(int k) { return k / 9 - 1; }
};
template <>
struct Stencil3<15> {
    __host__ __device__ static constexpr int dx(int k)
    {
        return k == 0 ? -1 : k == 1 ? 0 : k == 2 ? -1 : k == 3 ? 0 : k == 4 ? -1 : k == 5 ? 0 : k == 6 ? -1 :
               k == 7 ? 0 : k == 8 ? 1 : k == 9 ? 0 : k == 10 ? 1 : k == 11 ? 0 : k == 12 ? 1 : k == 13 ? 0 : 1;
    }
    __host__ __device__ static constexpr int dy(int k)
    {
        return k == 0 ? -1 : k == 1 ? -1 : k == 2 ? 0 : k == 3 ? 0 : k == 4 ? -1 : k == 5 ? -1 : k == 6 ? 0 :
               k == 7 ? 0 : k == 8 ? 0 : k == 9 ? 1 : k == 10 ? 1 : k == 11 ? 0 : k == 12 ? 0 : k == 13 ? 1 : 1;
    }
    __host__ __device__ static constexpr int dz(int k) { return k < 4 ? -1 : (k < 11 ? 0 : 1); }
};

// 4- or 8-byte asynchronous copy global -> shared; zero fill when !valid
template <class T>
__device__ __forceinline__ void cp_async(unsigned dst, const T *src, bool valid)
{
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");
    const int n = valid ? (int)sizeof(T) : 0;
    if constexpr (sizeof(T) == 4)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(dst), "l"(src), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ unsigned smem_addr(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ int ring4(int p) { return (p + 4) & 3; }

// widening of a level-precision value to FP64 (identity for FP64)
__device__ __forceinline__ double widen(double v) { return v; }
__device__ __forceinline__ double widen(float v) { return f32_to_f64(v); }

// shared-memory plan of one block
template <class V, int S, int TY>
struct Sweep2Smem {
    static constexpr int NTH = 32 * TY;
    static constexpr int XW = 36, XH = TY + 4, XP = XW * XH;   // staged xA: block columns + 2 on each side
    static constexpr int DW = 34, DH = TY + 2, DP = DW * DH;   // ring region: block columns + 1 on each side
    static constexpr int NX = (XP + NTH - 1) / NTH;            // staged xA elements per thread
    // byte offsets: FP64 r_rho first (8-byte alignment), then level-precision buffers
    static constexpr size_t RR = 0;                                  // [2][NTH] double
    static constexpr size_t M = RR + 2 * NTH * sizeof(double);       // [2][S][DP] operator tiles
    static constexpr size_t X = M + 2 * S * DP * sizeof(V);          // [4][XP] staged xA planes
    static constexpr size_t D = X + 4 * XP * sizeof(V);              // [4][DP] d1 planes
    static constexpr size_t B = D + 4 * DP * sizeof(V);              // [2][DP] step A's defect (dbA != xA)
    static constexpr size_t SC = B + 2 * DP * sizeof(V);             // [2][NTH] sc of the block's rows
    static constexpr size_t DI = SC + 2 * NTH * sizeof(V);           // [2][NTH] dinv of the block's rows
    static constexpr size_t BYTES = DI + 2 * NTH * sizeof(V);
};

// Software pipeline over the planes of the block's chunk.  Iteration p:
//   wait for the copies of plane p (operator tile of the ring region, step
//   A's defect, the block's sc and dinv) and of xA plane p+dir, issued one
//   iteration earlier; issue the copies of plane p+dir and xA plane p+2dir;
//   step A on plane p; step B on plane p-dir.
// Every position outside the level is zero-filled by the copies (operator
// entries and vectors alike), so step A gives d1 = 0 there without a branch.
// Planes live in rings of 4 buffers: plane p in slot (p + 4) & 3.
template <class V, int S, int TY, bool RHO>
__global__ void __launch_bounds__(32 * TY, S <= 15 ? 3 : 2) k_sweep2(const Sweep2Args<V> a)
{
    using SM = Sweep2Smem<V, S, TY>;
    using ST = Stencil3<S>;
    constexpr int NTH = SM::NTH, XW = SM::XW, XP = SM::XP, DW = SM::DW, DP = SM::DP, NX = SM::NX;
    constexpr int NRING = 2 * DW + 2 * TY;
    extern __shared__ __align__(16) unsigned char smem[];
    double *RR = reinterpret_cast<double *>(smem + SM::RR);
    V *M = reinterpret_cast<V *>(smem + SM::M);
    V *X = reinterpret_cast<V *>(smem + SM::X);
    V *D = reinterpret_cast<V *>(smem + SM::D);
    V *B = reinterpret_cast<V *>(smem + SM::B);
    V *SC = reinterpret_cast<V *>(smem + SM::SC);
    V *DI = reinterpret_cast<V *>(smem + SM::DI);
    PDL_ENTRY();
    if (a.skip && *a.skip) return;

    const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
    int b = blockIdx.x;
    const int bx = b % a.ntx;
    b /= a.ntx;
    const int by = b % a.nty, bz = b / a.nty;
    const int nx = a.nx, ny = a.ny, nz = a.nz, PS = nx * ny;
    const int x0 = bx * 32, y0 = by * TY;
    const int z0 = bz * a.tz, z1 = min(z0 + a.tz, nz);
    const int dir = (bz & 1) ? -1 : 1;
    const size_t ld = (size_t)a.ld;
    const bool sep_db = a.dbA != nullptr;
    const bool read_sc = a.modeA != SC_SET_FROM_BASE;

    // this thread's own vertex: ring-region slot, staged-plane slot, in-plane index
    const int gx = x0 + tx, gy = y0 + ty;
    const bool own = gx < nx && gy < ny;
    const int opos = (ty + 1) * DW + tx + 1, oxs = (ty + 2) * XW + tx + 2;
    const int ogi = own ? gx + nx * gy : 0;
    // this thread's place in step A's ring of one vertex around the block
    int rrx = 0, rry = 0;
    if (tid < NRING) {
        if (tid < DW) {
            rrx = tid;
        } else if (tid < 2 * DW) {
            rrx = tid - DW;
            rry = TY + 1;
        } else if (tid < 2 * DW + TY) {
            rry = tid - 2 * DW + 1;
        } else {
            rrx = DW - 1;
            rry = tid - 2 * DW - TY + 1;
        }
    }
    const int rpos = rry * DW + rrx, rxs = (rry + 1) * XW + rrx + 1;
    const int rgx = x0 - 1 + rrx, rgy = y0 - 1 + rry;
    const bool ring_in = tid < NRING && rgx >= 0 && rgx < nx && rgy >= 0 && rgy < ny;
    const int rgi = ring_in ? rgx + nx * rgy : 0;
    // the staged-plane elements this thread copies
    int xgi[NX];
    bool xin[NX];
#pragma unroll
    for (int j = 0; j < NX; ++j) {
        const int e = tid + j * NTH, rx = e % XW, ry = e / XW;
        const int x = x0 - 2 + rx, y = y0 - 2 + ry;
        xin[j] = e < XP && x >= 0 && x < nx && y >= 0 && y < ny;
        xgi[j] = xin[j] ? x + nx * y : 0;
    }
    const unsigned sM = smem_addr(M), sX = smem_addr(X), sB = smem_addr(B), sSC = smem_addr(SC),
                   sDI = smem_addr(DI), sRR = smem_addr(RR);

    auto stage_x = [&](int pl) {
        const bool zin = pl >= 0 && pl < nz;
        const int po = zin ? pl * PS : 0;
        const unsigned dst = sX + (unsigned)(ring4(pl) * XP * sizeof(V));
#pragma unroll
        for (int j = 0; j < NX; ++j) {
            const int e = tid + j * NTH;
            if (j + 1 < NX || e < XP) cp_async(dst + (unsigned)(e * sizeof(V)), a.xA + (po + xgi[j]), zin && xin[j]);
        }
    };
    // copies of plane p (and xA plane p + dir) into the buffers of parity p
    auto issue = [&](int p) {
        const int mb = p & 1;
        const bool zin = p >= 0 && p < nz;
        const int po = zin ? p * PS : 0;
        const unsigned mdst = sM + (unsigned)(mb * S * DP * sizeof(V));
        {
            const bool in = zin && own;
            const int i = po + ogi;
            const V *src = a.val + i;
#pragma unroll
            for (int k = 0; k < S; ++k)
                cp_async(mdst + (unsigned)((k * DP + opos) * sizeof(V)), src + k * ld, in);
            if (sep_db) cp_async(sB + (unsigned)((mb * DP + opos) * sizeof(V)), a.dbA + i, in);
            if (in && p >= z0 && p < z1) {
                if (read_sc) cp_async(sSC + (unsigned)((mb * NTH + tid) * sizeof(V)), a.sc + i, true);
                cp_async(sDI + (unsigned)((mb * NTH + tid) * sizeof(V)), a.dinv + i, true);
            }
            // r_rho of plane p - dir: used by step B one iteration after this copy
            const int q = p - dir;
            if (RHO && own && q >= z0 && q < z1)
                cp_async(sRR + (unsigned)((mb * NTH + tid) * sizeof(double)), a.r_rho + (q * PS + ogi), true);
        }
        if (tid < NRING) {
            const bool in = zin && ring_in;
            const int i = po + rgi;
            const V *src = a.val + i;
#pragma unroll
            for (int k = 0; k < S; ++k)
                cp_async(mdst + (unsigned)((k * DP + rpos) * sizeof(V)), src + k * ld, in);
            if (sep_db) cp_async(sB + (unsigned)((mb * DP + rpos) * sizeof(V)), a.dbA + i, in);
        }
        stage_x(p + dir);
        cp_async_commit();
    };

    V acur[S];   // operator row of this thread's vertex on the plane step B works on next
    V sc_cur = (V)0, di_cur = (V)0, sc_new = (V)0, di_new = (V)0;
    double rsum = 0.0;

    const int pstart = dir > 0 ? z0 - 1 : z1, pend = dir > 0 ? z1 + 1 : z0 - 2;
    stage_x(pstart - dir);
    stage_x(pstart);
    issue(pstart);
    for (int p = pstart; p != pend; p += dir) {
        cp_async_wait_all();
        __syncthreads();
        if (p + dir != pend) issue(p + dir);
        const int mb = p & 1;
        const V *Mo = M + mb * S * DP + opos;
        // ---- step A on plane p (block rows and ring; zero-filled outside)
        {
            const V *xm = X + ring4(p - 1) * XP, *xc = X + ring4(p) * XP, *xp = X + ring4(p + 1) * XP;
            const V *xom = xm + oxs, *xoc = xc + oxs, *xop = xp + oxs;
            V acc = (V)0;
#pragma unroll
            for (int k = 0; k < S; ++k) {
                const V *pl = ST::dz(k) < 0 ? xom : (ST::dz(k) > 0 ? xop : xoc);
                acc = fma_rn(Mo[k * DP], pl[ST::dy(k) * XW + ST::dx(k)], acc);
            }
            const V db = sep_db ? B[mb * DP + opos] : xoc[0];
            V *d1 = D + ring4(p) * DP;
            if (own && p >= z0 && p < z1) {
                const V so = read_sc ? SC[mb * NTH + tid] : (V)0;
                di_new = DI[mb * NTH + tid];
                d1[opos] = jacobi_row<V>(acc, db, di_new, a.modeA, so, sc_new);
            } else {
                d1[opos] = sub_rn(db, acc);
            }
            if (tid < NRING) {
                const V *Mr = M + mb * S * DP + rpos;
                const V *xrm = xm + rxs, *xrc = xc + rxs, *xrp = xp + rxs;
                V racc = (V)0;
#pragma unroll
                for (int k = 0; k < S; ++k) {
                    const V *pl = ST::dz(k) < 0 ? xrm : (ST::dz(k) > 0 ? xrp : xrc);
                    racc = fma_rn(Mr[k * DP], pl[ST::dy(k) * XW + ST::dx(k)], racc);
                }
                const V rdb = sep_db ? B[mb * DP + rpos] : xrc[0];
                d1[rpos] = sub_rn(rdb, racc);
            }
        }
        __syncthreads();
        // ---- step B on plane q (step A is done on q-1, q, q+1)
        const int q = p - dir;
        if (own && q >= z0 && q < z1) {
            const V *dm = D + ring4(q - 1) * DP + opos, *dc = D + ring4(q) * DP + opos,
                    *dp = D + ring4(q + 1) * DP + opos;
            V acc = (V)0;
#pragma unroll
            for (int k = 0; k < S; ++k) {
                const V *pl = ST::dz(k) < 0 ? dm : (ST::dz(k) > 0 ? dp : dc);
                acc = fma_rn(acur[k], pl[ST::dy(k) * DW + ST::dx(k)], acc);
            }
            V s;
            const V dn = jacobi_row<V>(acc, dc[0], di_cur, a.modeB, sc_cur, s);
            const int i = q * PS + ogi;
            a.sc[i] = s;
            if (a.dout) a.dout[i] = dn;
            if (RHO || a.z64) {
                const double s64 = widen(s);
                if (a.z64) a.z64[i] = s64;
                if (RHO) rsum += s64 * RR[mb * NTH + tid];
            }
        }
        // plane p's tile stays in place until the next iteration's wait
#pragma unroll
        for (int k = 0; k < S; ++k) acur[k] = Mo[k * DP];
        sc_cur = sc_new;
        di_cur = di_new;
    }
    cp_async_wait_all();
    if constexpr (RHO) {
        double v[1] = {rsum};
        KScal *ks = a.red.ks;
        const int kind = a.rho_kind;
        grid_reduce<NTH, 1>(v, a.red.partials, a.red.counter, [&](const double(&tot)[1]) {
            if (kind == 0) {
                ks->rho_old = tot[0];
            } else {
                ks->rho = tot[0];
                ks->beta = tot[0] / ks->rho_old;
                ks->rho_old = tot[0];
            }
        });
    }
}

constexpr int kTY = 8;

// offsets of the constant-offset layout as (dx, dy, dz) in {-1, 0, 1}^3
bool decode_offsets(const int *off, int S, int nx, int ny, signed char *dx, signed char *dy, signed char *dz)
{
    if (nx < 3 || ny < 3) return false;
    for (int k = 0; k < S; ++k) {
        bool found = false;
        for (int c = -1; c <= 1 && !found; ++c)
            for (int bb = -1; bb <= 1 && !found; ++bb)
                for (int aa = -1; aa <= 1 && !found; ++aa)
                    if (aa + nx * (bb + ny * c) == off[k]) {
                        dx[k] = (signed char)aa;
                        dy[k] = (signed char)bb;
                        dz[k] = (signed char)c;
                        found = true;
                    }
        if (!found) return false;
    }
    return true;
}

// the layout's offsets are those of the compile-time stencil of width S
template <int S>
bool stencil_is(const int *off, int nx, int ny)
{
    for (int k = 0; k < S; ++k)
        if (off[k] != Stencil3<S>::dx(k) + nx * (Stencil3<S>::dy(k) + ny * Stencil3<S>::dz(k))) return false;
    return true;
}
bool stencil_matches(const int *off, int S, int nx, int ny)
{
    if (nx < 3 || ny < 3) return false;
    if (S == 27) return stencil_is<27>(off, nx, ny);
    if (S == 15) return stencil_is<15>(off, nx, ny);
    return false;
}

struct Stencil {
    signed char dx[kMaxDiag], dy[kMaxDiag], dz[kMaxDiag];
};

// counts stored entries that are nonzero although their grid neighbour lies
// outside the level (the one-step kernels would multiply them with the
// vertex the offset wraps around to; the fused kernel with 0)
template <class V>
__global__ void k_count_wrapped(const V *__restrict__ val, int ld, int S, Stencil st, int nx, int ny, int nz,
                                unsigned int *count)
{
    const int n = nx * ny * nz;
    unsigned int bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int x = i % nx, y = (i / nx) % ny, z = i / (nx * ny);
        for (int k = 0; k < S; ++k) {
            const int xx = x + st.dx[k], yy = y + st.dy[k], zz = z + st.dz[k];
            const bool inside = xx >= 0 && xx < nx && yy >= 0 && yy < ny && zz >= 0 && zz < nz;
            if (!inside && val[(size_t)k * ld + i] != (V)0) ++bad;
        }
    }
    if (bad) atomicAdd(count, bad);
}

template <class V, int S, bool RHO>
void launch_sweep2(Ctx &c, const Sweep2Args<V> &a, int blocks)
{
    constexpr size_t bytes = Sweep2Smem<V, S, kTY>::BYTES;
    UG_LAUNCH_PDL(c, (k_sweep2<V, S, kTY, RHO>), blocks, 32 * kTY, bytes, a);
}

template <class V, int S>
void sweep2_attributes()
{
    const int bytes = (int)Sweep2Smem<V, S, kTY>::BYTES;
    UG_CUDA(cudaFuncSetAttribute(k_sweep2<V, S, kTY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    UG_CUDA(cudaFuncSetAttribute(k_sweep2<V, S, kTY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

}  // namespace

template <class V>
bool smooth_pair(Ctx &c, const OpMat<V> &At, const GridPair &gp, const V *xA, const V *dbA, const V *dinv, V *sc,
                 V *dout, int modeA, int modeB, const int *skip, const double *r_rho, RedArgs *red, int rho_kind,
                 double *z64)
{
    if constexpr (sizeof(V) != 4) {
        return false;   // FP64 steps are bound by the FP64 FMA rate, not by operator bytes
    } else {
        if (!(c.sweep_fusion & 1) || At.kind != 1 || gp.dim != 3) return false;
        const Dia<V> &D = At.dia;
        if (D.S != 15 && D.S != 27) return false;
        const int nx = gp.nx, ny = gp.ny, nz = gp.nz;
        if ((int64_t)nx * ny * nz != D.nrows || D.nrows != D.ncols) return false;
        if (!(c.sweep_fusion & 2) && D.nrows < c.sweep_fusion_min_rows) return false;
        if (modeB == SC_SET_FROM_BASE) return false;
        Sweep2Args<V> a{};
        if (!stencil_matches(D.off.o, D.S, nx, ny)) return false;
        a.val = D.val.p;
        a.ld = D.ld;
        a.nx = nx;
        a.ny = ny;
        a.nz = nz;
        a.tz = c.sweep_fusion_tz > 0 ? c.sweep_fusion_tz : 16;
        a.ntx = (int)div_up(nx, 32);
        a.nty = (int)div_up(ny, kTY);
        const int nzc = (int)div_up(nz, a.tz);
        const int64_t blocks = (int64_t)a.ntx * a.nty * nzc;
        if (blocks > kRedMaxBlocks) return false;
        a.xA = xA;
        a.dbA = dbA;
        a.dinv = dinv;
        a.sc = sc;
        a.dout = dout;
        a.modeA = modeA;
        a.modeB = modeB;
        a.skip = skip;
        a.r_rho = r_rho;
        if (red) a.red = *red;
        a.rho_kind = rho_kind;
        a.z64 = z64;
        const bool rho = r_rho != nullptr;
        if (D.S == 15) {
            if (rho) launch_sweep2<V, 15, true>(c, a, (int)blocks);
            else launch_sweep2<V, 15, false>(c, a, (int)blocks);
        } else {
            if (rho) launch_sweep2<V, 27, true>(c, a, (int)blocks);
            else launch_sweep2<V, 27, false>(c, a, (int)blocks);
        }
        return true;
    }
}

template <class V>
bool sweep2_supported(Ctx &c, const OpMat<V> &At, const GridPair &gp)
{
    if constexpr (sizeof(V) != 4) {
        return false;
    } else {
        if (At.kind != 1 || gp.dim != 3) return false;
        const Dia<V> &D = At.dia;
        if (D.S != 15 && D.S != 27) return false;
        if ((int64_t)gp.nx * gp.ny * gp.nz != D.nrows || D.nrows != D.ncols) return false;
        if (!stencil_matches(D.off.o, D.S, gp.nx, gp.ny)) return false;
        Stencil st{};
        if (!decode_offsets(D.off.o, D.S, gp.nx, gp.ny, st.dx, st.dy, st.dz)) return false;
        DevBuf<unsigned int> cnt;
        cnt.alloc(1);
        UG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned int), c.stream));
        UG_LAUNCH(c, k_count_wrapped<V>, row_grid(c, D.nrows), 256, 0, D.val.p, D.ld, D.S, st, gp.nx, gp.ny, gp.nz,
                  cnt.p);
        unsigned int bad = 0;
        UG_CUDA(cudaMemcpyAsync(&bad, cnt.p, sizeof(bad), cudaMemcpyDeviceToHost, c.stream));
        UG_CUDA(cudaStreamSynchronize(c.stream));
        if (bad) return false;
        // dynamic shared memory above 48 KB is opted into once, outside any capture
        if (D.S == 15) sweep2_attributes<V, 15>();
        else sweep2_attributes<V, 27>();
        return true;
    }
}
template bool sweep2_supported<float>(Ctx &, const OpMat<float> &, const GridPair &);
template bool sweep2_supported<double>(Ctx &, const OpMat<double> &, const GridPair &);

template bool smooth_pair<float>(Ctx &, const OpMat<float> &, const GridPair &, const float *, const float *,
                                 const float *, float *, float *, int, int, const int *, const double *, RedArgs *, int,
                                 double *);
template bool smooth_pair<double>(Ctx &, const OpMat<double> &, const GridPair &, const double *, const double *,
                                  const double *, double *, double *, int, int, const int *, const double *,
                                  RedArgs *, int, double *);

}  // namespace ug4gb

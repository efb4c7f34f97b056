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
//       d1 = dA - At xA        (xA staged in a ring of shared planes)
//   step B on plane p - dir, for the block's vertices:
//       d2 = d1 - At d1        (d1 kept in a second ring of shared planes)
// The block's operator tile of a plane (all diagonals, the block's lines and
// the ring) arrives with ONE tiled TMA load into shared memory, issued one
// plane ahead and completed on an mbarrier; the rows are read from HBM once
// for both steps, and the defect between the steps never leaves the SM.
// Consecutive z chunks march in opposite directions, so the two chunks that
// both read a plane next to their common boundary read it at about the same
// time (the second read comes from L2).
//
// TMA needs 16-byte multiples for the strides of the tensor it reads, so the
// operator is kept a second time for this kernel with every grid line padded
// to a multiple of 4 values: value (x, y, z) of diagonal k at
// ((k*nz + z)*ny + y)*xpad + x.  The tensor map gives the hardware the level
// extents, and it fills everything outside them with zeros.
//
// The level operator is the column-scaled At = A diag(dinv): diagonal k
// couples vertex (x, y, z) with (x+dx_k, y+dy_k, z+dz_k); an entry whose
// neighbour lies outside the level is 0 (checked at set-up).  Each row update
// runs through the explicitly rounded helpers of k_solve.cuh in the diagonal
// order of the one-step kernels, so sc and the defects are bit-identical to
// theirs.
#include <cuda.h>

#include "k_solve.cuh"

namespace ug4gb {

namespace {

template <class V>
struct Sweep2Args {
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
    int *err;                    // set when a bounded wait for the block's own copies runs out
    // failure test only (0 in every solve): extra bytes block 0 announces for
    // its first operator plane, which no copy delivers, so that its bounded
    // wait runs out (the give-up path exercised without a fault)
    unsigned test_extra_tx;
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

// ---- asynchronous copies ----------------------------------------------------
// 4- or 8-byte copy global -> shared (cp.async); zero fill when !valid
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

// tiled TMA load of a 4D box at (c0, c1, c2, c3) into shared memory,
// completion counted in bytes on an mbarrier
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *map, int c0, int c1, int c2, int c3,
                                            unsigned bar)
{
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(dst),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(bar)
        : "memory");
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity)
{
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for a phase of the block's own copies: gives up after about a
// second, reports it through *err and lets the kernel run to its end
// bounded by time, whatever try_wait's own suspension is: 0.5 s (a copy
// that has not landed by then is reported, never waited for indefinitely)
constexpr unsigned long long kWaitNs = 500000000ULL;
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int *err)
{
    const unsigned long long t0 = global_ns();
    for (unsigned t = 0;; ++t) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((t & 63u) == 63u && global_ns() - t0 > kWaitNs) break;
    }
    if (err) atomicExch(err, 1);
    return false;
}

__device__ __forceinline__ int ring4(int p) { return (p + 4) & 3; }

// widening of an FP32 level value to FP64 (integer path, as the one-step kernels)
__device__ __forceinline__ double widen(float v) { return f32_to_f64(v); }

// shared-memory plan of one block
template <class V, int S, int TY>
struct Sweep2Smem {
    static constexpr int NTH = 32 * TY;
    static constexpr int NL = TY + 2;                            // grid lines of step A (block + ring)
    static constexpr int LW = 40;                                // values per line of the operator box: x0-4 .. x0+35
    static constexpr int XW = 36, XH = TY + 4, XP = XW * XH;     // staged xA: block columns + 2 on each side
    static constexpr int DW = 34, DH = TY + 2, DP = DW * DH;     // ring region: block columns + 1 on each side
    static constexpr int NX = (XP + NTH - 1) / NTH;              // staged xA elements per thread
    static constexpr int MT = S * NL * LW;                       // operator box of one plane (elements)
    static constexpr size_t MTB = (MT * sizeof(V) + 127) / 128 * 128;
    // byte offsets (TMA destinations 128-byte aligned)
    static constexpr size_t BAR = 0;                                 // 2 mbarriers
    static constexpr size_t M = 128;                                 // [2] operator boxes [S][NL][LW]
    static constexpr size_t RR = M + 2 * MTB;                        // [2][NTH] double
    static constexpr size_t X = RR + 2 * NTH * sizeof(double);       // [4][XP] staged xA planes
    static constexpr size_t D = X + 4 * XP * sizeof(V);              // [4][DP] d1 planes
    static constexpr size_t B = D + 4 * DP * sizeof(V);              // [2][DP] step A's defect (dbA != xA)
    static constexpr size_t SC = B + 2 * DP * sizeof(V);             // [2][NTH] sc of the block's rows
    static constexpr size_t DI = SC + 2 * NTH * sizeof(V);           // [2][NTH] dinv of the block's rows
    static constexpr size_t BYTES = DI + 2 * NTH * sizeof(V) + 128;   // + slack to align the base to 128
};

// Software pipeline over the planes of the block's chunk.  Iteration p:
//   wait for the copies of plane p (issued one iteration earlier): the
//   operator box (one TMA load on the mbarrier of its buffer) and step A's
//   defect, the block's sc, dinv and r_rho, and xA plane p+dir (cp.async,
//   zero-filled outside the level); issue the copies of plane p+dir and xA
//   plane p+2dir; step A on plane p; step B on plane p-dir.
// Planes live in rings of 4 buffers (plane p in slot (p + 4) & 3), operator
// boxes in 2 (parity of p).  The box of plane p starts at (x0-4, y0-1, p, 0):
// a 16-byte aligned x, the block's lines and the ring, all diagonals.
template <class V, int S, int TY, bool RHO>
__global__ void __launch_bounds__(32 * TY, S <= 15 ? 3 : 2)
    k_sweep2(const __grid_constant__ CUtensorMap tmap, const Sweep2Args<V> a)
{
    using SM = Sweep2Smem<V, S, TY>;
    using ST = Stencil3<S>;
    constexpr int NTH = SM::NTH, NL = SM::NL, LW = SM::LW, XW = SM::XW, XP = SM::XP, DW = SM::DW, DP = SM::DP;
    constexpr int NX = SM::NX, MT = SM::MT;
    constexpr int MTE = (int)(SM::MTB / sizeof(V));   // elements between the two operator buffers
    constexpr int NRING = 2 * DW + 2 * TY;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    // the plan starts at the first 128-byte boundary of the dynamic window
    unsigned char *smem = smem_raw + ((128u - (smem_addr(smem_raw) & 127u)) & 127u);
    const V *M = reinterpret_cast<const V *>(smem + SM::M);
    const double *RR = reinterpret_cast<const double *>(smem + SM::RR);
    const V *X = reinterpret_cast<const V *>(smem + SM::X);
    V *D = reinterpret_cast<V *>(smem + SM::D);
    const V *B = reinterpret_cast<const V *>(smem + SM::B);
    const V *SC = reinterpret_cast<const V *>(smem + SM::SC);
    const V *DI = reinterpret_cast<const V *>(smem + SM::DI);
    const unsigned s0 = smem_addr(smem);
    const unsigned sBar = s0 + SM::BAR, sM = s0 + SM::M, sX = s0 + SM::X, sB = s0 + SM::B, sSC = s0 + SM::SC,
                   sDI = s0 + SM::DI, sRR = s0 + SM::RR;
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

    if (tid == 0) {
        mbar_init(sBar, 1);
        mbar_init(sBar + 8, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    const int pstart = dir > 0 ? z0 - 1 : z1, pend = dir > 0 ? z1 + 1 : z0 - 2;
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
        if (tid == 0) {
            // the block's reads of this buffer (its previous use, ordered by the
            // barrier before this call) precede the asynchronous copy into it
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const bool test = a.test_extra_tx && p == pstart && blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0;
            mbar_arrive_expect_tx(sBar + 8 * mb, (unsigned)(MT * sizeof(V)) + (test ? a.test_extra_tx : 0u));
            tma_load_4d(sM + (unsigned)(mb * SM::MTB), &tmap, x0 - 4, y0 - 1, p, 0, sBar + 8 * mb);
        }
        const bool in = zin && own;
        const int i = (zin ? p * PS : 0) + ogi;
        if (sep_db) cp_async(sB + (unsigned)((mb * DP + opos) * sizeof(V)), a.dbA + i, in);
        if (in && p >= z0 && p < z1) {
            if (read_sc) cp_async(sSC + (unsigned)((mb * NTH + tid) * sizeof(V)), a.sc + i, true);
            cp_async(sDI + (unsigned)((mb * NTH + tid) * sizeof(V)), a.dinv + i, true);
        }
        // r_rho of plane p - dir: used by step B one iteration after this copy
        const int q = p - dir;
        if (RHO && own && q >= z0 && q < z1)
            cp_async(sRR + (unsigned)((mb * NTH + tid) * sizeof(double)), a.r_rho + (q * PS + ogi), true);
        if (sep_db && tid < NRING)
            cp_async(sB + (unsigned)((mb * DP + rpos) * sizeof(V)), a.dbA + ((zin ? p * PS : 0) + rgi), zin && ring_in);
        stage_x(p + dir);
        cp_async_commit();
    };

    V acur[S], anew[S];   // operator row of this thread's vertex: plane of step B / of step A
    V sc_cur = (V)0, di_cur = (V)0, sc_new = (V)0, di_new = (V)0;
    double rsum = 0.0;
    unsigned phase = 0;   // bit b: parity of the next phase of operator buffer b
    bool ok = true;

    stage_x(pstart - dir);
    stage_x(pstart);
    issue(pstart);
    for (int p = pstart; p != pend; p += dir) {
        const int mb = p & 1;
        cp_async_wait_all();
        const unsigned par = (phase >> mb) & 1u;
        if (ok) ok = mbar_wait(sBar + 8 * mb, par, a.err);
        phase ^= 1u << mb;
        // the block gives up together when a wait ran out: no further copies
        // are issued, the copy of this plane gets one more bounded wait, and
        // the block still joins the grid reduction below (its result is
        // discarded: the host reports the error after the solve)
        if (!__syncthreads_and(ok)) {
            if (tid == 0) (void)mbar_wait(sBar + 8 * mb, par, nullptr);
            break;
        }
        if (p + dir != pend) issue(p + dir);
        const bool zin = p >= 0 && p < nz;
        const V *Mo = M + mb * MTE + (ty + 1) * LW + tx + 4;
        // ---- step A on plane p (block rows and ring)
        {
            const V *xom = X + ring4(p - 1) * XP + oxs, *xoc = X + ring4(p) * XP + oxs,
                    *xop = X + ring4(p + 1) * XP + oxs;
            V *d1 = D + ring4(p) * DP;
            V dn = (V)0;
            if (zin && own) {
                V acc = (V)0;
#pragma unroll
                for (int k = 0; k < S; ++k) {
                    const V *pl = ST::dz(k) < 0 ? xom : (ST::dz(k) > 0 ? xop : xoc);
                    anew[k] = Mo[k * NL * LW];
                    acc = fma_rn(anew[k], pl[ST::dy(k) * XW + ST::dx(k)], acc);
                }
                const V db = sep_db ? B[mb * DP + opos] : xoc[0];
                if (p >= z0 && p < z1) {
                    const V so = read_sc ? SC[mb * NTH + tid] : (V)0;
                    di_new = DI[mb * NTH + tid];
                    dn = jacobi_row<V>(acc, db, di_new, a.modeA, so, sc_new);
                } else {
                    dn = sub_rn(db, acc);
                }
            }
            d1[opos] = dn;
            if (tid < NRING) {
                V rdn = (V)0;
                if (zin && ring_in) {
                    const V *Mr = M + mb * MTE + rry * LW + rrx + 3;
                    const V *xrm = X + ring4(p - 1) * XP + rxs, *xrc = X + ring4(p) * XP + rxs,
                            *xrp = X + ring4(p + 1) * XP + rxs;
                    V racc = (V)0;
#pragma unroll
                    for (int k = 0; k < S; ++k) {
                        const V *pl = ST::dz(k) < 0 ? xrm : (ST::dz(k) > 0 ? xrp : xrc);
                        racc = fma_rn(Mr[k * NL * LW], pl[ST::dy(k) * XW + ST::dx(k)], racc);
                    }
                    const V rdb = sep_db ? B[mb * DP + rpos] : xrc[0];
                    rdn = sub_rn(rdb, racc);
                }
                d1[rpos] = rdn;
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
            const V dnb = jacobi_row<V>(acc, dc[0], di_cur, a.modeB, sc_cur, s);
            const int i = q * PS + ogi;
            a.sc[i] = s;
            if (a.dout) a.dout[i] = dnb;
            if (RHO || a.z64) {
                const double s64 = widen(s);
                if (a.z64) a.z64[i] = s64;
                if (RHO) rsum += s64 * RR[mb * NTH + tid];
            }
        }
#pragma unroll
        for (int k = 0; k < S; ++k) acur[k] = anew[k];
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

// the padded operator copy: value (x, y, z) of diagonal k at ((k*nz + z)*ny + y)*xpad + x
__global__ void k_pad_operator(const float *__restrict__ val, int ld, int S, int nx, int ny, int nz, int xpad,
                               float *__restrict__ out)
{
    const size_t n = (size_t)nx * ny * nz, total = n * S;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
        const int k = (int)(t / n);
        const int i = (int)(t - (size_t)k * n);
        const int x = i % nx, yz = i / nx;   // yz = y + ny*z
        out[((size_t)k * nz * ny + yz) * xpad + x] = val[(size_t)k * ld + i];
    }
}

template <int S, bool RHO>
void launch_sweep2(Ctx &c, const CUtensorMap &map, const Sweep2Args<float> &a, int blocks)
{
    constexpr size_t bytes = Sweep2Smem<float, S, kTY>::BYTES;
    UG_LAUNCH_PDL(c, (k_sweep2<float, S, kTY, RHO>), blocks, 32 * kTY, bytes, map, a);
}

template <int S>
void sweep2_attributes()
{
    const int bytes = (int)Sweep2Smem<float, S, kTY>::BYTES;
    UG_CUDA(cudaFuncSetAttribute(k_sweep2<float, S, kTY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    UG_CUDA(cudaFuncSetAttribute(k_sweep2<float, S, kTY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
}

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_tiled()
{
    static EncodeTiled fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        UG_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
        UG_REQUIRE(p && q == cudaDriverEntryPointSuccess, UG4GB_ERR_CUDA, "cuTensorMapEncodeTiled not available");
        fn = reinterpret_cast<EncodeTiled>(p);
    }
    return fn;
}

}  // namespace

// the fused pairs run on a level of n vertices (the bit mask
// Ctx::sweep_fusion)
static bool sweep2_wanted(const Ctx &c, int64_t n)
{
    return (c.sweep_fusion & 1) && ((c.sweep_fusion & 2) || n >= c.sweep_fusion_min_rows);
}

struct Sweep2Op {
    CUtensorMap map;        // 4D (x, y, z, diagonal) over pad, box 40 x (TY+2) x 1 x S
    DevBuf<float> pad;      // the operator with 16-byte aligned grid lines
    int S = 0, nx = 0, ny = 0, nz = 0;
};

template <class V>
std::shared_ptr<Sweep2Op> sweep2_prepare(Ctx &c, const OpMat<V> &At, const GridPair &gp)
{
    if constexpr (sizeof(V) != 4) {
        return nullptr;   // FP64 steps are bound by the FP64 FMA rate, not by operator bytes
    } else {
        if (At.kind != 1 || gp.dim != 3) return nullptr;
        const Dia<V> &D = At.dia;
        if (D.S != 15 && D.S != 27) return nullptr;
        // no padded copy for a level the pairs will not run on
        if (!sweep2_wanted(c, (int64_t)gp.nx * gp.ny * gp.nz)) return nullptr;
        if ((int64_t)gp.nx * gp.ny * gp.nz != D.nrows || D.nrows != D.ncols) return nullptr;
        if (!stencil_matches(D.off.o, D.S, gp.nx, gp.ny)) return nullptr;
        Stencil st{};
        if (!decode_offsets(D.off.o, D.S, gp.nx, gp.ny, st.dx, st.dy, st.dz)) return nullptr;
        DevBuf<unsigned int> cnt;
        cnt.alloc(1);
        UG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(unsigned int), c.stream));
        UG_LAUNCH(c, k_count_wrapped<V>, row_grid(c, D.nrows), 256, 0, D.vals(), D.ld, D.S, st, gp.nx, gp.ny, gp.nz,
                  cnt.p);
        unsigned int bad = 0;
        UG_CUDA(cudaMemcpyAsync(&bad, cnt.p, sizeof(bad), cudaMemcpyDeviceToHost, c.stream));
        UG_CUDA(cudaStreamSynchronize(c.stream));
        if (bad) return nullptr;

        auto op = std::make_shared<Sweep2Op>();
        op->S = D.S;
        op->nx = gp.nx;
        op->ny = gp.ny;
        op->nz = gp.nz;
        const int xpad = (gp.nx + 3) / 4 * 4;
        const size_t total = (size_t)D.S * gp.nz * gp.ny * xpad;
        op->pad.alloc(total);
        UG_CUDA(cudaMemsetAsync(op->pad.p, 0, op->pad.bytes(), c.stream));
        UG_LAUNCH(c, k_pad_operator, c.num_sms * 8, 256, 0, D.vals(), D.ld, D.S, gp.nx, gp.ny, gp.nz, xpad, op->pad.p);
        const cuuint64_t dims[4] = {(cuuint64_t)gp.nx, (cuuint64_t)gp.ny, (cuuint64_t)gp.nz, (cuuint64_t)D.S};
        const cuuint64_t strides[3] = {(cuuint64_t)xpad * 4, (cuuint64_t)xpad * gp.ny * 4,
                                       (cuuint64_t)xpad * gp.ny * gp.nz * 4};
        const cuuint32_t box[4] = {(cuuint32_t)Sweep2Smem<float, 15, kTY>::LW, (cuuint32_t)(kTY + 2), 1,
                                   (cuuint32_t)D.S};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        const CUresult r = encode_tiled()(&op->map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, op->pad.p, dims, strides, box,
                                          estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                          CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        UG_REQUIRE(r == CUDA_SUCCESS, UG4GB_ERR_CUDA, "cuTensorMapEncodeTiled failed for the fused smoother");
        UG_CUDA(cudaStreamSynchronize(c.stream));
        // dynamic shared memory above 48 KB is opted into once, outside any capture
        if (D.S == 15) sweep2_attributes<15>();
        else sweep2_attributes<27>();
        return op;
    }
}

template <class V>
bool smooth_pair(Ctx &c, const Sweep2Op *op, const GridPair &gp, const V *xA, const V *dbA, const V *dinv, V *sc,
                 V *dout, int modeA, int modeB, const int *skip, const double *r_rho, RedArgs *red, int rho_kind,
                 double *z64)
{
    if constexpr (sizeof(V) != 4) {
        return false;
    } else {
        if (!op) return false;
        if (op->nx != gp.nx || op->ny != gp.ny || op->nz != gp.nz) return false;
        const int64_t n = (int64_t)gp.nx * gp.ny * gp.nz;
        if (!sweep2_wanted(c, n)) return false;
        if (modeB == SC_SET_FROM_BASE) return false;
        Sweep2Args<float> a{};
        a.nx = gp.nx;
        a.ny = gp.ny;
        a.nz = gp.nz;
        a.tz = c.sweep_fusion_tz > 0 ? c.sweep_fusion_tz : 16;
        a.ntx = (int)div_up(gp.nx, 32);
        a.nty = (int)div_up(gp.ny, kTY);
        const int nzc = (int)div_up(gp.nz, a.tz);
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
        a.err = c.dev_err.p;
        // the failure test applies to one launch only
        a.test_extra_tx = (unsigned)c.sweep_wait_test;
        c.sweep_wait_test = 0;
        c.dev_err_possible = true;
        const bool rho = r_rho != nullptr;
        if (op->S == 15) {
            if (rho) launch_sweep2<15, true>(c, op->map, a, (int)blocks);
            else launch_sweep2<15, false>(c, op->map, a, (int)blocks);
        } else {
            if (rho) launch_sweep2<27, true>(c, op->map, a, (int)blocks);
            else launch_sweep2<27, false>(c, op->map, a, (int)blocks);
        }
        return true;
    }
}

template std::shared_ptr<Sweep2Op> sweep2_prepare<float>(Ctx &, const OpMat<float> &, const GridPair &);
template std::shared_ptr<Sweep2Op> sweep2_prepare<double>(Ctx &, const OpMat<double> &, const GridPair &);
template bool smooth_pair<float>(Ctx &, const Sweep2Op *, const GridPair &, const float *, const float *,
                                 const float *, float *, float *, int, int, const int *, const double *, RedArgs *, int,
                                 double *);
template bool smooth_pair<double>(Ctx &, const Sweep2Op *, const GridPair &, const double *, const double *,
                                  const double *, double *, double *, int, int, const int *, const double *,
                                  RedArgs *, int, double *);

}  // namespace ug4gb

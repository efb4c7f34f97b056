// k_coarse.cu -- the coarse end of a multigrid V-cycle in one launch.
//
// Below a few thousand rows a level's smoothing steps, transfers and the base
// solve are latency work: every one of them is a separate launch of about
// 1.5-2 us in which a handful of blocks touch a few KB.  The coarse levels of
// the hierarchy are therefore cycled by a single block of 1024 threads with
// every such level (operator, Jacobi factors, vectors) and the base inverse
// in shared memory, one __syncthreads between the phases that the separate
// launches would order:
//   per level, from the entry level down:   nu1 damped-Jacobi steps, then
//                                           restriction to the level below
//   base level:                             sc = Ainv d (dense inverse)
//   per level, back up:                     prolongation (sc += t, w = t*dfac),
//                                           nu2 damped-Jacobi steps
// (AssembledMultiGridCycle::lmgc, mg_solver_impl.hpp:2091-2134, for
// gamma = 1 below the entry level).  Every row is computed with the
// arithmetic of the separate kernels (diagonal-layout row product with the
// same clamped columns and FMA order, jacobi_row, prolong_value,
// restrict_row, the base solve's per-lane partial sums and warp reduction),
// so corrections are bit-identical to those of the separate launches.
#include "k_solve.cuh"

namespace ug4gb {

constexpr int kCoarseThreads = 1024;

// Asynchronous copies global -> shared (cp.async): every thread issues all
// of its copies before waiting, so the staging of a few hundred KB is bound
// by bandwidth, not by one load's latency per thread and iteration.
__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void *dst, const void *src)
{
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// bytes from src to dst, both 16-byte aligned: 16-byte copies, the tail
// (bytes % 16, a multiple of 4) in 4-byte copies
__device__ __forceinline__ void stage(void *dst, const void *src, size_t bytes)
{
    const size_t n16 = bytes / 16;
    for (size_t i = threadIdx.x; i < n16; i += blockDim.x)
        cp_async16((char *)dst + 16 * i, (const char *)src + 16 * i);
    for (size_t i = 16 * n16 + 4 * threadIdx.x; i < bytes; i += 4 * blockDim.x)
        cp_async4((char *)dst + i, (const char *)src + i);
}

// (At x)_i of the diagonal layout: DiaMV::dot's order of operations (the
// same clamped columns, the same FMA chain), with the operator a (S x ld)
// and x in shared memory; S fixed at compile time, so every load of the row
// is issued before the chain starts
template <class V, int S>
__device__ __forceinline__ V coarse_dot(const CoarseLevel<V> &L, const V *a, const V *x, int i)
{
    V av[S], xv[S];
#pragma unroll
    for (int k = 0; k < S; ++k) {
        int j = i + L.off[k];
        j = j < 0 ? 0 : (j >= L.ncols ? L.ncols - 1 : j);
        av[k] = a[k * L.ld + i];
        xv[k] = x[j];
    }
    V acc = (V)0;
#pragma unroll
    for (int k = 0; k < S; ++k) acc = fma_rn(av[k], xv[k], acc);
    return acc;
}

// one damped-Jacobi step of level L: dn = db - At x; sc (=|+=) dinv*(db|dn);
// dout (nullable) = dn.  Everything in shared memory.
template <class V, int S>
__device__ __forceinline__ void coarse_step(const CoarseLevel<V> &L, const V *a, const V *dinv, const V *x,
                                            const V *db, V *sc, V *dout, int mode)
{
    for (int i = threadIdx.x; i < L.n; i += blockDim.x) {
        const V acc = coarse_dot<V, S>(L, a, x, i);
        V s;
        const V dn = jacobi_row<V>(acc, db[i], dinv[i], mode, mode == SC_SET_FROM_BASE ? (V)0 : sc[i], s);
        if (dout) dout[i] = dn;
        sc[i] = s;
    }
}

template <class V, int S>
__global__ void __launch_bounds__(kCoarseThreads, 1)
    k_coarse_cycle(const CoarsePlan<V> *__restrict__ plan, const int *skip)
{
    __shared__ CoarsePlan<V> P;
    extern __shared__ __align__(16) unsigned char coarse_smem[];
    const int tid = threadIdx.x, nt = blockDim.x;
    {
        // the plan, the operators, the Jacobi factors and the base inverse
        // are written at set-up, never by a solve kernel: staged before the
        // wait for the predecessor, so the copies overlap its tail
        static_assert(sizeof(CoarsePlan<V>) % 16 == 0, "plan copied in 16-byte words");
        const int4 *src = reinterpret_cast<const int4 *>(plan);
        int4 *dst = reinterpret_cast<int4 *>(&P);
        for (int i = tid; i < (int)(sizeof(CoarsePlan<V>) / 16); i += nt) dst[i] = __ldg(src + i);
    }
    __syncthreads();
    double *ainv = reinterpret_cast<double *>(coarse_smem);
    V *vr = reinterpret_cast<V *>(coarse_smem + P.vbase);
    stage(ainv, P.Ainv, (size_t)P.nbase * P.nbase * sizeof(double));
    for (int l = 1; l < P.m; ++l) {
        const CoarseLevel<V> &L = P.lev[l];
        stage(vr + L.aofs, L.val, (size_t)L.S * L.ld * sizeof(V));
        stage(vr + L.iofs, L.dinv, (size_t)L.n * sizeof(V));
        stage(vr + L.fofs, L.dfac, (size_t)L.n * sizeof(V));
    }
    pdl_trigger();
    pdl_wait();
    if (skip && *skip) {
        cp_async_wait_all();   // no copy outlives the block
        return;
    }
    const int top = P.m - 1;
    // vectors of level l: sc, dA, dB, w (the base level: sc, dA)
    auto vsc = [&](int l) { return vr + P.lev[l].vofs; };
    auto vdA = [&](int l) { return vr + P.lev[l].vofs + P.lev[l].n; };
    auto vdB = [&](int l) { return vr + P.lev[l].vofs + 2 * P.lev[l].n; };
    auto vw = [&](int l) { return vr + P.lev[l].vofs + 3 * P.lev[l].n; };
    {
        V *d = vdA(top);
        for (int i = tid; i < P.lev[top].n; i += nt) d[i] = P.d_in[i];
    }
    cp_async_wait_all();
    __syncthreads();
    // ---- down: pre-smoothing and restriction (the defect of a level
    // arrives in its dA; the steps alternate dA -> dB -> dA ...)
    for (int l = top; l >= 1; --l) {
        const CoarseLevel<V> &L = P.lev[l];
        const V *a = vr + L.aofs, *dinv = vr + L.iofs;
        V *sc = vsc(l), *dA = vdA(l), *dB = vdB(l);
        if (P.nu1 == 0) {
            for (int i = tid; i < L.n; i += nt) sc[i] = (V)0;
            __syncthreads();
        }
        V *cur = dA;
        for (int k = 0; k < P.nu1; ++k) {
            V *out = (cur == dA) ? dB : dA;
            coarse_step<V, S>(L, a, dinv, cur, cur, sc, out, k == 0 ? SC_SET_FROM_BASE : SC_ADD_FROM_BASE);
            __syncthreads();
            cur = out;
        }
        const GridPair &g = L.gp;
        V *dc = vdA(l - 1);
        const int nc = g.cnx * g.cny * g.cnz;
        for (int q = tid; q < nc; q += nt)
            restrict_row<V>(g, cur, dc, q % g.cnx, (q / g.cnx) % g.cny, q / (g.cnx * g.cny));
        __syncthreads();
    }
    // ---- base: sc = Ainv d, one warp per row (k_base_solve's partial sums);
    // an FP32 defect is widened once per entry first (conversions issue on
    // the FP64 pipe), into the nbase doubles after Ainv
    {
        const int n0 = P.nbase, warp = tid >> 5, lane = tid & 31;
        const double *d;
        if constexpr (sizeof(V) == sizeof(double)) {
            d = reinterpret_cast<const double *>(vdA(0));
        } else {
            double *dw = ainv + n0 * n0;
            const V *dv = vdA(0);
            for (int j = tid; j < n0; j += nt) dw[j] = (double)dv[j];
            __syncthreads();
            d = dw;
        }
        V *sc = vsc(0);
        for (int row = warp; row < n0; row += nt >> 5) {
            const double *arow = ainv + row * n0;
            double s = 0.0;
            for (int j = lane; j < n0; j += 32) s = fma_rn(arow[j], d[j], s);
            s = warp_sum(s);
            if (lane == 0) sc[row] = (V)s;
        }
        __syncthreads();
    }
    // ---- up: prolongation and post-smoothing
    for (int l = 1; l <= top; ++l) {
        const CoarseLevel<V> &L = P.lev[l];
        const GridPair &g = L.gp;
        const V *a = vr + L.aofs, *dinv = vr + L.iofs, *dfac = vr + L.fofs;
        V *sc = vsc(l), *dA = vdA(l), *dB = vdB(l), *w = vw(l);
        const V *scc = vsc(l - 1);
        for (int f = tid; f < L.n; f += nt) {
            V t = prolong_value<V>(g, scc, f % g.nx, (f / g.nx) % g.ny, f / (g.nx * g.ny));
            if (g.dprol != 1.0) t = mul_rn(t, (V)g.dprol);
            sc[f] = add_rn(sc[f], t);
            if (P.nu2 > 0) w[f] = mul_rn(t, dfac[f]);
        }
        __syncthreads();
        V *dbase = (P.nu1 & 1) ? dB : dA;   // the defect after pre-smoothing
        for (int k = 0; k < P.nu2; ++k) {
            const V *x = (k == 0) ? w : dbase;
            V *out = (k < P.nu2 - 1) ? ((dbase == dA) ? dB : dA) : nullptr;
            coarse_step<V, S>(L, a, dinv, x, dbase, sc, out, SC_ADD_FROM_NEW);
            __syncthreads();
            if (out) dbase = out;
        }
    }
    {
        const V *sc = vsc(top);
        for (int i = tid; i < P.lev[top].n; i += nt) P.sc_out[i] = sc[i];
    }
}

template <class V>
void coarse_cycle(Ctx &c, const CoarsePlan<V> *plan_dev, int S, size_t smem_bytes, const int *skip)
{
    switch (S) {
    case 9: UG_LAUNCH_PDL(c, (k_coarse_cycle<V, 9>), 1, kCoarseThreads, smem_bytes, plan_dev, skip); break;
    case 15: UG_LAUNCH_PDL(c, (k_coarse_cycle<V, 15>), 1, kCoarseThreads, smem_bytes, plan_dev, skip); break;
    case 27: UG_LAUNCH_PDL(c, (k_coarse_cycle<V, 27>), 1, kCoarseThreads, smem_bytes, plan_dev, skip); break;
    default: throw Error{UG4GB_ERR_INVALID, "coarse cycle: unsupported stencil width"};
    }
}

bool coarse_width_ok(int S) { return S == 9 || S == 15 || S == 27; }

template <class V>
void coarse_prepare(size_t smem_bytes)
{
    UG_CUDA(cudaFuncSetAttribute(k_coarse_cycle<V, 9>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes));
    UG_CUDA(cudaFuncSetAttribute(k_coarse_cycle<V, 15>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes));
    UG_CUDA(cudaFuncSetAttribute(k_coarse_cycle<V, 27>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_bytes));
}

template void coarse_cycle<double>(Ctx &, const CoarsePlan<double> *, int, size_t, const int *);
template void coarse_cycle<float>(Ctx &, const CoarsePlan<float> *, int, size_t, const int *);
template void coarse_prepare<double>(size_t);
template void coarse_prepare<float>(size_t);

}  // namespace ug4gb

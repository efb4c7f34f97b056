// k_rap.cu -- Galerkin coarse operator M = R A P on the GPU.
//
// AssembledMultiGridCycle::init_rap_operator (mg_solver_impl.hpp:830-1012)
// builds every coarse level operator as R_l A_l P_l of the level above with
// AddMultiplyOf(M, R, A, P) (lib_algebra/algebra_common/sparsematrix_util.h:
// 167-241) into an empty M: for row i, the products R_ik A_kl P_lj are taken
// in the order k (R's row), l (A's row), j (P's row), entries equal to 0 are
// skipped, ab = R_ik A_kl is rounded, and ab * P_lj is rounded before it is
// added to the running value of column j; every column reached is stored,
// also when its sum cancels to 0.
//
// Here one thread owns one row of M and keeps its running values in a small
// open-addressing table in shared memory (kRapCap slots; the structured
// hierarchies reach at most 27 columns per coarse row).  Two passes: the
// first counts the distinct columns of each row (rows beyond kRapCap set an
// overflow flag), a scan gives the row pointers, the second accumulates the
// values in the order above with explicitly rounded multiplies and adds (so
// they equal the reference's products bit for bit) and writes the row with
// its columns sorted.
#include "common.cuh"

namespace ug4gb {

namespace {

constexpr int kRapRows = 32;   // rows (threads) per block

__device__ __forceinline__ int rap_slot(int j) { return (int)(((unsigned)j * 2654435761u) >> 26); }   // 64 slots
static_assert(kRapCap == 64, "rap_slot hashes into 64 slots");

// pass 0: rowlen[i] = distinct columns of row i; pass 1: write the row
__global__ void __launch_bounds__(kRapRows) k_rap(const int *__restrict__ Rrp, const int *__restrict__ Rci,
                                                  const double *__restrict__ Rva, const int *__restrict__ Arp,
                                                  const int *__restrict__ Aci, const double *__restrict__ Ava,
                                                  const int *__restrict__ Prp, const int *__restrict__ Pci,
                                                  const double *__restrict__ Pva, int nr, int pass,
                                                  int *__restrict__ rowlen, const int *__restrict__ rowptr,
                                                  int *__restrict__ Mci, double *__restrict__ Mva,
                                                  int *__restrict__ overflow)
{
    // one padding slot per thread row spreads the threads' tables over the banks
    __shared__ int key[kRapRows][kRapCap + 1];
    __shared__ double acc[kRapRows][kRapCap + 1];
    const int t = threadIdx.x, i = blockIdx.x * kRapRows + t;
    if (i >= nr) return;
    int *kk = key[t];
    double *aa = acc[t];
    for (int s = 0; s < kRapCap; ++s) kk[s] = -1;
    int count = 0;
    bool full = false;
    for (int a = Rrp[i]; a < Rrp[i + 1] && !full; ++a) {
        const double rv = Rva[a];
        if (rv == 0.0) continue;
        const int k = Rci[a];
        for (int b = Arp[k]; b < Arp[k + 1] && !full; ++b) {
            const double av = Ava[b];
            if (av == 0.0) continue;
            const int l = Aci[b];
            const double ab = __dmul_rn(rv, av);
            for (int c = Prp[l]; c < Prp[l + 1]; ++c) {
                const double pv = Pva[c];
                if (pv == 0.0) continue;
                const int j = Pci[c];
                int s = rap_slot(j), probes = 0;
                while (kk[s] != -1 && kk[s] != j && probes < kRapCap) {
                    s = (s + 1) & (kRapCap - 1);
                    ++probes;
                }
                if (probes == kRapCap) {
                    full = true;
                    break;
                }
                if (kk[s] == -1) {
                    kk[s] = j;
                    aa[s] = 0.0;
                    ++count;
                }
                if (pass == 1) aa[s] = __dadd_rn(aa[s], __dmul_rn(ab, pv));
            }
        }
    }
    if (full) {
        atomicExch(overflow, 1);
        if (pass == 0) rowlen[i] = 0;
        return;
    }
    if (pass == 0) {
        rowlen[i] = count;
        return;
    }
    // the row's columns in increasing order
    int *oc = Mci + rowptr[i];
    double *ov = Mva + rowptr[i];
    int m = 0;
    for (int s = 0; s < kRapCap; ++s) {
        if (kk[s] == -1) continue;
        const int j = kk[s];
        const double v = aa[s];
        int q = m++;
        while (q > 0 && oc[q - 1] > j) {
            oc[q] = oc[q - 1];
            ov[q] = ov[q - 1];
            --q;
        }
        oc[q] = j;
        ov[q] = v;
    }
}

}  // namespace

void csr_rap(Ctx &c, const Csr &R, const Csr &A, const Csr &P, Csr &M)
{
    UG_REQUIRE(R.ncols == A.nrows && A.ncols == P.nrows, UG4GB_ERR_INVALID, "Galerkin product: size mismatch");
    const int nr = R.nrows;
    M.nrows = nr;
    M.ncols = P.ncols;
    DevBuf<int> len, flag;
    len.alloc((size_t)nr + 1);
    flag.alloc(1);
    UG_CUDA(cudaMemsetAsync(len.p, 0, len.bytes(), c.stream));
    UG_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), c.stream));
    const unsigned grid = div_up(nr > 0 ? nr : 1, kRapRows);
    UG_LAUNCH(c, k_rap, grid, kRapRows, 0, R.rowptr.p, R.col.p, R.val.p, A.rowptr.p, A.col.p, A.val.p, P.rowptr.p,
              P.col.p, P.val.p, nr, 0, len.p, (const int *)nullptr, (int *)nullptr, (double *)nullptr, flag.p);
    int over = 0;
    UG_CUDA(cudaMemcpyAsync(&over, flag.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    UG_CUDA(cudaStreamSynchronize(c.stream));
    UG_REQUIRE(!over, UG4GB_ERR_INVALID, "Galerkin product R A P: a coarse row reaches more than 64 columns");
    M.rowptr.alloc((size_t)nr + 1);
    int64_t nnz = 0;
    exclusive_scan_int(c, len.p, M.rowptr.p, nr + 1, &nnz);
    M.nnz = nnz;
    M.col.alloc(nnz > 0 ? nnz : 1);
    M.val.alloc(nnz > 0 ? nnz : 1);
    UG_LAUNCH(c, k_rap, grid, kRapRows, 0, R.rowptr.p, R.col.p, R.val.p, A.rowptr.p, A.col.p, A.val.p, P.rowptr.p,
              P.col.p, P.val.p, nr, 1, (int *)nullptr, (const int *)M.rowptr.p, M.col.p, M.val.p, flag.p);
    UG_CUDA(cudaStreamSynchronize(c.stream));
}

}  // namespace ug4gb

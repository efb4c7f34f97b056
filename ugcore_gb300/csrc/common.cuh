// common.cuh -- internal types and helpers of libug4gb (sm_103a).
//
// Device data layout (all levels resident in HBM):
//   grid level   coords  nv*dim FP64 (AoS), elems ne*k int32 (corners in
//                reference order), bnd nv uint8, parents nv*8 int32 + npar.
//   CRS          rowptr (n+1) int32, col nnz int32 (sorted per row),
//                val nnz FP64 -- the defragmented ug::SparseMatrix form.
//   SELL-32      slices of 32 consecutive rows; slice s stores width w_s =
//                max row length, entries column-major inside the slice
//                (entry k of row 32s+lane at sptr[s] + 32k + lane), padded
//                with (col = a valid column, val = 0).  Thread-per-row loads
//                are fully coalesced (32 x 4 or 8 bytes per k).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/ug4gb.h"

namespace ug4gb {

struct Error {
    int code;
    std::string msg;
};

#define UG_CUDA(call)                                                                              \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            throw ::ug4gb::Error{e_ == cudaErrorMemoryAllocation ? UG4GB_ERR_NOMEM : UG4GB_ERR_CUDA, \
                                 std::string(#call) + ": " + cudaGetErrorString(e_)};              \
    } while (0)

#define UG_REQUIRE(cond, code, text)                                                               \
    do {                                                                                           \
        if (!(cond)) throw ::ug4gb::Error{(code), std::string(text)};                             \
    } while (0)

#ifdef UG4GB_GUARDED
// guarded build: buffers between guard zones (ug4gb_debug_guard_check)
constexpr size_t kGuardBytes = 4096;
void guard_register(char *base, void *user, size_t user_bytes);
char *guard_release(void *user) noexcept;
#endif

// NVTX range around a library call ("ug4gb:<call>"), visible to profilers
// that record NVTX (ncu --nvtx, Nsight Systems); it costs nothing while no
// such tool is attached.  Stands in for ugcore's PROFILE_FUNC regions.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Owning device buffer (move-only).
template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevBuf &operator=(DevBuf &&o) noexcept
    {
        if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
        return *this;
    }
    ~DevBuf() { release(); }
    void alloc(size_t count)
    {
        if (count == n && p) return;
        release();
        if (count == 0) return;
#ifdef UG4GB_GUARDED
        char *base = nullptr;
        UG_CUDA(cudaMalloc((void **)&base, count * sizeof(T) + 2 * kGuardBytes));
        p = (T *)(base + kGuardBytes);
        guard_register(base, p, count * sizeof(T));
#else
        UG_CUDA(cudaMalloc((void **)&p, count * sizeof(T)));
#endif
        n = count;
    }
    void release()
    {
#ifdef UG4GB_GUARDED
        if (p) cudaFree(guard_release(p));
#else
        if (p) cudaFree(p);
#endif
        p = nullptr;
        n = 0;
    }
    size_t bytes() const { return n * sizeof(T); }
};

// Per-launch CUDA-event profiler (off by default; never active while a
// graph is being captured).  Records (kernel name, rows) -> event pairs.
struct ProfRec {
    std::string name;
    cudaEvent_t a, b;
};

struct Ctx {
    int device = 0;
    int num_sms = 152;
    cudaStream_t stream = nullptr;
    std::string err;
    int64_t launches = 0;
    bool profiling = false;
    bool allow_dia = true;      // operators with <= 27 offsets use the diagonal layout
    bool pdl = true;            // programmatic dependent launch on the solve path
    // structured levels: stationary assembly row by row (1), and with one
    // coefficient for all elements from the one interior stencil (2)
    int row_assembly = 2;
    // two Jacobi steps per pass on structured 3D FP32 levels (bit mask):
    // 1 = on, 2 = every level size (else >= sweep_fusion_min_rows vertices)
    int sweep_fusion = 0;
    int sweep_fusion_min_rows = 1 << 18;
    int sweep_fusion_tz = 8;    // z planes per block
    int sweep_wait_test = 0;    // failure test only: bytes no copy delivers (fused sweeps' bounded waits run out)
    // levels above the base cycled by the one-block coarse kernel (-1: as
    // many as its cost model finds faster than separate launches, 0: none)
    int coarse_levels = -1;
    std::string prof_tag;       // set by the orchestration (level / phase)
    std::vector<ProfRec> prof;
    std::vector<cudaEvent_t> ev_pool;
    // grid-reduction scratch: partial sums per block and a completion counter
    DevBuf<double> red_partials;        // kRedMaxBlocks * kRedMaxValues
    DevBuf<unsigned int> red_counter;   // one counter per reduction slot
    DevBuf<double> red_result;          // results of plain reductions
    DevBuf<int> dev_err;                // set by a kernel whose bounded device-side wait ran out
    bool dev_err_possible = false;      // a kernel that can set dev_err was launched or captured
    double *host_pinned = nullptr;      // small pinned readback area
};

constexpr int kRedMaxBlocks = 16384;
constexpr int kRedMaxValues = 2;
constexpr int kSliceH = 32;

cudaEvent_t prof_event(Ctx &c);

// Kernel launch accounting; every launch of the library goes through this.
#define UG_LAUNCH(ctx, kernel, grid, block, shmem, ...)                                            \
    do {                                                                                           \
        cudaEvent_t ev_a_ = nullptr;                                                               \
        if ((ctx).profiling) {                                                                     \
            ev_a_ = ::ug4gb::prof_event(ctx);                                                      \
            UG_CUDA(cudaEventRecord(ev_a_, (ctx).stream));                                         \
        }                                                                                          \
        kernel<<<(grid), (block), (shmem), (ctx).stream>>>(__VA_ARGS__);                           \
        (ctx).launches++;                                                                          \
        UG_CUDA(cudaGetLastError());                                                               \
        if ((ctx).profiling) {                                                                     \
            cudaEvent_t ev_b_ = ::ug4gb::prof_event(ctx);                                          \
            UG_CUDA(cudaEventRecord(ev_b_, (ctx).stream));                                         \
            (ctx).prof.push_back(::ug4gb::ProfRec{(ctx).prof_tag + "|" + #kernel, ev_a_, ev_b_});  \
        }                                                                                          \
    } while (0)

// Programmatic dependent launch for the solve-path kernels: the next kernel
// of the stream is scheduled while the current one still runs, and waits in
// griddepcontrol.wait until its predecessor has completed and its memory is
// visible.  Every kernel launched this way starts with PDL_ENTRY(), before
// it reads anything (including its skip flag): a kernel that could finish
// without waiting would let its successor overtake its own predecessor.
__device__ __forceinline__ void pdl_entry()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
#define PDL_ENTRY() ::ug4gb::pdl_entry()
// The two halves, for kernels that first load data no kernel of the solve
// writes (operator values, Jacobi factors): those loads overlap the
// predecessor's tail instead of following it.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

#define UG_LAUNCH_PDL(ctx, kernel, grid, block, shmem, ...)                                        \
    do {                                                                                           \
        if (!(ctx).pdl || (ctx).profiling) {                                                       \
            UG_LAUNCH(ctx, kernel, grid, block, shmem, __VA_ARGS__);                               \
            break;                                                                                 \
        }                                                                                          \
        cudaLaunchConfig_t cfg_ = {};                                                              \
        cfg_.gridDim = dim3(grid);                                                                 \
        cfg_.blockDim = dim3(block);                                                               \
        cfg_.dynamicSmemBytes = (shmem);                                                           \
        cfg_.stream = (ctx).stream;                                                                \
        cudaLaunchAttribute at_[1];                                                                \
        at_[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;                            \
        at_[0].val.programmaticStreamSerializationAllowed = 1;                                     \
        cfg_.attrs = at_;                                                                          \
        cfg_.numAttrs = 1;                                                                         \
        UG_CUDA(cudaLaunchKernelEx(&cfg_, kernel, __VA_ARGS__));                                   \
        (ctx).launches++;                                                                          \
    } while (0)

inline unsigned div_up(size_t a, size_t b) { return (unsigned)((a + b - 1) / b); }

// --------------------------------------------------------------- CRS/SELL --
struct Csr {
    int nrows = 0, ncols = 0;
    int64_t nnz = 0;
    DevBuf<int> rowptr, col;
    DevBuf<double> val;
};

template <class T>
struct Sell {
    int nrows = 0, ncols = 0, nslices = 0;
    int64_t stored = 0;     // padded entry count
    DevBuf<int> sptr;       // nslices + 1
    DevBuf<int> swidth;     // nslices
    DevBuf<int> col;        // stored
    DevBuf<T> val;          // stored
};

template <class T>
struct SellView {
    int nrows;
    const int *__restrict__ sptr;
    const int *__restrict__ swidth;
    const int *__restrict__ col;
    const T *__restrict__ val;
};

template <class T>
inline SellView<T> view(const Sell<T> &s)
{
    return SellView<T>{s.nrows, s.sptr.p, s.swidth.p, s.col.p, s.val.p};
}

// Constant-offset (diagonal) layout: row i couples to columns i + off[k],
// k < S; values stored diagonal-major, val[k*nrows + i]; entries that are
// absent in the CRS (or fall outside the matrix) are 0 and their column is
// clamped into range.  Used automatically when a matrix has at most 27
// distinct column offsets (every level operator of a structured hierarchy:
// 9, 15 or 27 of them); it carries no column indices at all and its loads do
// not depend on each other.
constexpr int kMaxDiag = 32;
struct Offs {
    int o[kMaxDiag];
};

template <class T>
struct Dia {
    // the value array carries kGuard zero elements before diagonal 0 and
    // after the last one, so aligned bulk copies of a grid line that start
    // up to 4 elements early or end up to 64 elements late stay inside it
    static constexpr int kGuard = 64;
    int nrows = 0, ncols = 0, S = 0;
    int ld = 0;       // stride between diagonals: nrows rounded up to 32 (128-byte aligned rows of values)
    Offs off{};
    DevBuf<T> val;    // kGuard + S * ld + kGuard elements
    const T *vals() const { return val.p + kGuard; }
    T *vals() { return val.p + kGuard; }
};

// An operator in its solve format: SELL-32 (general) or diagonal.
template <class T>
struct OpMat {
    int kind = 0;   // 0 = SELL-32, 1 = diagonal
    int nrows = 0, ncols = 0;
    Sell<T> sell;
    Dia<T> dia;
    int64_t stored_bytes() const
    {
        if (kind == 1) return (int64_t)dia.S * dia.ld * (int64_t)sizeof(T);
        return sell.stored * (int64_t)(sizeof(T) + sizeof(int)) + (int64_t)sell.nslices * 8;
    }
};

// ------------------------------------------------------------- grid level --
struct Level {
    int elem_type = 0, dim = 2, k = 4;
    int nx = 0, ny = 0, nz = 1, nv = 0, ne = 0;   // nx, ny, nz: structured levels only
    bool structured = true;      // lexicographic box level (grid transfers, diagonal stencils)
    DevBuf<double> coords;
    DevBuf<int> elems;
    DevBuf<unsigned char> bnd;
    DevBuf<int> npar, par;       // parents in the next coarser level
    DevBuf<int> color;           // vertex colour (parity on structured levels)
    int ncolors = 0;             // vertex colours (multicolour Gauss-Seidel)
    // unstructured levels: elements grouped by colour, no two elements of a
    // colour sharing a vertex (the assembly's race-free scatter order)
    std::vector<int> ecol_off;   // colour q: ecol[ecol_off[q] .. ecol_off[q+1])
    DevBuf<int> ecol;
};

// ------------------------------------------------------ device utilities --
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Streaming loads of matrix data: read once per sweep, keep L1/L2 for vectors.
__device__ __forceinline__ double ld_stream(const double *p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float *p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int *p) { return __ldcs(p); }

// FP32 <-> FP64 conversions in integer arithmetic, from the IEEE-754 binary
// formats.  On GB300 the hardware conversions issue on the FP64 pipe at a
// fraction of the FMA rate, which made them the limiter of the FP64 vector
// kernels that also produce or consume the FP32 multigrid vectors.  Normal
// numbers and zeros take the integer path (widening is exact; narrowing
// rounds to nearest, ties to even, as cvt.rn.f32.f64); subnormal, out-of-
// range, infinite and NaN inputs fall back to the hardware conversion.  The
// fallbacks are separate, non-inlined functions so that the compiler cannot
// turn the rare branch into a select that runs the FP64-pipe conversion for
// every value.
static __device__ __noinline__ double f32_to_f64_hw(float f) { return (double)f; }
static __device__ __noinline__ float f64_to_f32_hw(double d) { return (float)d; }

__device__ __forceinline__ double f32_to_f64(float f)
{
    const unsigned int u = __float_as_uint(f);
    const unsigned int e = (u >> 23) & 0xffu;
    const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
    if (e == 0u && (u & 0x7fffffu) == 0u) return __longlong_as_double((long long)sgn);
    if (__builtin_expect(e == 0u || e == 0xffu, 0)) return f32_to_f64_hw(f);
    const unsigned long long bits =
        sgn | ((unsigned long long)(e + (1023u - 127u)) << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
    return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ float f64_to_f32(double d)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    const unsigned int sgn = (unsigned int)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7ffu);
    const unsigned long long m = b & 0xfffffffffffffULL;
    if (e == 0 && m == 0) return __uint_as_float(sgn);
    int fe = e - 1023 + 127;
    if (__builtin_expect(fe <= 0 || fe >= 255, 0)) return f64_to_f32_hw(d);
    unsigned int mant = (unsigned int)(m >> 29);
    const unsigned long long rest = m & ((1ULL << 29) - 1), half = 1ULL << 28;
    if (rest > half || (rest == half && (mant & 1u))) {
        mant += 1u;
        if (mant == (1u << 23)) {
            mant = 0u;
            fe += 1;
            if (__builtin_expect(fe >= 255, 0)) return f64_to_f32_hw(d);
        }
    }
    return __uint_as_float(sgn | ((unsigned int)fe << 23) | mant);
}

// W values of type T that fill 16 bytes, moved with one vector load/store
template <class T, int W>
struct alignas(16) Pack {
    T v[W];
};
template <class T, int W>
__device__ __forceinline__ Pack<T, W> ld_stream_pack(const T *p)
{
    static_assert(sizeof(T) * W == 16, "16-byte packs only");
    Pack<T, W> r;
    if constexpr (sizeof(T) == 4) {
        float4 q = __ldcs(reinterpret_cast<const float4 *>(p));
        r.v[0] = q.x, r.v[1] = q.y, r.v[2] = q.z, r.v[3] = q.w;
    } else {
        double2 q = __ldcs(reinterpret_cast<const double2 *>(p));
        r.v[0] = q.x, r.v[1] = q.y;
    }
    return r;
}
template <class T, int W>
__device__ __forceinline__ Pack<T, W> ld_pack(const T *p)
{
    return *reinterpret_cast<const Pack<T, W> *>(p);
}
template <class T, int W>
__device__ __forceinline__ void st_pack(T *p, const Pack<T, W> &v)
{
    *reinterpret_cast<Pack<T, W> *>(p) = v;
}

// Deterministic grid-wide sum of NV values per thread.  Each block reduces
// in a fixed tree, writes its partials, and the last block to finish sums
// the partials in block order and calls fin(total) with thread 0.
template <int NT, int NV, class Fin>
__device__ __forceinline__ void grid_reduce(const double (&v)[NV], double *partials, unsigned int *counter,
                                            Fin fin)
{
    __shared__ double sh[NV][NT / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = warp_sum(v[q]);
        if (lane == 0) sh[q][warp] = s;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = (lane < NT / 32) ? sh[q][lane] : 0.0;
            s = warp_sum(s);
            if (lane == 0) partials[q * kRedMaxBlocks + blockIdx.x] = s;
        }
        if (lane == 0) {
            __threadfence();
            unsigned t = atomicAdd(counter, 1u);
            is_last = (t == gridDim.x - 1);
        }
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double tot[NV];
#pragma unroll
    for (int q = 0; q < NV; ++q) {
        double s = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += NT) s += __ldcg(partials + q * kRedMaxBlocks + b);
        s = warp_sum(s);
        if (lane == 0) sh[q][warp] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = 0.0;
            for (int w = 0; w < NT / 32; ++w) s += sh[q][w];
            tot[q] = s;
        }
        *counter = 0u;
        fin(tot);
    }
}

// splitmix64 counter hash -> U[0,1), identical to the oracle's generator.
// m * 2^-53 for m < 2^53, built from the IEEE-754 fields with integer
// operations (the value is exact, the same as the converted product; the
// hardware integer-to-FP64 conversion issues on GB300's slow FP64 pipe)
__host__ __device__ __forceinline__ double u53_scaled(uint64_t m)
{
    if (m == 0) return 0.0;
#ifdef __CUDA_ARCH__
    const int top = 63 - __clzll((long long)m);
#else
    const int top = 63 - __builtin_clzll(m);
#endif
    // leading bit at position top: value 2^(top-53) * (1.mantissa)
    const uint64_t mant = (m << (52 - top)) & ((1ULL << 52) - 1);
    const uint64_t bits = ((uint64_t)(top - 53 + 1023) << 52) | mant;
    double d;
    memcpy(&d, &bits, sizeof(d));
    return d;
}

__host__ __device__ __forceinline__ double hash_uniform(uint64_t seed, uint64_t i)
{
    uint64_t z = (seed ^ (i * 0xD1B54A32D192ED03ULL)) + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z = z ^ (z >> 31);
    return u53_scaled(z >> 11);
}

// ----------------------------------------------------- host-side helpers --
bool is_device_ptr(const void *p);
// copies n elements from a host-or-device pointer into device memory
void copy_in(Ctx &c, void *dst_dev, const void *src, size_t bytes);
void copy_out(Ctx &c, void *dst, const void *src_dev, size_t bytes);

// kernels shared between translation units
void exclusive_scan_int(Ctx &c, const int *in, int *out, int n, int64_t *total_out);
void csr_from_elements(Ctx &c, const Level &L, Csr &A);
void csr_transpose(Ctx &c, const Csr &B, Csr &T, bool keep_zeros);
void csr_copy(Ctx &c, const Csr &src, Csr &dst);
// Galerkin product M = R A P (k_rap.cu), the product ugcore's AddMultiplyOf
// forms for set_rap(true); at most kRapCap distinct columns per row of M
constexpr int kRapCap = 64;
void csr_rap(Ctx &c, const Csr &R, const Csr &A, const Csr &P, Csr &M);
template <class T>
void sell_from_csr(Ctx &c, const Csr &A, Sell<T> &S, const double *col_scale /* nullable */);
// distinct column offsets (col - row) of A, sorted; false if more than max_s
bool csr_offsets(Ctx &c, const Csr &A, int max_s, std::vector<int> &offs);
template <class T>
void dia_from_csr(Ctx &c, const Csr &A, Dia<T> &D, const std::vector<int> &offs, const double *col_scale,
                  bool refill = false);
// solve format: diagonal when A is square with <= 27 offsets and allow_dia, else SELL-32
template <class T>
void op_from_csr(Ctx &c, const Csr &A, OpMat<T> &M, const double *col_scale, bool allow_dia);
// The layout an operator's solve format was built with (diagonal offsets or
// SELL-32 slices).  While the caller knows the CRS pattern is unchanged (the
// same level, re-assembled), op_from_csr_cached refills the values of the
// existing buffers in place: no host round trip, no allocation, the same
// device pointers (captured CUDA graphs stay valid).
struct OpLayout {
    bool known = false;
    int kind = 0;                 // 0 SELL-32, 1 diagonal
    int nrows = 0;
    int64_t nnz = 0;
    std::vector<int> offs;        // diagonal offsets (padded)
};
template <class T>
void op_from_csr_cached(Ctx &c, const Csr &A, OpMat<T> &M, const double *col_scale, bool allow_dia, OpLayout &lay);
// T = A^T (structural zeros kept) and perm[k] = position in A of the entry
// that lands at position k of T; transpose_values refills T's values from
// A's through perm (the same pattern)
void transpose_perm(Ctx &c, const Csr &A, Csr &T, DevBuf<int> &perm);
void transpose_values(Ctx &c, const Csr &A, Csr &T, const DevBuf<int> &perm);
// the same row pointers and column indices (one host round trip)
bool csr_same_pattern(Ctx &c, const Csr &A, const Csr &B);
// the pattern holds (j, i) for every (i, j) (one host round trip)
bool csr_pattern_symmetric(Ctx &c, const Csr &A);
// A = A^T in place for a symmetric pattern: every pair (i, j), (j, i) of
// values swapped; no extra memory
void csr_transpose_symmetric_inplace(Ctx &c, Csr &A);
void fill_double(Ctx &c, double *p, size_t n, double v);
// after a synchronisation of the stream: throws if a kernel reported that one
// of its bounded waits ran out (and clears the flag)
void check_device_error(Ctx &c);

}  // namespace ug4gb

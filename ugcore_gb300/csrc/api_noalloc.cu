// api_noalloc.cu -- ug4gb_vector_dot_noalloc: the FP64 dot product for
// callers that must not allocate device memory.
//
// Who needs it: a host application that already owns every byte of the GPU
// through its own allocator, or that calls in from a phase where a
// cudaMalloc/cudaFree would be wrong (cudaFree synchronises the whole
// device, and a failed allocation in the middle of a time step cannot be
// recovered).  Such a caller cannot create a ug4gb context (which allocates
// its reduction buffers), so this entry point takes plain device pointers
// and a stream and keeps its reduction scratch in a fixed, statically sized
// __device__ array of this library instead.
//
// Scratch and its limit: one FP64 partial per block of kChunk elements, at
// most kMaxBlocks blocks (64 KiB of partials plus one counter), so n is
// limited to kChunk * kMaxBlocks = 67,108,864 elements; larger n is rejected
// with UG4GB_ERR_INVALID before anything is launched.
//
// Set-up: the first call in each CUDA context (normally the primary context
// of a device, with that device current) looks up the device address of the
// scratch with cudaGetSymbolAddress.  The address is cached per context, by
// the context's process-unique id (cuCtxGetId), so a context created after
// cudaDeviceReset or by cuCtxCreate gets its own look-up.  That first call
// can make the CUDA runtime load this library's kernels onto the device
// (the runtime, not this library, then places the code and the 64 KiB array
// in device memory), so a caller with a strict no-allocation phase makes one
// call (n = 1 is enough) before it, and before any stream capture.
//
// Every call clears the block counter on the caller's stream before its
// launch (a memset, no allocation), so a call cut short by an earlier error
// cannot leave a count behind that corrupts the next result.
//
// Concurrency: all calls in one context share the one scratch array.  Calls
// that overlap in time on that device (two streams, or two host threads
// without ordering between them) race on it and give wrong results; order
// them on one stream or synchronise between them.
//
// Result: every block sums a fixed slice in a fixed order and the last block
// adds the partials in block order, so the value depends only on n and the
// data, not on the GPU or on timing.  It is a different summation order than
// ug4gb_vector_dot's grid-stride reduction, so the two agree to rounding.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/ug4gb.h"

namespace {

constexpr int kThreads = 256;
constexpr int kChunk = 8192;          // elements per block (32 per thread)
constexpr int kMaxBlocks = 8192;      // partial slots in the scratch
constexpr int64_t kMaxN = (int64_t)kChunk * kMaxBlocks;
static_assert(kMaxN == UG4GB_DOT_NOALLOC_MAX_N, "header limit out of date");

struct DotScratch {
    double partial[kMaxBlocks];
    unsigned int counter;             // blocks finished; must read 0 when a call starts
};

// zero-initialised when the module is loaded; every call clears the counter
// on its stream before the launch, and the last block resets it to 0
static __device__ __align__(256) DotScratch g_dot_scratch;

__device__ __forceinline__ double warp_sum64(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(kThreads) k_dot_static(const double *__restrict__ a, const double *__restrict__ b,
                                                          int64_t n, double *result, DotScratch *s)
{
    __shared__ double sh[kThreads / 32];
    __shared__ bool is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t lo = (int64_t)blockIdx.x * kChunk;
    const int64_t hi = (lo + kChunk < n) ? lo + kChunk : n;
    double sum = 0.0;
    for (int64_t i = lo + threadIdx.x; i < hi; i += kThreads) sum += __ldcs(a + i) * __ldcs(b + i);
    sum = warp_sum64(sum);
    if (lane == 0) sh[warp] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += sh[w];
        s->partial[blockIdx.x] = t;
        __threadfence();
        unsigned int done = atomicAdd(&s->counter, 1u);
        is_last = (done == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return;
    __threadfence();
    double tot = 0.0;
    for (int q = threadIdx.x; q < (int)gridDim.x; q += kThreads) tot += __ldcg(s->partial + q);
    tot = warp_sum64(tot);
    if (lane == 0) sh[warp] = tot;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kThreads / 32; ++w) t += sh[w];
        *result = t;
        s->counter = 0u;
    }
}

std::mutex g_setup_mutex;
struct ScratchEntry {
    unsigned long long ctx_id;
    DotScratch *p;
};
constexpr int kMaxContexts = 64;
ScratchEntry g_scratch[kMaxContexts] = {};
int g_num_scratch = 0;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// process-unique id of the current context (0 if unavailable)
unsigned long long current_context_id()
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (CtxGetCurrentFn)p;
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (CtxGetIdFn)p;
        (void)cudaGetLastError();
        looked_up = true;
    }
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c || get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

int fail(char *err, int cap, int code, const char *fmt, ...)
{
    if (err && cap > 0) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, (size_t)cap, fmt, ap);
        va_end(ap);
    }
    return code;
}

// device memory of the current device (plain or managed)
bool on_device(const void *p, int dev)
{
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == dev;
}

}  // namespace

extern "C" int ug4gb_vector_dot_noalloc(const double *a, const double *b, int64_t n, double *result, void *stream,
                                        char *err, int err_capacity)
{
    if (err && err_capacity > 0) err[0] = '\0';
    if (n < 0 || n > kMaxN)
        return fail(err, err_capacity, UG4GB_ERR_INVALID,
                    "ug4gb_vector_dot_noalloc: n = %lld outside [0, %lld] (the static scratch holds %d partials "
                    "of %d elements)",
                    (long long)n, (long long)kMaxN, kMaxBlocks, kChunk);
    if (!result || (n > 0 && (!a || !b)))
        return fail(err, err_capacity, UG4GB_ERR_INVALID, "ug4gb_vector_dot_noalloc: null pointer argument");
    if (((uintptr_t)a | (uintptr_t)b | (uintptr_t)result) % alignof(double) != 0)
        return fail(err, err_capacity, UG4GB_ERR_INVALID, "ug4gb_vector_dot_noalloc: pointers must be 8-byte aligned");
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return fail(err, err_capacity, UG4GB_ERR_CUDA, "ug4gb_vector_dot_noalloc: cudaGetDevice: %s",
                    cudaGetErrorString(e));
    if (!on_device(result, dev) || (n > 0 && (!on_device(a, dev) || !on_device(b, dev))))
        return fail(err, err_capacity, UG4GB_ERR_INVALID,
                    "ug4gb_vector_dot_noalloc: a, b and result must be device memory of the current device %d", dev);
    cudaStream_t st = (cudaStream_t)stream;
    DotScratch *s = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        unsigned long long id = current_context_id();
        for (int i = 0; i < g_num_scratch && id; ++i)
            if (g_scratch[i].ctx_id == id) s = g_scratch[i].p;
        if (!s) {
            void *p = nullptr;
            e = cudaGetSymbolAddress(&p, g_dot_scratch);
            if (e != cudaSuccess)
                return fail(err, err_capacity, UG4GB_ERR_CUDA, "ug4gb_vector_dot_noalloc: cudaGetSymbolAddress: %s",
                            cudaGetErrorString(e));
            s = (DotScratch *)p;
            // the look-up made the device's primary context current if no
            // context was; a context without an id is looked up every call
            if (!id) id = current_context_id();
            if (id && g_num_scratch < kMaxContexts) g_scratch[g_num_scratch++] = ScratchEntry{id, s};
        }
    }
    if (n == 0) {
        e = cudaMemsetAsync(result, 0, sizeof(double), st);
        if (e != cudaSuccess)
            return fail(err, err_capacity, UG4GB_ERR_CUDA, "ug4gb_vector_dot_noalloc: %s", cudaGetErrorString(e));
        return UG4GB_OK;
    }
    e = cudaMemsetAsync(&s->counter, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess)
        return fail(err, err_capacity, UG4GB_ERR_CUDA, "ug4gb_vector_dot_noalloc: clearing the counter: %s",
                    cudaGetErrorString(e));
    const unsigned int blocks = (unsigned int)((n + kChunk - 1) / kChunk);
    void *args[] = {(void *)&a, (void *)&b, (void *)&n, (void *)&result, (void *)&s};
    e = cudaLaunchKernel((const void *)k_dot_static, dim3(blocks), dim3(kThreads), args, 0, st);
    if (e != cudaSuccess)
        return fail(err, err_capacity, UG4GB_ERR_CUDA, "ug4gb_vector_dot_noalloc: launch: %s", cudaGetErrorString(e));
    return UG4GB_OK;
}

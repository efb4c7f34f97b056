// Checks the integer-arithmetic FP32<->FP64 conversions of the library
// (common.cuh: f32_to_f64, f64_to_f32) against the hardware conversions,
// bit for bit, on random and on edge-case inputs (ties, range ends, zeros,
// subnormals, infinities, NaN).  Prints "mismatches <count> checked <n>".
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../ugcore_gb300/csrc/common.cuh"

using namespace ug4gb;

__global__ void k_check(const unsigned long long *in64, const unsigned int *in32, int n, unsigned long long *bad)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = __longlong_as_double((long long)in64[i]);
    const float a = f64_to_f32(d), b = (float)d;
    // NaN payloads are not compared, only NaN-ness
    const bool nan_ok = (a != a) && (b != b);
    if (!nan_ok && __float_as_uint(a) != __float_as_uint(b)) atomicAdd(bad, 1ULL);
    const float f = __uint_as_float(in32[i]);
    const double c = f32_to_f64(f), e = (double)f;
    const bool nan_ok2 = (c != c) && (e != e);
    if (!nan_ok2 && __double_as_longlong(c) != __double_as_longlong(e)) atomicAdd(bad, 1ULL);
}

static unsigned long long rng(unsigned long long &s)
{
    s += 0x9E3779B97F4A7C15ULL;
    unsigned long long z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

int main()
{
    const int n = 1 << 24;
    std::vector<unsigned long long> h64(n);
    std::vector<unsigned int> h32(n);
    unsigned long long s = 12345;
    for (int i = 0; i < n; ++i) {
        unsigned long long r = rng(s);
        int kind = i % 8;
        if (kind < 3) {
            h64[i] = r;   // any bit pattern
        } else if (kind < 6) {
            // doubles in and around the FP32 range, many exactly halfway
            unsigned long long e = 1023 - 140 + (r % 280);
            unsigned long long m = rng(s) & 0xfffffffffffffULL;
            if (kind == 4) m = (m & ~((1ULL << 29) - 1)) | (1ULL << 28);   // tie
            if (kind == 5) m = (m | ((1ULL << 29) - 1));                    // just below carry
            h64[i] = (r & (1ULL << 63)) | (e << 52) | m;
        } else {
            double v = (double)(r % 2000001) - 1000000.0;
            v *= 1e-7;
            memcpy(&h64[i], &v, 8);
        }
        h32[i] = (unsigned int)rng(s);
    }
    const unsigned long long edges64[] = {0ULL, 1ULL << 63, 0x7ff0000000000000ULL, 0xfff0000000000000ULL,
                                          0x7ff8000000000000ULL, 0x47efffffe0000000ULL, 0x47efffff10000000ULL,
                                          0x3810000000000000ULL, 0x380fffffffffffffULL, 0x3800000000000000ULL, 1ULL};
    const unsigned int edges32[] = {0u, 0x80000000u, 0x7f800000u, 0xff800000u, 0x7fc00000u, 1u, 0x007fffffu,
                                    0x00800000u, 0x7f7fffffu};
    for (size_t k = 0; k < sizeof(edges64) / 8; ++k) h64[k] = edges64[k];
    for (size_t k = 0; k < sizeof(edges32) / 4; ++k) h32[k] = edges32[k];
    unsigned long long *d64, *bad;
    unsigned int *d32;
    if (cudaMalloc(&d64, 8ull * n) || cudaMalloc(&d32, 4ull * n) || cudaMalloc(&bad, 8)) return 2;
    cudaMemcpy(d64, h64.data(), 8ull * n, cudaMemcpyHostToDevice);
    cudaMemcpy(d32, h32.data(), 4ull * n, cudaMemcpyHostToDevice);
    cudaMemset(bad, 0, 8);
    k_check<<<(n + 255) / 256, 256>>>(d64, d32, n, bad);
    unsigned long long hb = 0;
    if (cudaMemcpy(&hb, bad, 8, cudaMemcpyDeviceToHost) != cudaSuccess) return 3;
    printf("mismatches %llu checked %d\n", hb, 2 * n);
    return hb == 0 ? 0 : 1;
}

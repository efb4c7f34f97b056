// guard.cu -- guard zones around device buffers in the guarded (debug) build.
//
// Built with -DUG4GB_GUARDED, every DevBuf allocation is 4 KB larger on both
// sides; the zones and the buffer itself are set to 0xFF bytes (NaN in every
// floating-point type, -1 in the integer types).  A kernel that writes past
// either end of a buffer changes a zone: the zones of a buffer are compared
// when it is freed and, for all live buffers, by ug4gb_debug_guard_check.
// A kernel that reads memory nobody wrote gets NaN (or -1), which the parity
// tests run against such a build then see in their results.  This stands in
// for a device bounds checker; the normal build carries none of it.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "common.cuh"

#ifdef UG4GB_GUARDED

namespace ug4gb {
namespace {

struct Guarded {
    char *base;
    size_t bytes;   // user bytes between the zones
};

struct Registry {
    std::mutex mu;
    std::unordered_map<void *, Guarded> live;
    std::vector<std::string> damaged;
};

Registry &registry()
{
    static Registry *r = new Registry;   // outlives every static DevBuf
    return *r;
}

// the zones of one buffer as 0xFF bytes?  Appends a line per damaged zone.
void check_zones(const Guarded &g, std::vector<std::string> &out)
{
    std::vector<unsigned char> h(kGuardBytes);
    const char *zone[2] = {g.base, g.base + kGuardBytes + g.bytes};
    for (int side = 0; side < 2; ++side) {
        if (cudaMemcpy(h.data(), zone[side], kGuardBytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
            cudaGetLastError();
            return;   // context gone (process exit): nothing to check
        }
        size_t first = kGuardBytes, count = 0;
        for (size_t i = 0; i < kGuardBytes; ++i)
            if (h[i] != 0xFF) {
                if (first == kGuardBytes) first = i;
                ++count;
            }
        if (count) {
            // offset of the first changed byte relative to the buffer start
            const long long off = side == 0 ? (long long)first - (long long)kGuardBytes
                                            : (long long)g.bytes + (long long)first;
            out.push_back("buffer of " + std::to_string(g.bytes) + " bytes: " + std::to_string(count) +
                          " bytes changed " + (side == 0 ? "before" : "after") + " it, first at offset " +
                          std::to_string(off));
        }
    }
}

}  // namespace

void guard_register(char *base, void *user, size_t user_bytes)
{
    // on the legacy stream, finished before any stream of the library uses it
    UG_CUDA(cudaMemset(base, 0xFF, user_bytes + 2 * kGuardBytes));
    UG_CUDA(cudaDeviceSynchronize());
    Registry &r = registry();
    std::lock_guard<std::mutex> lk(r.mu);
    r.live[user] = Guarded{base, user_bytes};
}

char *guard_release(void *user) noexcept
{
    Registry &r = registry();
    Guarded g{nullptr, 0};
    {
        std::lock_guard<std::mutex> lk(r.mu);
        auto it = r.live.find(user);
        if (it == r.live.end()) return static_cast<char *>(user);
        g = it->second;
        r.live.erase(it);
    }
    try {
        // kernels still running on the buffer finish first
        if (cudaDeviceSynchronize() == cudaSuccess) {
            std::vector<std::string> found;
            check_zones(g, found);
            std::lock_guard<std::mutex> lk(r.mu);
            for (auto &s : found) r.damaged.push_back(s);
        } else {
            cudaGetLastError();
        }
    } catch (...) {
    }
    return g.base;
}

}  // namespace ug4gb

extern "C" int ug4gb_debug_guard_check(char *buf, int capacity)
{
    using namespace ug4gb;
    Registry &r = registry();
    if (cudaDeviceSynchronize() != cudaSuccess) {
        cudaGetLastError();
        return UG4GB_ERR_CUDA;
    }
    std::vector<Guarded> all;
    {
        std::lock_guard<std::mutex> lk(r.mu);
        for (auto &kv : r.live) all.push_back(kv.second);
    }
    std::vector<std::string> found;
    for (const Guarded &g : all) check_zones(g, found);
    std::string text;
    int n = 0;
    {
        std::lock_guard<std::mutex> lk(r.mu);
        for (auto &s : r.damaged) text += s + "\n";
        n = (int)r.damaged.size();
    }
    for (auto &s : found) text += s + "\n";
    n += (int)found.size();
    if (buf && capacity > 0) {
        const size_t k = std::min(text.size(), (size_t)capacity - 1);
        std::memcpy(buf, text.data(), k);
        buf[k] = '\0';
    }
    return n;
}

#else

extern "C" int ug4gb_debug_guard_check(char *buf, int capacity)
{
    if (buf && capacity > 0) buf[0] = '\0';
    return UG4GB_ERR_STATE;
}

#endif

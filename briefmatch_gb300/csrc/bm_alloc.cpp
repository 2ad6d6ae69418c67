// bm_alloc.cpp -- the engine's device allocator and its test hooks.
//
// Every device allocation of the contexts, batches and proposal networks goes
// through device_malloc / device_free.  Two host-only test hooks sit on that path,
// both off unless a test turns them on:
//  - bm_debug_fail_alloc(k): the k-th allocation from then on fails as if the device
//    were out of memory (the path a real cudaMalloc failure takes);
//  - bm_debug_guard_bands(on): allocations made while it is on carry 256-byte guard
//    bands before and after the buffer, filled with a known byte; bm_debug_check_guards
//    reads every live band back and reports the first one a kernel overwrote.
// The reference's counterpart is HANDLE_ERROR -> CudaException around every
// CUDA_constructor (util_cuda.h:102-112, util_cuda.cu:206-210); it has no hooks.
#include <atomic>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "bm_internal.h"

namespace {

constexpr size_t kGuard = 256;            // bytes before and after a guarded buffer
constexpr unsigned char kGuardByte = 0xA5;

std::atomic<uint64_t> g_allocs{0};
std::atomic<int64_t> g_live{0};           // allocations made and not yet freed
std::atomic<uint64_t> g_fail_at{0};       // absolute allocation number that fails, 0 = none
std::atomic<int> g_guard_on{0};
std::mutex g_mu;
std::map<void*, size_t> g_guarded;        // user pointer -> user bytes

}  // namespace

namespace bmk {

cudaError_t device_malloc(void** p, size_t bytes)
{
    *p = nullptr;
    const uint64_t k = ++g_allocs;
    const uint64_t fail = g_fail_at.load();
    if (fail && k == fail) return cudaErrorMemoryAllocation;
    if (!g_guard_on.load()) {
        const cudaError_t e = cudaMalloc(p, bytes);
        if (e == cudaSuccess) ++g_live;
        else *p = nullptr;
        return e;
    }
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, bytes + 2 * kGuard);
    if (e != cudaSuccess) return e;
    // the bands and the buffer itself start as the guard byte (so a read of memory no
    // kernel wrote shows up as a changed result); finished before any stream uses it
    e = cudaMemset(base, kGuardByte, bytes + 2 * kGuard);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        cudaFree(base);
        return e;
    }
    *p = static_cast<unsigned char*>(base) + kGuard;
    ++g_live;
    std::lock_guard<std::mutex> lock(g_mu);
    g_guarded[*p] = bytes;
    return cudaSuccess;
}

void device_free(void* p)
{
    if (!p) return;
    --g_live;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        auto it = g_guarded.find(p);
        if (it != g_guarded.end()) {
            g_guarded.erase(it);
            cudaFree(static_cast<unsigned char*>(p) - kGuard);
            return;
        }
    }
    cudaFree(p);
}

}  // namespace bmk

extern "C" {

void bm_debug_fail_alloc(uint64_t k) { g_fail_at = k ? g_allocs.load() + k : 0; }

uint64_t bm_debug_alloc_count(void) { return g_allocs.load(); }

int64_t bm_debug_live_allocs(void) { return g_live.load(); }

void bm_debug_guard_bands(int on) { g_guard_on = on ? 1 : 0; }

bm_status bm_debug_check_guards(uint64_t* checked)
{
    std::vector<std::pair<void*, size_t>> live;
    {
        std::lock_guard<std::mutex> lock(g_mu);
        live.assign(g_guarded.begin(), g_guarded.end());
    }
    if (checked) *checked = live.size();
    if (cudaDeviceSynchronize() != cudaSuccess) {
        bmk::set_error_text("bm_debug_check_guards: device error before the check");
        return BM_ERR_CUDA;
    }
    std::vector<unsigned char> band(kGuard);
    for (const auto& kv : live) {
        const unsigned char* user = static_cast<const unsigned char*>(kv.first);
        const unsigned char* where[2] = {user - kGuard, user + kv.second};
        for (int side = 0; side < 2; side++) {
            if (cudaMemcpy(band.data(), where[side], kGuard, cudaMemcpyDeviceToHost) != cudaSuccess) {
                bmk::set_error_text("bm_debug_check_guards: copy failed");
                return BM_ERR_CUDA;
            }
            for (size_t i = 0; i < kGuard; i++)
                if (band[i] != kGuardByte) {
                    char buf[200];
                    std::snprintf(buf, sizeof(buf),
                                  "guard band %s a %zu-byte buffer overwritten at byte %zu (0x%02x)",
                                  side ? "after" : "before", kv.second, i, band[i]);
                    bmk::set_error_text(buf);
                    return BM_ERR_STATE;
                }
        }
    }
    return BM_OK;
}

}  // extern "C"

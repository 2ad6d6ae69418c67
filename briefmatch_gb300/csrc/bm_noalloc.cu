// bm_noalloc.cu -- flow refinement for callers that must not allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc once they are running: video
// and capture pipelines that allocate everything at start-up and treat any later
// allocation as a fault, plugin hosts that own the device memory budget and hand
// the plugin only the frames it works on, and real-time threads that must not take
// the implicit device synchronisation a cudaMalloc/cudaFree can cause.
// bm_refine_noalloc gives them the refinement stage (the median filter and the
// cross-trilateral filter of BriefMatch::process) on buffers they own.  Its
// intermediate planes live in the fixed array below, which is part of the loaded
// module: every GPU that loads this library holds it until the process exits.
#include <cmath>
#include <cstdio>
#include <mutex>

#include "bm_internal.h"

// Largest input frame the entry point accepts: 2,097,152 pixels (1920x1080 fits).
#define BM_NOALLOC_MAX_PIXELS (2u * 1024u * 1024u)

// Four planes of BM_NOALLOC_MAX_PIXELS floats (32 MiB): the horizontal median of u
// and v, then the full median of u and v.
static __device__ __align__(256) float g_refine_scratch[4 * (size_t)BM_NOALLOC_MAX_PIXELS];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_mu;
float* g_scratch_ptr[kMaxDevices] = {};
bm_status noalloc_fail(bm_status st, const char* msg)
{
    bmk::set_error_text(msg);
    return st;
}

// Device address of the scratch array on the current device.  Host code only
// knows the array's host-side stand-in, so the address is looked up once per
// device (with that device current) and cached.
bm_status scratch_on_current_device(float** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return noalloc_fail(BM_ERR_CUDA, "bm_refine_noalloc: no current CUDA device");
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_refine_scratch);
        if (e != cudaSuccess || !p) {
            char buf[256];
            std::snprintf(buf, sizeof(buf), "bm_refine_noalloc: scratch address lookup failed: %s",
                          cudaGetErrorString(e));
            return noalloc_fail(BM_ERR_CUDA, buf);
        }
        g_scratch_ptr[dev] = static_cast<float*>(p);
    }
    *out = g_scratch_ptr[dev];
    return BM_OK;
}

}  // namespace

extern "C" {

uint64_t bm_refine_noalloc_max_pixels(void) { return BM_NOALLOC_MAX_PIXELS; }

bm_status bm_refine_noalloc(const float* d_u, const float* d_v, const float* d_guide, float* d_uo, float* d_vo,
                            uint32_t width, uint32_t height, uint32_t fsize, float sEPE, float sI, float sS,
                            void* stream)
{
    if (!d_u || !d_v || !d_guide || !d_uo || !d_vo)
        return noalloc_fail(BM_ERR_INVALID, "bm_refine_noalloc: null buffer");
    if (width == 0 || height == 0) return noalloc_fail(BM_ERR_INVALID, "bm_refine_noalloc: zero size");
    const uint64_t n = (uint64_t)width * height;
    if (n > BM_NOALLOC_MAX_PIXELS) {
        char buf[256];
        std::snprintf(buf, sizeof(buf),
                      "bm_refine_noalloc: %ux%u is %llu pixels, more than its fixed scratch holds (%u pixels); "
                      "use bm_process on a context instead",
                      width, height, (unsigned long long)n, BM_NOALLOC_MAX_PIXELS);
        return noalloc_fail(BM_ERR_LIMIT, buf);
    }
    if (fsize > BM_MAX_MEDIAN) return noalloc_fail(BM_ERR_LIMIT, "bm_refine_noalloc: median size above 47");
    if (!(sEPE > 0) || !(sI > 0) || !(sS > 0))
        return noalloc_fail(BM_ERR_INVALID, "bm_refine_noalloc: filter sigmas must be positive");
    float* scratch = nullptr;
    bm_status st = scratch_on_current_device(&scratch);
    if (st != BM_OK) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    float* hU = scratch;
    float* hV = scratch + n;
    float* mU = scratch + 2 * n;
    float* mV = scratch + 3 * n;
    const int fs = fsize == 0 ? 1 : (int)fsize;
    const int w = (int)width, h = (int)height;
    // Every scratch element is written before it is read, so nothing is cleared.
    cudaError_t e = bmk::median_pass(d_u, d_v, hU, hV, 1, fs, w, h, s);
    if (e == cudaSuccess) e = bmk::median_pass(hU, hV, mU, mV, 0, fs, w, h, s);
    const int tri_s = (int)std::ceil(2.5 * (double)std::sqrt(sS * sS));
    if (e == cudaSuccess)
        e = bmk::trilateral(d_u, d_v, mU, mV, d_guide, d_uo, d_vo, w, h, tri_s, sEPE * sEPE, sI * sI, sS * sS, s);
    if (e != cudaSuccess) {
        char buf[256];
        std::snprintf(buf, sizeof(buf), "bm_refine_noalloc: launch failed: %s", cudaGetErrorString(e));
        return noalloc_fail(BM_ERR_CUDA, buf);
    }
    return BM_OK;
}

}  // extern "C"

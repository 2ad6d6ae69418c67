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
#include <cuda.h>  // CUcontext / CUresult types only; the driver entry points are fetched at run time
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
// Per device: the scratch array's device address and the id of the CUDA context it
// was looked up in.  cudaDeviceReset destroys the context and the module with it; the
// next context has another id, so the address is looked up again there.
struct ScratchSlot {
    float* ptr;
    unsigned long long ctx_id;
};
ScratchSlot g_slot[kMaxDevices] = {};

bm_status noalloc_fail(bm_status st, const char* msg)
{
    bmk::set_error_text(msg);
    return st;
}

// Unique id of the calling thread's current CUDA context (0 when none is current or
// the driver does not offer the query).  The two driver calls are fetched through the
// runtime, so the library does not link the driver library itself.
unsigned long long current_context_id()
{
    typedef CUresult (*GetCurrent)(CUcontext*);
    typedef CUresult (*GetId)(CUcontext, unsigned long long*);
    static GetCurrent get_current = nullptr;
    static GetId get_id = nullptr;
    static bool looked_up = false;
    if (!looked_up) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess) {
            get_current = reinterpret_cast<GetCurrent>(f1);
            get_id = reinterpret_cast<GetId>(f2);
        }
        looked_up = true;
    }
    if (!get_current || !get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array in the current device's context.  Host code
// only knows the array's host-side stand-in, so the address is looked up with that
// device current and kept for as long as the same context is current.
bm_status scratch_on_current_device(float** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return noalloc_fail(BM_ERR_CUDA, "bm_refine_noalloc: no current CUDA device");
    std::lock_guard<std::mutex> lock(g_mu);
    const unsigned long long id = current_context_id();
    if (!g_slot[dev].ptr || id == 0 || g_slot[dev].ctx_id != id) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_refine_scratch);
        if (e != cudaSuccess || !p) {
            char buf[256];
            std::snprintf(buf, sizeof(buf), "bm_refine_noalloc: scratch address lookup failed: %s",
                          cudaGetErrorString(e));
            return noalloc_fail(BM_ERR_CUDA, buf);
        }
        g_slot[dev].ptr = static_cast<float*>(p);
        g_slot[dev].ctx_id = current_context_id();  // the lookup makes the primary context current
    }
    *out = g_slot[dev].ptr;
    return BM_OK;
}

// True when the byte ranges [a, a + na) and [b, b + nb) overlap.
bool overlaps(const void* a, size_t na, const void* b, size_t nb)
{
    const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    return x < y + nb && y < x + na;
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
    const int tri_s = bmk::trilateral_half_window(sEPE, sI, sS, width, height);
    if (tri_s == -1) return noalloc_fail(BM_ERR_INVALID, "bm_refine_noalloc: filter sigmas must be finite and positive");
    if (tri_s == -2)
        return noalloc_fail(BM_ERR_LIMIT, "bm_refine_noalloc: trilateral window wider than twice the frame");
    // the filter reads neighbouring input samples while other threads write outputs
    const size_t plane = (size_t)n * sizeof(float);
    const void* ins[3] = {d_u, d_v, d_guide};
    for (const void* in : ins)
        if (overlaps(d_uo, plane, in, plane) || overlaps(d_vo, plane, in, plane))
            return noalloc_fail(BM_ERR_INVALID, "bm_refine_noalloc: an output plane overlaps an input plane");
    if (overlaps(d_uo, plane, d_vo, plane))
        return noalloc_fail(BM_ERR_INVALID, "bm_refine_noalloc: the two output planes overlap");
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

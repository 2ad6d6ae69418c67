// bm_internal.h -- engine-private declarations shared by the kernel and API units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "briefmatch_gb300.h"

namespace bmk {

// Sets the text bm_last_error() returns on this thread.
void set_error_text(const char* msg);

// The engine's device allocator (bm_alloc.cpp): cudaMalloc/cudaFree behind the test
// hooks bm_debug_fail_alloc and bm_debug_guard_bands.
cudaError_t device_malloc(void** p, size_t bytes);
void device_free(void* p);

// Random-search stream position for one launch (briefmatch_cuda.cu:237-241).
struct RsArgs {
    int enabled;                 // fuse a random-search candidate into the launch
    int mode;                    // BM_RNG_XORWOW or BM_RNG_PHILOX
    unsigned long long seed;     // Philox key
    unsigned long long call;     // index of this random-search call in the stream
    float dist;                  // search radius, briefmatch.cpp:271
};

// Flow words: low 16 bits nx, high 16 bits ny, both int16.
__host__ __device__ inline uint32_t pack_flow(int nx, int ny)
{
    return (uint32_t)(uint16_t)(int16_t)nx | ((uint32_t)(uint16_t)(int16_t)ny << 16);
}

// Words per descriptor in the engine layout: ceil(N/32) rounded up to 1, 2, 4, 8 or 16.
inline uint32_t feature_stride(uint32_t N)
{
    uint32_t ns = (N + 31) / 32;
    uint32_t s = 1;
    while (s < ns) s <<= 1;
    return s;
}

cudaError_t lanczos_tables(float* w, int* idx, int n_in, int n_out, cudaStream_t st);
cudaError_t upsample_f32(const float* in, float* out, int sxi, int syi, int sxo, int syo,
                         const float* lx, const int* ix, const float* ly, const int* iy, cudaStream_t st);
cudaError_t upsample_u8(const uint8_t* in, float* out, int sxi, int syi, int sxo, int syo,
                        const float* lx, const int* ix, const float* ly, const int* iy, cudaStream_t st);
// Up-sampling into an image with an edge-replicated margin of m pixels on every
// side; `out` is the start of the (sxo + 2m) x (syo + 2m) buffer, row pitch `pitch`.
cudaError_t upsample_u8_pad(const uint8_t* in, float* out, int pitch, int m, int sxi, int syi, int sxo, int syo,
                            const float* lx, const int* ix, const float* ly, const int* iy, cudaStream_t st);
cudaError_t u8_to_f32(const uint8_t* in, float* out, size_t n, cudaStream_t st);

// Linear image offsets (o1, o2) of every BRIEF sample for one image width, padded
// with zeros to a whole number of 32-bit words; passed by value as a kernel
// parameter (4 KB) so that the sample loop reads them as constants.
struct PatternOffsets {
    int2 off[BM_PATCH_MAX / 4];
};

cudaError_t features(const float* up, uint32_t* F, int sx, int sy, int N, int nsp,
                     const int4* pat, int rmax, const PatternOffsets& po, int rev, cudaStream_t st);

// Descriptors from an edge-replicated image: `up` points at pixel (0, 0), row pitch
// `pitch`, with a margin no narrower than the largest pattern offset; `po` holds the
// offsets for that pitch.
cudaError_t features_pad(const float* up, int pitch, uint32_t* F, int sx, int sy, int nsp,
                         const PatternOffsets& po, int rev, cudaStream_t st);

cudaError_t initialize(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_prev,
                       uint32_t* flow_out, uint16_t* cost, int sx, int sy, int nsp, int first, int rev,
                       cudaStream_t st);

cudaError_t seed_field(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_prev, uint32_t* flow_out,
                       uint16_t* cost, int sx, int sy, int nsp, int first, const float* pred, int w4, int h4,
                       float scale_x, float scale_y, float logit_min, cudaStream_t st);

cudaError_t local_step(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_in, uint32_t* flow_out,
                       uint16_t* cost, int sx, int sy, int nsp, int r, int rev, cudaStream_t st);

cudaError_t jump_level(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_in,
                       uint32_t* flow_out, uint16_t* cost, int sx, int sy, int nsp,
                       int p, int pd, int doubleProp, const RsArgs& rs, int rev, cudaStream_t st);

cudaError_t random_search(const uint32_t* F1, const uint32_t* F2, uint32_t* flow, uint16_t* cost,
                          int sx, int sy, int nsp, const RsArgs& rs, cudaStream_t st);

cudaError_t normals(float2* out, int sx, int sy, const RsArgs& rs, cudaStream_t st);

cudaError_t nn_table(unsigned int* idx, int n_up, int n_in, cudaStream_t st);
cudaError_t downsample(const uint32_t* flow, float* U, float* V, int sx, int sy, int sx_in, int sy_in,
                       const float* taps, int P, float mx, float my, const unsigned int* nnx,
                       const unsigned int* nny, cudaStream_t st);

cudaError_t flow_to_planes(const uint32_t* flow, float* U, float* V, size_t n, cudaStream_t st);

cudaError_t median_pass(const float* inU, const float* inV, float* outU, float* outV,
                        int dir, int fsize, int sx, int sy, cudaStream_t st);

// Half window of the cross-trilateral filter, s = ceil(2.5*sqrt(sS^2))
// (briefmatch_cuda.cu:266), for an input frame of w x h pixels.  Returns -1 when a
// sigma is not a finite positive number, -2 when s would exceed the frame's larger
// side (such a window adds only clamped edge samples, and its cost grows as s^2).
inline int trilateral_half_window(float sEPE, float sI, float sS, uint32_t w, uint32_t h)
{
    const float big = 3.0e38f;
    if (!(sEPE > 0 && sEPE < big) || !(sI > 0 && sI < big) || !(sS > 0 && sS < big)) return -1;
    const double s = __builtin_ceil(2.5 * (double)__builtin_sqrtf(sS * sS));
    const uint32_t side = w > h ? w : h;
    if (s > (double)side) return -2;
    return (int)s;
}

cudaError_t ensure_trilateral_smem(int s);
cudaError_t trilateral(const float* U, const float* V, const float* Um, const float* Vm,
                       const float* I, float* Uo, float* Vo, int sx, int sy, int s,
                       float sigmaEPE2, float sigmaI2, float sigmaS2, cudaStream_t st);

// Colour coding of a flow field (u, v planes of n floats) into n*3 bytes R G B
// (briefmatch.cpp:373-421, colorcode.cpp:52-74).  max_motion > 0 normalises by it;
// otherwise by the largest known vector length, measured into the device word
// d_word first.
cudaError_t flow_colors(const float* U, const float* V, size_t n, float max_motion, int* d_word, uint8_t* rgb,
                        cudaStream_t st);

cudaError_t export_field(const uint32_t* flow, const uint16_t* cost, int16_t* nx, int16_t* ny,
                         float* dist, size_t n, int N, cudaStream_t st);
cudaError_t import_field(const int16_t* nx, const int16_t* ny, const uint16_t* cost_in,
                         uint32_t* flow, uint16_t* cost, size_t n, cudaStream_t st);

}  // namespace bmk

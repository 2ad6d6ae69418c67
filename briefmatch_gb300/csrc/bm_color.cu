// bm_color.cu -- colour coding of flow fields on the GPU (BriefMatch::computeColors,
// briefmatch.cpp:373-421, with the Middlebury colour wheel of util/colorcode.cpp:52-74).
//
// This unit is compiled WITHOUT -use_fast_math and spells every rounding step out
// (__fmul_rn, __dadd_rn, ...), so that no multiply-add is contracted: the reference
// evaluates this code on the host in float and double arithmetic without fused
// operations, and the output bytes follow from that arithmetic.  The one deliberate
// definition: the reference's float atan2 is whatever the host math library returns
// (glibc 2.39's atan2f is one unit in the last place off the correctly rounded value
// on about 15 % of inputs); here, as in the oracle, it is the correctly rounded float
// of atan2 (a double evaluation rounded once).
#include <stdint.h>

#include <algorithm>

#include "bm_internal.h"

namespace bmk {
namespace {

// The colour wheel, colorcode.cpp:27-50: integer channel values from integer
// divisions, 15 + 6 + 4 + 11 + 13 + 6 = 55 entries (r, g, b), kept as the floats
// computeColor forms from them (value / 255.0, rounded once).
struct Wheel {
    float f[55][3];  // colorwheel[k][b] / 255.0 rounded to float (colorcode.cpp:64-65)
};

Wheel make_wheel()
{
    const int RY = 15, YG = 6, GC = 4, CB = 11, BM = 13, MR = 6;
    Wheel w;
    int k = 0;
    auto set = [&](int r, int g, int b) {
        w.f[k][0] = (float)(r / 255.0);
        w.f[k][1] = (float)(g / 255.0);
        w.f[k][2] = (float)(b / 255.0);
        k++;
    };
    for (int i = 0; i < RY; i++) set(255, 255 * i / RY, 0);
    for (int i = 0; i < YG; i++) set(255 - 255 * i / YG, 255, 0);
    for (int i = 0; i < GC; i++) set(0, 255, 255 * i / GC);
    for (int i = 0; i < CB; i++) set(0, 255 - 255 * i / CB, 255);
    for (int i = 0; i < BM; i++) set(255 * i / BM, 0, 255);
    for (int i = 0; i < MR; i++) set(255, 0, 255 - 255 * i / MR);
    return w;
}

__device__ __forceinline__ bool unknown_flow(float u, float v)
{
    // flowIO.cpp:35-39 (UNKNOWN_FLOW_THRESH 1e9, flowIO.h:5)
    return fabsf(u) > 1e9f || fabsf(v) > 1e9f || u != u || v != v;
}

__device__ __forceinline__ float radius(float u, float v) { return __fsqrt_rn(__fadd_rn(__fmul_rn(u, u), __fmul_rn(v, v))); }

// Largest vector length over the known vectors, as the bits of a non-negative float
// in an int (ordered like the floats); the word starts at -1 (no known vector).
__global__ void __launch_bounds__(256) k_max_radius(const float* __restrict__ U, const float* __restrict__ V, size_t n,
                                                    int* __restrict__ out)
{
    int best = -1;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const float u = __ldg(U + i), v = __ldg(V + i);
        if (!unknown_flow(u, v)) best = max(best, __float_as_int(radius(u, v)));
    }
    for (int o = 16; o > 0; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
    __shared__ int warp_best[8];
    if ((threadIdx.x & 31) == 0) warp_best[threadIdx.x >> 5] = best;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); w++) best = max(best, warp_best[w]);
        if (best >= 0) atomicMax(out, best);
    }
}

// computeColor (colorcode.cpp:52-74) of (u/maxrad, v/maxrad) per pixel, R G B bytes.
// maxrad comes from `fixed` when the pointer `measured` is null, else from the
// measured word (briefmatch.cpp:400-406: a measured 0 becomes 1, no known vector
// leaves -1).
__global__ void __launch_bounds__(256) k_flow_color(const float* __restrict__ U, const float* __restrict__ V, size_t n,
                                                    float fixed, const int* __restrict__ measured, Wheel wheel,
                                                    uint8_t* __restrict__ rgb)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float maxrad = fixed;
    if (measured) {
        const int m = *measured;
        maxrad = m < 0 ? -1.0f : __int_as_float(m);
        if (maxrad == 0.0f) maxrad = 1.0f;
    }
    const float u = U[i], v = V[i];
    uint8_t* pix = rgb + 3 * i;
    if (unknown_flow(u, v)) {
        pix[0] = pix[1] = pix[2] = 0;
        return;
    }
    // colorcode.cpp:57-72 with the declared types: rad, a, fk, f, col0, col1 and col are
    // float; the constants 1.0, 2.0, M_PI, .75 and 255.0 make their expressions double
    const float fx = __fdiv_rn(u, maxrad), fy = __fdiv_rn(v, maxrad);
    const float rad = radius(fx, fy);
    const float at = __double2float_rn(atan2(-(double)fy, -(double)fx));  // correctly rounded float atan2
    const float a = __double2float_rn(__ddiv_rn((double)at, 3.14159265358979323846));
    const int ncols = 55;
    // (a + 1.0) / 2.0 * (ncols - 1); halving is exact, so it is a multiply by 0.5
    const float fk = __double2float_rn(__dmul_rn(__dmul_rn(__dadd_rn((double)a, 1.0), 0.5), (double)(ncols - 1)));
    const int k0 = (int)fk;
    const int k1 = (k0 + 1) % ncols;
    const float f = __fsub_rn(fk, (float)k0);
    const float omf = __fsub_rn(1.0f, f);
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const float col0 = wheel.f[k0][b], col1 = wheel.f[k1][b];
        float col = __fadd_rn(__fmul_rn(omf, col0), __fmul_rn(f, col1));
        if (rad <= 1.0f)
            col = __fsub_rn(1.0f, __fmul_rn(rad, __fsub_rn(1.0f, col)));  // saturation grows with radius
        else
            col = __double2float_rn(__dmul_rn((double)col, 0.75));  // out of range
        // the reference stores BGR (pix[2 - b]) and its PNG writer swaps to RGB: byte b here
        pix[b] = (uint8_t)__double2int_rz(__dmul_rn(255.0, (double)col));
    }
}

}  // namespace

cudaError_t flow_colors(const float* U, const float* V, size_t n, float max_motion, int* d_word, uint8_t* rgb,
                        cudaStream_t st)
{
    static const Wheel wheel = make_wheel();
    if (n == 0) return cudaSuccess;
    const int* measured = nullptr;
    if (!(max_motion > 0)) {
        cudaError_t e = cudaMemsetAsync(d_word, 0xff, sizeof(int), st);  // -1
        if (e != cudaSuccess) return e;
        const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 4 * 152);
        k_max_radius<<<blocks, 256, 0, st>>>(U, V, n, d_word);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        measured = d_word;
    }
    k_flow_color<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(U, V, n, max_motion, measured, wheel, rgb);
    return cudaGetLastError();
}

}  // namespace bmk

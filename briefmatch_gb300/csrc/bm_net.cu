// bm_net.cu -- the learned flow proposal: a 6-layer 3x3 convolutional network at
// quarter resolution that predicts an initial flow and a confidence for PatchMatch.
//
//   layer 0: 32 -> 32 channels, ReLU      (input: both frames at quarter resolution,
//                                          each 4x4 block of pixels as 16 channels)
//   layers 1-4: 32 -> 32 channels, ReLU   (dilations 2, 4, 8, 1)
//   layer 5: 32 -> 3 channels, linear     (u/4, v/4 in quarter-resolution pixels, confidence logit)
//
// Every layer is a 3x3 convolution; the dilated middle layers widen the receptive
// field to 63 cells (252 pixels) at the same cost per layer.
//
// Weights and activations are BF16, accumulation FP32, on the tensor cores.  The
// forward pass of every layer and the backward-data pass of the 32-channel layers run
// on the fifth-generation tensor cores (k_conv_umma): per CTA 128 cells of one image
// row are the GEMM's M, the nine taps' 32 input channels its K (two K=16 steps per
// tap), the output channels its N; TMA brings each tap's 128x32 activation tile and
// the weights into shared memory in the 64-byte-swizzled K-major layout the MMA
// reads, tcgen05.mma accumulates in tensor memory and tcgen05.ld hands each thread
// its cell's channels for the epilogue.  The mma.sync m16n8k16 kernels (k_conv) stay
// for the backward-data pass of the head (16 gradient channels), as the alternative
// forward path (bm_net_set_umma), and the weight gradients (k_conv_wgrad: pixels as
// the reduction dimension).  Activations are NHWC with the channel count padded to a
// multiple of 16 (32-byte rows).  Training keeps FP32 master weights and Adam
// moments; every step repacks the BF16 copies the kernels read.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda.h>  // CUtensorMap and its enums; the encoder is fetched through the runtime
#include <cuda_bf16.h>

#include "bm_internal.h"

namespace {

constexpr int NL = 6;                               // layers
constexpr int CIN_R[NL] = {32, 32, 32, 32, 32, 32};  // real input channels
constexpr int COUT_R[NL] = {32, 32, 32, 32, 32, 3};
constexpr int CIN_P[NL] = {32, 32, 32, 32, 32, 32};  // padded (multiple of 16)
constexpr int COUT_P[NL] = {32, 32, 32, 32, 32, 16};  // padded (multiple of 16: the head is N=16 on tcgen05)
constexpr int DIL[NL] = {1, 2, 4, 8, 1, 1};          // dilation of each layer's 3x3 taps
constexpr int NIN = 32;                              // input channels: 16 pixels of each frame's 4x4 block

constexpr int BW = 16, BH = 8;  // output tile per block: 8 rows x 16 columns, 4 warps

// Shared memory of the forward/backward-data tile (input tile with a DIL-wide halo
// plus all nine taps' weights) and of the weight-gradient tile.
constexpr size_t conv_smem(int cinp, int coutp, int dil)
{
    return ((size_t)(BH + 2 * dil) * (BW + 2 * dil) * (cinp + 8) + (size_t)9 * coutp * (cinp + 8)) * 2;
}
constexpr size_t wgrad_smem(int cinp, int coutd, int dil)
{
    return ((size_t)coutd * (BW * BH + 8) + (size_t)cinp * ((BH + 2 * dil) * (BW + 2 * dil) + 8)) * 2;
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

enum Epi { EPI_RELU_BF16 = 0, EPI_LINEAR_F32 = 1, EPI_MASK_BF16 = 2 };

// Y[p, co] = sum_{tap, ci} X[p + DIL * (tap - 1), ci] * W[tap][co][ci]  (+ bias, ReLU) --
// or, for the backward-data pass, the same product followed by the ReLU mask of
// `act`.  X: [B][h][w][CINP] bf16; W: [9][COUTP][CINP] bf16; out per EPI.  Dynamic
// shared memory: conv_smem(CINP, COUTP, DIL) bytes.
template <int CINP, int COUTP, int EPI, int DIL>
__global__ void __launch_bounds__(128) k_conv(const __nv_bfloat16* __restrict__ X, const __nv_bfloat16* __restrict__ W,
                                              const float* __restrict__ bias, const __nv_bfloat16* __restrict__ act,
                                              void* __restrict__ out, int h, int w, int cout_real, int out_stride)
{
    constexpr int SP = CINP + 8;  // smem pixel stride (bf16): conflict-free fragment loads
    constexpr int NT = COUTP / 8;
    constexpr int HW = BW + 2 * DIL, HH = BH + 2 * DIL;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* s_in = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    __nv_bfloat16* s_w = s_in + HH * HW * SP;
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * BW, y0 = blockIdx.y * BH, b = blockIdx.z;
    const __nv_bfloat16* Xb = X + (size_t)b * h * w * CINP;
    // stage the input tile with a DIL-pixel zero halo, 16 bytes at a time
    constexpr int VPP = CINP / 8;  // 16-byte vectors per pixel
    for (int k = tid; k < HH * HW * VPP; k += 128) {
        const int pix = k / VPP, v = k - pix * VPP;
        const int hy = pix / HW, hx = pix - hy * HW;
        const int gy = y0 + hy - DIL, gx = x0 + hx - DIL;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (gy >= 0 && gy < h && gx >= 0 && gx < w)
            val = *reinterpret_cast<const uint4*>(Xb + ((size_t)gy * w + gx) * CINP + v * 8);
        *reinterpret_cast<uint4*>(s_in + pix * SP + v * 8) = val;
    }
    for (int k = tid; k < 9 * COUTP * VPP; k += 128) {
        const int row = k / VPP, v = k - row * VPP;
        *reinterpret_cast<uint4*>(s_w + row * SP + v * 8) = *reinterpret_cast<const uint4*>(W + (size_t)row * CINP + v * 8);
    }
    __syncthreads();

    const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const uint32_t* si = reinterpret_cast<const uint32_t*>(s_in);
    const uint32_t* sw = reinterpret_cast<const uint32_t*>(s_w);
    float acc[2][NT][4];
#pragma unroll
    for (int mt = 0; mt < 2; mt++)
#pragma unroll
        for (int nt = 0; nt < NT; nt++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[mt][nt][q] = 0.0f;

#pragma unroll
    for (int tap = 0; tap < 9; tap++) {
        const int dy = tap / 3, dx = tap - dy * 3;
#pragma unroll
        for (int kc = 0; kc < CINP / 16; kc++) {
            uint32_t bf[NT][2];
#pragma unroll
            for (int nt = 0; nt < NT; nt++) {
                const int base = ((tap * COUTP + nt * 8 + g) * SP + kc * 16 + 2 * t) >> 1;
                bf[nt][0] = sw[base];
                bf[nt][1] = sw[base + 4];
            }
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
                const int r = warp * 2 + mt;  // output row within the tile
                const int p0 = ((r + dy * DIL) * HW + g + dx * DIL) * SP + kc * 16 + 2 * t;
                const int p8 = ((r + dy * DIL) * HW + g + 8 + dx * DIL) * SP + kc * 16 + 2 * t;
                uint32_t a[4];
                a[0] = si[p0 >> 1];
                a[1] = si[p8 >> 1];
                a[2] = si[(p0 >> 1) + 4];
                a[3] = si[(p8 >> 1) + 4];
#pragma unroll
                for (int nt = 0; nt < NT; nt++) mma_bf16(acc[mt][nt], a, bf[nt][0], bf[nt][1]);
            }
        }
    }
    // epilogue: C fragment (row g / g+8 = pixel column, cols 2t, 2t+1 = channels)
#pragma unroll
    for (int mt = 0; mt < 2; mt++) {
        const int y = y0 + warp * 2 + mt;
        if (y >= h) continue;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const int x = x0 + g + half * 8;
            if (x >= w) continue;
            const size_t pix = ((size_t)b * h + y) * w + x;
#pragma unroll
            for (int nt = 0; nt < NT; nt++) {
                const int co = nt * 8 + 2 * t;
                float v0 = acc[mt][nt][half * 2 + 0], v1 = acc[mt][nt][half * 2 + 1];
                if constexpr (EPI == EPI_RELU_BF16) {
                    v0 = fmaxf(v0 + bias[co], 0.0f);
                    v1 = fmaxf(v1 + bias[co + 1], 0.0f);
                    reinterpret_cast<uint32_t*>(out)[(pix * out_stride + co) >> 1] = pack_bf16(v0, v1);
                } else if constexpr (EPI == EPI_MASK_BF16) {
                    const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162*>(act + pix * out_stride + co);
                    v0 = __bfloat162float(m.x) > 0.0f ? v0 : 0.0f;
                    v1 = __bfloat162float(m.y) > 0.0f ? v1 : 0.0f;
                    reinterpret_cast<uint32_t*>(out)[(pix * out_stride + co) >> 1] = pack_bf16(v0, v1);
                } else {
                    float* o = reinterpret_cast<float*>(out) + pix * out_stride;
                    if (co < cout_real) o[co] = v0 + bias[co];
                    if (co + 1 < cout_real) o[co + 1] = v1 + bias[co + 1];
                }
            }
        }
    }
}

// dW[co][tap][ci] += sum_p dY[p, co] * X[p + DIL * (tap - 1), ci] and db[co] += sum_p
// dY[p, co] over one 8x16 tile: A = dY^T (16 output channels x 16 pixels of one tile
// row), B = the shifted input (16 pixels x 8 input channels).  Each warp owns taps
// w, w+4, w+8.  Partial sums of the tile are added to the FP32 gradients atomically.
// Dynamic shared memory: wgrad_smem(CINP, COUTD, DIL) bytes.
template <int CINP, int COUTD, int DIL>
__global__ void __launch_bounds__(128) k_conv_wgrad(const __nv_bfloat16* __restrict__ X,
                                                    const __nv_bfloat16* __restrict__ dY, int dy_stride, int h, int w,
                                                    float* __restrict__ dW, float* __restrict__ db, int cin_real,
                                                    int cout_real)
{
    constexpr int HW = BW + 2 * DIL, HH = BH + 2 * DIL;
    constexpr int PX = BW * BH;        // 128 pixels
    constexpr int SPD = PX + 8;        // dY^T row stride (bf16)
    constexpr int SPX = HH * HW + 8;   // X^T row stride (bf16)
    constexpr int MT = COUTD / 16, NT = CINP / 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __nv_bfloat16* s_dy = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    __nv_bfloat16* s_x = s_dy + COUTD * SPD;
    const int tid = threadIdx.x;
    const int x0 = blockIdx.x * BW, y0 = blockIdx.y * BH, b = blockIdx.z;
    for (int k = tid; k < COUTD * PX; k += 128) {
        const int co = k / PX, p = k - co * PX;
        const int y = y0 + p / BW, x = x0 + (p % BW);
        __nv_bfloat16 v = __float2bfloat16(0.0f);
        if (co < cout_real && y < h && x < w) v = dY[(((size_t)b * h + y) * w + x) * dy_stride + co];
        s_dy[co * SPD + p] = v;
    }
    for (int k = tid; k < CINP * HH * HW; k += 128) {
        const int ci = k / (HH * HW), p = k - ci * (HH * HW);
        const int gy = y0 + p / HW - DIL, gx = x0 + (p % HW) - DIL;
        __nv_bfloat16 v = __float2bfloat16(0.0f);
        if (gy >= 0 && gy < h && gx >= 0 && gx < w) v = X[(((size_t)b * h + gy) * w + gx) * CINP + ci];
        s_x[ci * SPX + p] = v;
    }
    __syncthreads();
    // bias gradient
    for (int co = tid; co < cout_real; co += 128) {
        float s = 0.0f;
        for (int p = 0; p < PX; p++) s += __bfloat162float(s_dy[co * SPD + p]);
        atomicAdd(db + co, s);
    }
    const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    const unsigned short* sx16 = reinterpret_cast<const unsigned short*>(s_x);
    const uint32_t* sdy = reinterpret_cast<const uint32_t*>(s_dy);
    for (int tap = warp; tap < 9; tap += 4) {
        const int dyy = tap / 3, dxx = tap - dyy * 3;
        float acc[MT][NT][4];
#pragma unroll
        for (int mt = 0; mt < MT; mt++)
#pragma unroll
            for (int nt = 0; nt < NT; nt++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[mt][nt][q] = 0.0f;
#pragma unroll 2
        for (int ks = 0; ks < BH; ks++) {  // one tile row of 16 pixels per k-step
            uint32_t a[MT][4];
#pragma unroll
            for (int mt = 0; mt < MT; mt++) {
                const int r0 = (mt * 16 + g) * SPD + ks * 16 + 2 * t;
                const int r8 = (mt * 16 + g + 8) * SPD + ks * 16 + 2 * t;
                a[mt][0] = sdy[r0 >> 1];
                a[mt][1] = sdy[r8 >> 1];
                a[mt][2] = sdy[(r0 >> 1) + 4];
                a[mt][3] = sdy[(r8 >> 1) + 4];
            }
#pragma unroll
            for (int nt = 0; nt < NT; nt++) {
                const int ci = nt * 8 + g;
                const int row = (ks + dyy * DIL) * HW + dxx * DIL;  // shifted input row for pixels 0..15
                const int base = ci * SPX + row + 2 * t;
                const uint32_t b0 = (uint32_t)sx16[base] | ((uint32_t)sx16[base + 1] << 16);
                const uint32_t b1 = (uint32_t)sx16[base + 8] | ((uint32_t)sx16[base + 9] << 16);
#pragma unroll
                for (int mt = 0; mt < MT; mt++) mma_bf16(acc[mt][nt], a[mt], b0, b1);
            }
        }
        // C fragment: rows g / g+8 = output channel, cols 2t, 2t+1 = input channel
#pragma unroll
        for (int mt = 0; mt < MT; mt++)
#pragma unroll
            for (int nt = 0; nt < NT; nt++)
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int co = mt * 16 + g + (q >> 1) * 8;
                    const int ci = nt * 8 + 2 * t + (q & 1);
                    if (co < cout_real && ci < cin_real)
                        atomicAdd(dW + ((size_t)co * 9 + tap) * cin_real + ci, acc[mt][nt][q]);
                }
    }
}

// Two frames -> network input: each frame's 4x4 pixel block of a quarter-resolution
// cell as 16 channels (channel 4*j + i = pixel (i, j) of the block; frame 1 in
// channels 16..31), scaled to [-1, 1], as a 32-channel NHWC bf16 image.
__global__ void k_net_input(const uint8_t* __restrict__ f0, const uint8_t* __restrict__ f1, int W, int H,
                            __nv_bfloat16* __restrict__ out, int w4, int h4)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w4 || y >= h4) return;
    uint32_t v[16];
    // a cell's 4x4 block lies inside the frame (w4 = W / 4, h4 = H / 4); with W a
    // multiple of 4 each of its rows is one aligned 32-bit word
    const bool words = (W & 3) == 0 && (reinterpret_cast<uintptr_t>(f0) & 3) == 0 &&
                       (reinterpret_cast<uintptr_t>(f1) & 3) == 0;
    uint32_t row[2][4];
#pragma unroll
    for (int f = 0; f < 2; f++) {
        const uint8_t* src = f ? f1 : f0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint8_t* p = src + (size_t)(y * 4 + j) * W + x * 4;
            row[f][j] = words ? __ldg(reinterpret_cast<const uint32_t*>(p))
                              : (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
        }
    }
#pragma unroll
    for (int f = 0; f < 2; f++)
#pragma unroll
        for (int j = 0; j < 4; j++)
#pragma unroll
            for (int i = 0; i < 4; i += 2) {
                const float a = (float)((row[f][j] >> (8 * i)) & 0xFFu) / 127.5f - 1.0f;
                const float b = (float)((row[f][j] >> (8 * (i + 1))) & 0xFFu) / 127.5f - 1.0f;
                v[f * 8 + j * 2 + i / 2] = pack_bf16(a, b);
            }
    uint4* o = reinterpret_cast<uint4*>(out + ((size_t)y * w4 + x) * NIN);
#pragma unroll
    for (int q = 0; q < 4; q++) o[q] = make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

// The same from frames reduced by `red` (2 or 4, lg = log2(red)): the cell (x, y)
// covers the 4x4 reduced pixels (4x + i, 4y + j), each the mean of the red x red
// input pixels it stands for, rounded half to even to an 8-bit value (w4 = (W / red)
// / 4, h4 = (H / red) / 4, so every block lies inside the frame).
__global__ void k_net_input_reduced(const uint8_t* __restrict__ f0, const uint8_t* __restrict__ f1, int W,
                                    __nv_bfloat16* __restrict__ out, int w4, int h4, int red, int lg)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w4 || y >= h4) return;
    const uint32_t sh = 2u * (uint32_t)lg, half = 1u << (sh - 1), mask = (1u << sh) - 1u;
    uint32_t v[16];
#pragma unroll
    for (int f = 0; f < 2; f++) {
        const uint8_t* src = f ? f1 : f0;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float val[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const uint8_t* p = src + (size_t)((4 * y + j) * red) * W + (size_t)(4 * x + i) * red;
                uint32_t sum = 0;
                for (int a = 0; a < red; a++)
                    for (int b = 0; b < red; b++) sum += __ldg(p + (size_t)a * W + b);
                const uint32_t q = sum >> sh, rem = sum & mask;
                const uint32_t m = q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u);
                val[i] = (float)m / 127.5f - 1.0f;
            }
            v[f * 8 + j * 2] = pack_bf16(val[0], val[1]);
            v[f * 8 + j * 2 + 1] = pack_bf16(val[2], val[3]);
        }
    }
    uint4* o = reinterpret_cast<uint4*>(out + ((size_t)y * w4 + x) * NIN);
#pragma unroll
    for (int q = 0; q < 4; q++) o[q] = make_uint4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

// Loss of the head against BriefMatch's flow: smooth-L1 on (u, v) in quarter
// resolution pixels and binary cross-entropy of the confidence against "the
// predicted vector is within tau of the target", averaged over valid pixels.
// Writes dY (bf16, 16 channels) and adds the loss terms to loss[0..2].
__global__ void k_net_loss(const float* __restrict__ pred, const float* __restrict__ target, size_t n,
                           __nv_bfloat16* __restrict__ dY, float inv_count, float tau, float wconf,
                           float* __restrict__ loss)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    float lf = 0, lc = 0, acc = 0;
    if (i < n) {
        const float u = pred[i * 3], v = pred[i * 3 + 1], c = pred[i * 3 + 2];
        const float tu = target[i * 3], tv = target[i * 3 + 1], valid = target[i * 3 + 2];
        const float du = u - tu, dv = v - tv;
        auto sl1 = [](float d, float& g) {
            const float a = fabsf(d);
            if (a < 1.0f) {
                g = d;
                return 0.5f * d * d;
            }
            g = d > 0 ? 1.0f : -1.0f;
            return a - 0.5f;
        };
        float gu, gv;
        lf = (sl1(du, gu) + sl1(dv, gv)) * valid;
        const float label = (fabsf(du) + fabsf(dv) < tau) ? 1.0f : 0.0f;
        const float sig = 1.0f / (1.0f + expf(-c));
        lc = valid * (fmaxf(c, 0.0f) - c * label + log1pf(expf(-fabsf(c))));
        acc = valid * label;
        uint4* o = reinterpret_cast<uint4*>(dY + i * 16);
        o[0] = make_uint4(pack_bf16(gu * valid * inv_count, gv * valid * inv_count),
                          pack_bf16(wconf * (sig - label) * valid * inv_count, 0.0f), 0, 0);
        o[1] = make_uint4(0, 0, 0, 0);
    }
    // block reduction of the loss terms
    __shared__ float red[3][256];
    red[0][threadIdx.x] = lf;
    red[1][threadIdx.x] = lc;
    red[2][threadIdx.x] = acc;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int k = 0; k < 3; k++) red[k][threadIdx.x] += red[k][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        atomicAdd(loss + 0, red[0][0] * inv_count);
        atomicAdd(loss + 1, red[1][0] * inv_count);
        atomicAdd(loss + 2, red[2][0] * inv_count);
    }
}

// Adam on the FP32 master parameters (Kingma & Ba, ICLR 2015).
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       size_t n, float lr, float b1, float b2, float eps, float c1, float c2, float wd)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] + wd * p[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// FP32 master parameters of one layer -> the BF16 forward layout W[tap][COUTP][CINP]
// and the backward-data layout Wb[tap][CINP_as_out][COUTP16_as_in] (taps flipped).
__global__ void k_pack_layer(const float* __restrict__ master, int cin, int cout, int cinp, int coutp, int coutp16,
                             __nv_bfloat16* __restrict__ Wf, __nv_bfloat16* __restrict__ Wb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int nf = 9 * coutp * cinp;
    if (i < nf) {
        const int tap = i / (coutp * cinp), r = i - tap * coutp * cinp, co = r / cinp, ci = r - co * cinp;
        const float v = (co < cout && ci < cin) ? master[((size_t)co * 9 + tap) * cin + ci] : 0.0f;
        Wf[i] = __float2bfloat16(v);
    }
    const int nb = 9 * cinp * coutp16;
    if (Wb && i < nb) {
        const int tap = i / (cinp * coutp16), r = i - tap * cinp * coutp16, ci = r / coutp16, co = r - ci * coutp16;
        const int ftap = 8 - tap;
        const float v = (co < cout && ci < cin) ? master[((size_t)co * 9 + ftap) * cin + ci] : 0.0f;
        Wb[i] = __float2bfloat16(v);
    }
}

template <int CINP, int COUTP, int EPI, int D>
cudaError_t launch_conv(const __nv_bfloat16* X, const __nv_bfloat16* W, const float* bias, const __nv_bfloat16* act,
                        void* out, int B, int h, int w, int cout_real, int out_stride, cudaStream_t st)
{
    dim3 g((w + BW - 1) / BW, (h + BH - 1) / BH, B);
    k_conv<CINP, COUTP, EPI, D><<<g, 128, conv_smem(CINP, COUTP, D), st>>>(X, W, bias, act, out, h, w, cout_real,
                                                                            out_stride);
    return cudaGetLastError();
}

template <int CINP, int COUTD, int D>
cudaError_t launch_wgrad(const __nv_bfloat16* X, const __nv_bfloat16* dY, int dy_stride, int B, int h, int w,
                         float* dW, float* db, int cin_real, int cout_real, cudaStream_t st)
{
    dim3 g((w + BW - 1) / BW, (h + BH - 1) / BH, B);
    k_conv_wgrad<CINP, COUTD, D><<<g, 128, wgrad_smem(CINP, COUTD, D), st>>>(X, dY, dy_stride, h, w, dW, db, cin_real,
                                                                              cout_real);
    return cudaGetLastError();
}

// Forward and backward-data of layer l (dilation DIL[l]), weight gradient of layer l.
cudaError_t conv_fwd(int l, const __nv_bfloat16* X, const __nv_bfloat16* W, const float* bias, void* out, int B, int h,
                     int w, cudaStream_t st)
{
    switch (DIL[l]) {
    case 1: return launch_conv<32, 32, EPI_RELU_BF16, 1>(X, W, bias, nullptr, out, B, h, w, 32, 32, st);
    case 2: return launch_conv<32, 32, EPI_RELU_BF16, 2>(X, W, bias, nullptr, out, B, h, w, 32, 32, st);
    case 4: return launch_conv<32, 32, EPI_RELU_BF16, 4>(X, W, bias, nullptr, out, B, h, w, 32, 32, st);
    default: return launch_conv<32, 32, EPI_RELU_BF16, 8>(X, W, bias, nullptr, out, B, h, w, 32, 32, st);
    }
}
cudaError_t conv_bwd_data(int l, const __nv_bfloat16* dY, const __nv_bfloat16* Wb, const __nv_bfloat16* act, void* out,
                          int B, int h, int w, cudaStream_t st)
{
    switch (DIL[l]) {
    case 1: return launch_conv<32, 32, EPI_MASK_BF16, 1>(dY, Wb, nullptr, act, out, B, h, w, 32, 32, st);
    case 2: return launch_conv<32, 32, EPI_MASK_BF16, 2>(dY, Wb, nullptr, act, out, B, h, w, 32, 32, st);
    case 4: return launch_conv<32, 32, EPI_MASK_BF16, 4>(dY, Wb, nullptr, act, out, B, h, w, 32, 32, st);
    default: return launch_conv<32, 32, EPI_MASK_BF16, 8>(dY, Wb, nullptr, act, out, B, h, w, 32, 32, st);
    }
}
cudaError_t conv_wgrad(int l, const __nv_bfloat16* X, const __nv_bfloat16* dY, int B, int h, int w, float* dW, float* db,
                       cudaStream_t st)
{
    switch (DIL[l]) {
    case 1: return launch_wgrad<32, 32, 1>(X, dY, 32, B, h, w, dW, db, 32, 32, st);
    case 2: return launch_wgrad<32, 32, 2>(X, dY, 32, B, h, w, dW, db, 32, 32, st);
    case 4: return launch_wgrad<32, 32, 4>(X, dY, 32, B, h, w, dW, db, 32, 32, st);
    default: return launch_wgrad<32, 32, 8>(X, dY, 32, B, h, w, dW, db, 32, 32, st);
    }
}

// ---------------------------------------------------------------------------
// tcgen05 implicit-GEMM 3x3 convolution.  One CTA of 128 threads per run of UM = 128
// consecutive cells of one image row: D[cell][co] = sum over taps t and input channels
// ci of X[cell + shift(t)][ci] * W[t][co][ci].  Shared memory holds the nine taps'
// A tiles (128 cells x 32 channels, 8 KB each) and the weights B (9 x N x 32); both
// arrive by TMA with 64-byte swizzling, which is the canonical K-major layout the MMA
// descriptors name (rows of 64 bytes, 8-row groups 512 bytes apart).  A tap whose
// source row lies outside the image is neither loaded nor multiplied (its A tile would
// be zeros); a tap shifted past the left or right edge reads TMA's zero fill.  Thread 0
// issues the copies and the 18 MMAs (M=128, N, K=16) into a 32-column TMEM
// accumulator; all four warps then read their 32 TMEM lanes (cells) and apply the
// epilogue.  Every wait is bounded: a wait that gives up records an error word and the
// CTA still frees its tensor memory before it returns.
// ---------------------------------------------------------------------------
constexpr int UM = 128;                                 // cells per CTA (MMA M)
constexpr uint32_t U_TAP_A = UM * 32 * 2;               // bytes of one tap's A tile
constexpr unsigned long long U_POLLS = 1ull << 20;      // polls of a wait before it gives up

constexpr size_t umma_smem(int n) { return 1024 + 9 * (size_t)U_TAP_A + 9 * (size_t)n * 64; }

__device__ __forceinline__ uint32_t s_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_addr(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s_addr(bar)) : "memory");
}
// Polls the barrier's phase `parity` at most `polls` times; true once it completed.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long polls)
{
    for (unsigned long long i = 0; i < polls; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(s_addr(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (i > 1024) __nanosleep(64);
    }
    return false;
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(s_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(s_addr(bar))
        : "memory");
}
// Shared-memory matrix descriptor: K-major, 64-byte swizzle, 8-row groups 512 B apart.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);       // start address
    d |= (uint64_t)1 << 16;                       // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512 >> 4) << 32;              // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                       // descriptor version (sm_100 family)
    d |= (uint64_t)4 << 61;                       // swizzle mode: 64-byte
    return d;
}
// Instruction descriptor of kind::f16: BF16 A and B (K-major), FP32 D, M x N.
__host__ __device__ constexpr uint32_t umma_idesc(int m, int n)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

template <int EPI, int N>
__global__ void __launch_bounds__(128) k_conv_umma(const __grid_constant__ CUtensorMap tmX,
                                                   const __grid_constant__ CUtensorMap tmW,
                                                   const float* __restrict__ bias,
                                                   const __nv_bfloat16* __restrict__ act, void* __restrict__ out,
                                                   int h, int w, int dil, int cout_real, int out_stride,
                                                   int* __restrict__ err)
{
    static_assert(N == 16 || N == 32, "N is 16 or 32 output channels");
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = sm;                     // 9 taps x 8 KB
    unsigned char* sB = sm + 9 * U_TAP_A;       // 9 taps x N rows x 64 B
    __shared__ __align__(8) uint64_t bar_load, bar_mma;
    __shared__ uint32_t s_tmem;
    __shared__ int s_ok;

    const int tiles_x = (w + UM - 1) / UM;
    const int row = blockIdx.x / tiles_x;               // image row over the batch, b * h + y
    const int x0 = (blockIdx.x - row * tiles_x) * UM;
    const int y = row % h;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        mbar_init(&bar_load, 1);
        mbar_init(&bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_ok = 1;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(s_addr(&s_tmem))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;

    if (threadIdx.x == 0) {
        uint32_t taps = 0, bytes = 9u * N * 64;
        for (int t = 0; t < 9; t++) {
            const int r = y + (t / 3 - 1) * dil;
            if (r >= 0 && r < h) {
                taps |= 1u << t;
                bytes += U_TAP_A;
            }
        }
        mbar_expect_tx(&bar_load, bytes);
        tma_load_3d(sB, &tmW, 0, 0, 0, &bar_load);
        for (int t = 0; t < 9; t++)
            if (taps >> t & 1u)
                tma_load_3d(sA + t * U_TAP_A, &tmX, 0, x0 + (t % 3 - 1) * dil, row + (t / 3 - 1) * dil, &bar_load);
        if (mbar_wait(&bar_load, 0, U_POLLS)) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            constexpr uint32_t idesc = umma_idesc(UM, N);
            uint32_t acc = 0;
            for (int t = 0; t < 9; t++) {
                if (!(taps >> t & 1u)) continue;
                const uint32_t a0 = s_addr(sA + t * U_TAP_A), b0 = s_addr(sB + t * N * 64);
#pragma unroll
                for (int kh = 0; kh < 2; kh++) {  // K = 16 channels (32 bytes) per MMA
                    const uint64_t ad = umma_desc(a0 + kh * 32), bd = umma_desc(b0 + kh * 32);
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                        ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                        : "memory");
                    acc = 1;
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         ::"r"(s_addr(&bar_mma)) : "memory");
        } else {
            // the copies did not land in time: give them one more bounded wait (they
            // write this CTA's shared memory) and release the others without an MMA
            atomicExch(err, 1);
            s_ok = 0;
            mbar_wait(&bar_load, 0, U_POLLS);
            mbar_arrive(&bar_mma);
        }
    }
    // tcgen05.ld is warp-collective: the block agrees on one outcome of the wait
    const bool mine = mbar_wait(&bar_mma, 0, U_POLLS);
    const bool done = __syncthreads_and(mine ? 1 : 0) != 0;
    if (!done && threadIdx.x == 0) atomicExch(err, 2);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (done && s_ok) {
        uint32_t r[N];
        const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
        if constexpr (N == 32) {
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                  "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),
                  "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                : "r"(taddr));
        } else {
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
                "[%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(taddr));
        }
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        const int x = x0 + warp * 32 + lane;
        if (x < w) {
            const size_t pix = (size_t)row * w + x;
            if constexpr (EPI == EPI_LINEAR_F32) {
                float* o = reinterpret_cast<float*>(out) + pix * out_stride;
#pragma unroll
                for (int co = 0; co < N; co++)
                    if (co < cout_real) o[co] = __uint_as_float(r[co]) + __ldg(bias + co);
            } else {
                uint32_t packed[N / 2];
                if constexpr (EPI == EPI_MASK_BF16) {
                    const uint4* m4 = reinterpret_cast<const uint4*>(act + pix * out_stride);
#pragma unroll
                    for (int q = 0; q < N / 8; q++) {
                        const uint4 mv = m4[q];
                        const uint32_t mw[4] = {mv.x, mv.y, mv.z, mv.w};
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const int co = q * 8 + 2 * k;
                            const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162*>(&mw[k]);
                            const float v0 = __bfloat162float(m.x) > 0.0f ? __uint_as_float(r[co]) : 0.0f;
                            const float v1 = __bfloat162float(m.y) > 0.0f ? __uint_as_float(r[co + 1]) : 0.0f;
                            packed[co / 2] = pack_bf16(v0, v1);
                        }
                    }
                } else {
#pragma unroll
                    for (int co = 0; co < N; co += 2)
                        packed[co / 2] = pack_bf16(fmaxf(__uint_as_float(r[co]) + __ldg(bias + co), 0.0f),
                                                   fmaxf(__uint_as_float(r[co + 1]) + __ldg(bias + co + 1), 0.0f));
                }
                uint4* o4 = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out) + pix * out_stride);
#pragma unroll
                for (int q = 0; q < N / 8; q++)
                    o4[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem) : "memory");
}

// cuTensorMapEncodeTiled, fetched through the runtime (the library does not link the
// driver library itself).
typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encoder()
{
    // looked up once per process (a function-local static initialises thread-safely)
    static const EncodeTiled fn = []() -> EncodeTiled {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            return reinterpret_cast<EncodeTiled>(f);
        return nullptr;
    }();
    return fn;
}

// A 3-D BF16 tensor map with 64-byte rows: dims {32 channels, d1, d2}, box {32, b1, b2},
// 64-byte swizzle, zero fill out of bounds.
bool encode_map(CUtensorMap* map, const void* base, uint64_t d1, uint64_t d2, uint32_t b1, uint32_t b2)
{
    EncodeTiled enc = encoder();
    if (!enc) return false;
    const cuuint64_t dims[3] = {32, d1, d2};
    const cuuint64_t strides[2] = {64, 64 * d1};
    const cuuint32_t box[3] = {32, b1, b2};
    const cuuint32_t estr[3] = {1, 1, 1};
    return enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Activations [B*h][w][32] as the A operand of a conv layer.
bool act_map(CUtensorMap* map, const __nv_bfloat16* X, int B, int h, int w)
{
    return encode_map(map, X, (uint64_t)w, (uint64_t)B * h, UM, 1);
}
// Weights [9][n][32] as the B operand (all nine taps in one copy).
bool weight_map(CUtensorMap* map, const __nv_bfloat16* W, int n) { return encode_map(map, W, (uint64_t)n, 9, n, 9); }

template <int EPI, int N>
cudaError_t launch_conv_umma(const CUtensorMap& mx, const CUtensorMap& mw, const float* bias, const __nv_bfloat16* act,
                             void* out, int B, int h, int w, int dil, int cout_real, int out_stride, int* err,
                             cudaStream_t st)
{
    const unsigned tiles = (unsigned)(((w + UM - 1) / UM) * (size_t)B * h);
    k_conv_umma<EPI, N><<<tiles, 128, umma_smem(N), st>>>(mx, mw, bias, act, out, h, w, dil, cout_real, out_stride,
                                                           err);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// The whole forward pass in one cooperative launch (k_net_fused): every CTA keeps
// its tensor memory and barriers for all six layers and walks the layer's 128-cell
// tiles with a grid stride; between layers the CTAs meet at a bounded grid barrier,
// the outputs of a layer having been written with plain stores and fenced for the
// next layer's TMA reads (proxy fences on both sides of the barrier).  It replaces
// six launches and their per-launch set-up (barrier init, TMEM allocation, weight
// copy) with one.
// ---------------------------------------------------------------------------
struct NetGridBar {
    unsigned int arrived;
    unsigned int generation;
    unsigned int error;
};

struct NetFusedArgs {
    CUtensorMap in_map[NL];    // A operand of each layer (layer 0: the input image)
    CUtensorMap w_map[NL];     // B operand (weights) of each layer
    const float* bias[NL];
    __nv_bfloat16* act[NL - 1];  // outputs of layers 0..4
    float* head;                 // [cells][3]
    int h, w, rows;              // rows = B * h
    int dil[NL];
    unsigned long long polls;
    NetGridBar* bar;
    int* err;
};

// Bounded grid barrier: false when it gave up (then the error word is set).
__device__ __forceinline__ bool net_grid_sync(NetGridBar* gb, unsigned int nblocks, unsigned long long polls)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int* vgen = &gb->generation;
        volatile unsigned int* verr = &gb->error;
        const unsigned int gen = *vgen;
        __threadfence();
        if (atomicAdd(&gb->arrived, 1u) == nblocks - 1) {
            atomicExch(&gb->arrived, 0u);
            __threadfence();
            atomicAdd(&gb->generation, 1u);
        } else {
            unsigned long long i = 0;
            while (*vgen == gen) {
                if (*verr || ++i > polls) {
                    atomicExch(&gb->error, 1u);
                    ok = 0;
                    break;
                }
                if (i > 4096) __nanosleep(64);  // spin first: a layer's barrier clears in microseconds
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Epilogue of one tile: TMEM lanes of this warp -> the cells' output channels.
template <int EPI, int N>
__device__ __forceinline__ void umma_epilogue(uint32_t taddr, const float* __restrict__ bias, void* __restrict__ out,
                                              size_t pix, bool in_image, int cout_real, int out_stride)
{
    uint32_t r[N];
    if constexpr (N == 32) {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
              "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
              "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
              "=r"(r[30]), "=r"(r[31])
            : "r"(taddr));
    } else {
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
              "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
            : "r"(taddr));
    }
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (!in_image) return;
    if constexpr (EPI == EPI_LINEAR_F32) {
        float* o = reinterpret_cast<float*>(out) + pix * out_stride;
#pragma unroll
        for (int co = 0; co < N; co++)
            if (co < cout_real) o[co] = __uint_as_float(r[co]) + __ldg(bias + co);
    } else {
        uint32_t packed[N / 2];
#pragma unroll
        for (int co = 0; co < N; co += 2)
            packed[co / 2] = pack_bf16(fmaxf(__uint_as_float(r[co]) + __ldg(bias + co), 0.0f),
                                       fmaxf(__uint_as_float(r[co + 1]) + __ldg(bias + co + 1), 0.0f));
        uint4* o4 = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out) + pix * out_stride);
#pragma unroll
        for (int q = 0; q < N / 8; q++)
            o4[q] = make_uint4(packed[4 * q], packed[4 * q + 1], packed[4 * q + 2], packed[4 * q + 3]);
    }
}

__global__ void __launch_bounds__(128) k_net_fused(const __grid_constant__ NetFusedArgs a)
{
    extern __shared__ unsigned char smem_raw[];
    unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = sm;
    unsigned char* sB = sm + 9 * U_TAP_A;
    __shared__ __align__(8) uint64_t bar_load, bar_mma;
    __shared__ uint32_t s_tmem;
    __shared__ int s_ok;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tiles_x = (a.w + UM - 1) / UM;
    const int tiles = tiles_x * a.rows;

    if (threadIdx.x == 0) {
        mbar_init(&bar_load, 1);
        mbar_init(&bar_mma, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_ok = 1;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(s_addr(&s_tmem))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = s_tmem;
    uint32_t phase = 0;  // uses of bar_load / bar_mma so far (both advance together)

    for (int l = 0; l < NL; l++) {
        const int n = l == NL - 1 ? 16 : 32;
        const int dil = a.dil[l];
        bool weights_in = false;
        for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
            const int row = tile / tiles_x;
            const int x0 = (tile - row * tiles_x) * UM;
            const int y = row % a.h;
            if (threadIdx.x == 0 && s_ok) {
                uint32_t taps = 0, bytes = weights_in ? 0u : 9u * n * 64;
                for (int t = 0; t < 9; t++) {
                    const int r = y + (t / 3 - 1) * dil;
                    if (r >= 0 && r < a.h) {
                        taps |= 1u << t;
                        bytes += U_TAP_A;
                    }
                }
                // reads of the previous layer's outputs go through the async proxy
                asm volatile("fence.proxy.async.global;" ::: "memory");
                mbar_expect_tx(&bar_load, bytes);
                if (!weights_in) tma_load_3d(sB, &a.w_map[l], 0, 0, 0, &bar_load);
                for (int t = 0; t < 9; t++)
                    if (taps >> t & 1u)
                        tma_load_3d(sA + t * U_TAP_A, &a.in_map[l], 0, x0 + (t % 3 - 1) * dil, row + (t / 3 - 1) * dil,
                                    &bar_load);
                if (mbar_wait(&bar_load, phase & 1u, a.polls)) {
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t idesc = n == 16 ? umma_idesc(UM, 16) : umma_idesc(UM, 32);
                    uint32_t acc = 0;
                    for (int t = 0; t < 9; t++) {
                        if (!(taps >> t & 1u)) continue;
                        const uint32_t a0 = s_addr(sA + t * U_TAP_A), b0 = s_addr(sB + t * n * 64);
#pragma unroll
                        for (int kh = 0; kh < 2; kh++) {
                            const uint64_t ad = umma_desc(a0 + kh * 32), bd = umma_desc(b0 + kh * 32);
                            asm volatile(
                                "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
                                ::"r"(tmem), "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
                                : "memory");
                            acc = 1;
                        }
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                                 ::"r"(s_addr(&bar_mma)) : "memory");
                } else {
                    atomicExch(a.err, 1);
                    s_ok = 0;
                    mbar_wait(&bar_load, phase & 1u, a.polls);
                    mbar_arrive(&bar_mma);
                }
            }
            weights_in = true;
            __syncthreads();   // s_ok as thread 0 left it for this tile
            if (!s_ok) break;
            // tcgen05.ld is warp-collective: the block agrees on one outcome of the wait
            const bool mine = mbar_wait(&bar_mma, phase & 1u, a.polls);
            if (!__syncthreads_and(mine ? 1 : 0)) {
                if (threadIdx.x == 0) {
                    atomicExch(a.err, 2);
                    s_ok = 0;
                }
                __syncthreads();
            }
            phase++;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const int x = x0 + warp * 32 + lane;
            const size_t pix = (size_t)row * a.w + x;
            const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
            if (s_ok) {
                if (l == NL - 1)
                    umma_epilogue<EPI_LINEAR_F32, 16>(taddr, a.bias[l], a.head, pix, x < a.w, 3, 3);
                else
                    umma_epilogue<EPI_RELU_BF16, 32>(taddr, a.bias[l], a.act[l], pix, x < a.w, 32, 32);
            }
            // the accumulator is read before the next tile's MMAs overwrite it
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!s_ok) break;
        }
        if (!s_ok) atomicExch(&a.bar->error, 1u);  // the others stop at the barrier
        if (l == NL - 1) break;
        // this layer's plain stores, before other CTAs read them through TMA
        asm volatile("fence.proxy.async.global;" ::: "memory");
        if (!net_grid_sync(a.bar, gridDim.x, a.polls)) {
            if (threadIdx.x == 0) atomicExch(a.err, 3);
            break;
        }
        if (!s_ok) break;
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(tmem) : "memory");
}

// Dynamic shared-memory opt-in of every instantiation above 48 KB (once per process
// and device; called from bm_net_create, outside any stream capture).
cudaError_t conv_smem_optin()
{
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(mu);
    if (dev < 64 && done[dev]) return cudaSuccess;
    auto set = [](const void* f, size_t bytes) {
        return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    };
    const cudaError_t es[] = {
        set((const void*)k_conv<32, 32, EPI_RELU_BF16, 4>, conv_smem(32, 32, 4)),
        set((const void*)k_conv<32, 32, EPI_RELU_BF16, 8>, conv_smem(32, 32, 8)),
        set((const void*)k_conv<32, 32, EPI_MASK_BF16, 4>, conv_smem(32, 32, 4)),
        set((const void*)k_conv<32, 32, EPI_MASK_BF16, 8>, conv_smem(32, 32, 8)),
        set((const void*)k_conv_wgrad<32, 32, 4>, wgrad_smem(32, 32, 4)),
        set((const void*)k_conv_wgrad<32, 32, 8>, wgrad_smem(32, 32, 8)),
        set((const void*)k_conv_umma<EPI_RELU_BF16, 32>, umma_smem(32)),
        set((const void*)k_conv_umma<EPI_MASK_BF16, 32>, umma_smem(32)),
        set((const void*)k_conv_umma<EPI_LINEAR_F32, 16>, umma_smem(16)),
        set((const void*)k_net_fused, umma_smem(32)),
    };
    for (cudaError_t x : es)
        if (x != cudaSuccess) return x;
    // the tcgen05 kernels take 93 KB each: ask for the largest shared-memory carve-out
    // so that two CTAs share an SM (the fused launch then holds a 1024x436 frame's 218
    // tiles in one wave)
    const void* big[] = {(const void*)k_conv_umma<EPI_RELU_BF16, 32>, (const void*)k_conv_umma<EPI_MASK_BF16, 32>,
                         (const void*)k_conv_umma<EPI_LINEAR_F32, 16>, (const void*)k_net_fused};
    for (const void* f : big) {
        const cudaError_t e2 = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout,
                                                    (int)cudaSharedmemCarveoutMaxShared);
        if (e2 != cudaSuccess) return e2;
    }
    if (dev < 64) done[dev] = true;
    return cudaSuccess;
}

size_t layer_w_count(int l) { return (size_t)COUT_R[l] * 9 * CIN_R[l]; }
size_t layer_param_count(int l) { return layer_w_count(l) + COUT_R[l]; }

}  // namespace

struct bm_net {
    uint32_t maxB = 0, maxh = 0, maxw = 0;
    size_t nparam = 0;
    size_t poff[NL] = {};         // offset of layer l's weights in the parameter vector (bias follows)
    float* d_master = nullptr;    // FP32 parameters
    float* d_grad = nullptr;
    float* d_m = nullptr;
    float* d_v = nullptr;
    __nv_bfloat16* d_wf[NL] = {};
    __nv_bfloat16* d_wb[NL] = {};
    __nv_bfloat16* d_in = nullptr;      // [B][h][w][32]
    __nv_bfloat16* d_act[NL - 1] = {};  // outputs of layers 0..4, [B][h][w][32]
    __nv_bfloat16* d_dy[2] = {};        // gradient ping-pong, [B][h][w][32]
    float* d_out = nullptr;             // [B][h][w][3]
    float* d_loss = nullptr;            // 3 floats
    uint64_t step = 0;
    bool packed = false;
    // bm_net_snapshot: two slots, each a device copy of the master parameters and both
    // Adam moments (3 * nparam floats, allocated on first use) and the step count
    float* d_snap = nullptr;
    uint64_t snap_step[2] = {};
    bool has_snap[2] = {};

    // tcgen05 path (k_conv_umma): tensor maps of the weights (fixed buffers) and of the
    // activations for the last (B, h, w) seen; error word of its bounded waits
    bool umma = false;
    bool fused = false;          // the six layers in one cooperative launch (k_net_fused)
    int fused_grid_max = 0;      // co-resident CTAs of k_net_fused on this device
    NetGridBar* d_bar = nullptr;
    int* d_err = nullptr;
    CUtensorMap map_wf[NL];
    CUtensorMap map_wb[NL];
    uint32_t map_B = 0, map_h = 0, map_w = 0;
    CUtensorMap map_in;
    CUtensorMap map_act[NL - 1];
    CUtensorMap map_dy[2];
};

namespace {

bm_status nfail(bm_status st, const char* msg)
{
    bmk::set_error_text(msg);
    return st;
}

#define BN_CUDA(call)                                                       \
    do {                                                                    \
        cudaError_t e_ = (call);                                            \
        if (e_ != cudaSuccess) {                                            \
            char b_[256];                                                   \
            std::snprintf(b_, sizeof(b_), "bm_net: %s (line %d)", cudaGetErrorString(e_), __LINE__); \
            return nfail(BM_ERR_CUDA, b_);                                  \
        }                                                                   \
    } while (0)

bm_status pack_weights(bm_net* n, cudaStream_t st)
{
    for (int l = 0; l < NL; l++) {
        const int coutp16 = COUT_P[l] < 16 ? 16 : COUT_P[l];
        const int cnt = 9 * CIN_P[l] * coutp16 > 9 * COUT_P[l] * CIN_P[l] ? 9 * CIN_P[l] * coutp16 : 9 * COUT_P[l] * CIN_P[l];
        k_pack_layer<<<(cnt + 255) / 256, 256, 0, st>>>(n->d_master + n->poff[l], CIN_R[l], COUT_R[l], CIN_P[l], COUT_P[l],
                                                          coutp16, n->d_wf[l], l > 0 ? n->d_wb[l] : nullptr);
        BN_CUDA(cudaGetLastError());
    }
    n->packed = true;
    return BM_OK;
}

bm_status check_dims(bm_net* n, uint32_t B, uint32_t h, uint32_t w)
{
    if (B == 0 || h == 0 || w == 0 || B > n->maxB || (size_t)h * w > (size_t)n->maxh * n->maxw)
        return nfail(BM_ERR_LIMIT, "bm_net: batch or image size beyond the network's buffers");
    return BM_OK;
}

// Tensor maps of the activation buffers for a (B, h, w) call (host-side encoding only).
bool ensure_act_maps(bm_net* n, uint32_t B, uint32_t h, uint32_t w)
{
    if (n->map_B == B && n->map_h == h && n->map_w == w) return true;
    const int Bi = (int)B, hi = (int)h, wi = (int)w;
    bool ok = act_map(&n->map_in, n->d_in, Bi, hi, wi);
    for (int l = 0; ok && l < NL - 1; l++) ok = act_map(&n->map_act[l], n->d_act[l], Bi, hi, wi);
    for (int k = 0; ok && k < 2; k++) ok = act_map(&n->map_dy[k], n->d_dy[k], Bi, hi, wi);
    if (!ok) return false;
    n->map_B = B;
    n->map_h = h;
    n->map_w = w;
    return true;
}

bm_status forward(bm_net* n, uint32_t B, uint32_t h, uint32_t w, cudaStream_t st)
{
    if (!n->packed) {
        bm_status s = pack_weights(n, st);
        if (s != BM_OK) return s;
    }
    const int Bi = (int)B, hi = (int)h, wi = (int)w;
    if (n->umma) {
        if (!ensure_act_maps(n, B, h, w)) return nfail(BM_ERR_CUDA, "bm_net: tensor map encoding failed");
        if (n->fused) {
            NetFusedArgs a;
            for (int l = 0; l < NL; l++) {
                a.in_map[l] = l == 0 ? n->map_in : n->map_act[l - 1];
                a.w_map[l] = n->map_wf[l];
                a.bias[l] = n->d_master + n->poff[l] + layer_w_count(l);
                a.dil[l] = DIL[l];
            }
            for (int l = 0; l < NL - 1; l++) a.act[l] = n->d_act[l];
            a.head = n->d_out;
            a.h = hi;
            a.w = wi;
            a.rows = Bi * hi;
            a.polls = U_POLLS;
            a.bar = n->d_bar;
            a.err = n->d_err;
            const int tiles = ((wi + UM - 1) / UM) * Bi * hi;
            BN_CUDA(cudaMemsetAsync(n->d_bar, 0, sizeof(NetGridBar), st));
            void* args[] = {(void*)&a};
            cudaLaunchConfig_t cfg = {};
            cfg.blockDim = dim3(128);
            cfg.dynamicSmemBytes = umma_smem(32);
            cfg.stream = st;
            cudaLaunchAttribute attr;
            attr.id = cudaLaunchAttributeCooperative;
            attr.val.cooperative = 1;
            cfg.attrs = &attr;
            cfg.numAttrs = 1;
            cfg.gridDim = dim3((unsigned)std::min(tiles, n->fused_grid_max));
            BN_CUDA(cudaLaunchKernelExC(&cfg, (const void*)k_net_fused, args));
            return BM_OK;
        }
        for (int l = 0; l <= 4; l++)
            BN_CUDA((launch_conv_umma<EPI_RELU_BF16, 32>(l == 0 ? n->map_in : n->map_act[l - 1], n->map_wf[l],
                                                          n->d_master + n->poff[l] + layer_w_count(l), nullptr,
                                                          n->d_act[l], Bi, hi, wi, DIL[l], 32, 32, n->d_err, st)));
        BN_CUDA((launch_conv_umma<EPI_LINEAR_F32, 16>(n->map_act[4], n->map_wf[5],
                                                       n->d_master + n->poff[5] + layer_w_count(5), nullptr, n->d_out,
                                                       Bi, hi, wi, DIL[5], 3, 3, n->d_err, st)));
        return BM_OK;
    }
    for (int l = 0; l <= 4; l++)
        BN_CUDA(conv_fwd(l, l == 0 ? n->d_in : n->d_act[l - 1], n->d_wf[l], n->d_master + n->poff[l] + layer_w_count(l),
                         n->d_act[l], Bi, hi, wi, st));
    BN_CUDA((launch_conv<32, 16, EPI_LINEAR_F32, 1>(n->d_act[4], n->d_wf[5], n->d_master + n->poff[5] + layer_w_count(5),
                                                   nullptr, n->d_out, Bi, hi, wi, 3, 3, st)));
    return BM_OK;
}

}  // namespace

extern "C" {

size_t bm_net_param_count(void)
{
    size_t s = 0;
    for (int l = 0; l < NL; l++) s += layer_param_count(l);
    return s;
}

bm_status bm_net_create(uint32_t max_batch, uint32_t max_h4, uint32_t max_w4, bm_net** out)
{
    if (!out || max_batch == 0 || max_h4 == 0 || max_w4 == 0) return nfail(BM_ERR_INVALID, "bm_net_create: bad size");
    if (conv_smem_optin() != cudaSuccess) return nfail(BM_ERR_CUDA, "bm_net_create: shared-memory opt-in failed");
    bm_net* n = new bm_net();
    n->maxB = max_batch;
    n->maxh = max_h4;
    n->maxw = max_w4;
    size_t off = 0;
    for (int l = 0; l < NL; l++) {
        n->poff[l] = off;
        off += layer_param_count(l);
    }
    n->nparam = off;
    const size_t px = (size_t)max_batch * max_h4 * max_w4;
    bool ok = bmk::device_malloc((void**)&n->d_master, off * 4) == cudaSuccess &&
              bmk::device_malloc((void**)&n->d_grad, off * 4) == cudaSuccess &&
              bmk::device_malloc((void**)&n->d_m, off * 4) == cudaSuccess && bmk::device_malloc((void**)&n->d_v, off * 4) == cudaSuccess &&
              bmk::device_malloc((void**)&n->d_in, px * NIN * 2) == cudaSuccess &&
              bmk::device_malloc((void**)&n->d_out, px * 3 * 4) == cudaSuccess &&
              bmk::device_malloc((void**)&n->d_loss, 4 * 4) == cudaSuccess &&
              bmk::device_malloc((void**)&n->d_dy[0], px * 32 * 2) == cudaSuccess &&
              bmk::device_malloc((void**)&n->d_dy[1], px * 32 * 2) == cudaSuccess;
    for (int l = 0; ok && l < NL - 1; l++) ok = bmk::device_malloc((void**)&n->d_act[l], px * 32 * 2) == cudaSuccess;
    for (int l = 0; ok && l < NL; l++) {
        const int coutp16 = COUT_P[l] < 16 ? 16 : COUT_P[l];
        ok = bmk::device_malloc((void**)&n->d_wf[l], (size_t)9 * COUT_P[l] * CIN_P[l] * 2) == cudaSuccess &&
             bmk::device_malloc((void**)&n->d_wb[l], (size_t)9 * CIN_P[l] * coutp16 * 2) == cudaSuccess;
    }
    if (ok) ok = bmk::device_malloc((void**)&n->d_err, sizeof(int)) == cudaSuccess;
    if (ok) ok = bmk::device_malloc((void**)&n->d_bar, sizeof(NetGridBar)) == cudaSuccess;
    if (!ok) {
        bm_net_destroy(n);
        return nfail(BM_ERR_NOMEM, "bm_net_create: device allocation failed");
    }
    cudaMemset(n->d_err, 0, sizeof(int));
    // the tcgen05 path, when the driver encodes the weights' tensor maps
    n->umma = true;
    for (int l = 0; n->umma && l < NL; l++) n->umma = weight_map(&n->map_wf[l], n->d_wf[l], COUT_P[l]);
    for (int l = 1; n->umma && l < NL - 1; l++) n->umma = weight_map(&n->map_wb[l], n->d_wb[l], CIN_P[l]);
    {
        // co-resident CTAs of the fused launch (mode 2); the per-layer launches (mode 1)
        // measured faster and are the default
        int dev = 0, sms = 0, occ = 0, coop = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_net_fused, 128, umma_smem(32)) == cudaSuccess)
            n->fused_grid_max = occ * sms;
        n->fused = false;
    }
    cudaMemset(n->d_m, 0, off * 4);
    cudaMemset(n->d_v, 0, off * 4);
    cudaMemset(n->d_dy[0], 0, px * 32 * 2);
    cudaMemset(n->d_dy[1], 0, px * 32 * 2);
    // He initialisation from a fixed-seed LCG (deterministic across machines)
    std::vector<float> p(off, 0.0f);
    uint64_t s = 0x9E3779B97F4A7C15ull;
    auto uni = [&]() {
        s = s * 6364136223846793005ull + 1442695040888963407ull;
        return ((s >> 40) + 0.5) / 16777216.0;
    };
    for (int l = 0; l < NL; l++) {
        const double bound = std::sqrt(6.0 / (9.0 * CIN_R[l])) * (l == NL - 1 ? 0.1 : 1.0);
        for (size_t k = 0; k < layer_w_count(l); k++) p[n->poff[l] + k] = (float)((2 * uni() - 1) * bound);
    }
    // the clears and the upload run on the legacy stream; finish them before the
    // caller's streams (possibly non-blocking) use the buffers
    if (cudaMemcpy(n->d_master, p.data(), off * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaStreamSynchronize(cudaStreamLegacy) != cudaSuccess) {
        bm_net_destroy(n);
        return nfail(BM_ERR_CUDA, "bm_net_create: parameter upload failed");
    }
    *out = n;
    return BM_OK;
}

bm_status bm_net_destroy(bm_net* n)
{
    if (!n) return BM_OK;
    void* ptrs[] = {n->d_master, n->d_grad, n->d_m, n->d_v, n->d_in, n->d_out, n->d_loss, n->d_dy[0], n->d_dy[1],
                    n->d_err, n->d_bar, n->d_snap};
    for (void* q : ptrs)
        if (q) bmk::device_free(q);
    for (int l = 0; l < NL; l++) {
        if (n->d_wf[l]) bmk::device_free(n->d_wf[l]);
        if (n->d_wb[l]) bmk::device_free(n->d_wb[l]);
        if (l < NL - 1 && n->d_act[l]) bmk::device_free(n->d_act[l]);
    }
    delete n;
    return BM_OK;
}

bm_status bm_net_set_params(bm_net* n, const float* h_params, size_t count)
{
    if (!n || !h_params || count != n->nparam) return nfail(BM_ERR_INVALID, "bm_net_set_params: wrong parameter count");
    BN_CUDA(cudaMemcpy(n->d_master, h_params, count * 4, cudaMemcpyHostToDevice));
    BN_CUDA(cudaMemset(n->d_m, 0, count * 4));
    BN_CUDA(cudaMemset(n->d_v, 0, count * 4));
    BN_CUDA(cudaStreamSynchronize(cudaStreamLegacy));  // see bm_net_create
    n->step = 0;
    n->packed = false;
    return BM_OK;
}

bm_status bm_net_get_params(bm_net* n, float* h_params, size_t count)
{
    if (!n || !h_params || count != n->nparam) return nfail(BM_ERR_INVALID, "bm_net_get_params: wrong parameter count");
    BN_CUDA(cudaMemcpy(h_params, n->d_master, count * 4, cudaMemcpyDeviceToHost));
    return BM_OK;
}

// Training state (master parameters, Adam moments, step count) copied into snapshot
// slot 0 or 1 on `stream`, and copied back by bm_net_restore: a training loop rolls
// back to a validated snapshot when the loss spikes instead of continuing from a
// collapsed network.
bm_status bm_net_snapshot(bm_net* n, uint32_t slot, void* stream)
{
    if (!n || slot > 1) return nfail(BM_ERR_INVALID, "bm_net_snapshot: null network or slot not 0 or 1");
    const size_t np = n->nparam;
    if (!n->d_snap && bmk::device_malloc((void**)&n->d_snap, 6 * np * sizeof(float)) != cudaSuccess) {
        n->d_snap = nullptr;
        return nfail(BM_ERR_NOMEM, "bm_net_snapshot: allocation failed");
    }
    float* dst = n->d_snap + 3 * np * slot;
    cudaStream_t st = (cudaStream_t)stream;
    BN_CUDA(cudaMemcpyAsync(dst, n->d_master, np * 4, cudaMemcpyDeviceToDevice, st));
    BN_CUDA(cudaMemcpyAsync(dst + np, n->d_m, np * 4, cudaMemcpyDeviceToDevice, st));
    BN_CUDA(cudaMemcpyAsync(dst + 2 * np, n->d_v, np * 4, cudaMemcpyDeviceToDevice, st));
    n->snap_step[slot] = n->step;
    n->has_snap[slot] = true;
    return BM_OK;
}

bm_status bm_net_restore(bm_net* n, uint32_t slot, void* stream)
{
    if (!n || slot > 1) return nfail(BM_ERR_INVALID, "bm_net_restore: null network or slot not 0 or 1");
    if (!n->has_snap[slot]) return nfail(BM_ERR_STATE, "bm_net_restore: no snapshot in this slot");
    const size_t np = n->nparam;
    const float* src = n->d_snap + 3 * np * slot;
    cudaStream_t st = (cudaStream_t)stream;
    BN_CUDA(cudaMemcpyAsync(n->d_master, src, np * 4, cudaMemcpyDeviceToDevice, st));
    BN_CUDA(cudaMemcpyAsync(n->d_m, src + np, np * 4, cudaMemcpyDeviceToDevice, st));
    BN_CUDA(cudaMemcpyAsync(n->d_v, src + 2 * np, np * 4, cudaMemcpyDeviceToDevice, st));
    n->step = n->snap_step[slot];
    n->packed = false;   // the BF16 layouts are rebuilt from the restored parameters
    return BM_OK;
}

// Network input of image b from two 8-bit frames W x H (device), reduced by `reduce`.
bm_status bm_net_prepare_reduced(bm_net* n, uint32_t b, const uint8_t* d_f0, const uint8_t* d_f1, uint32_t W,
                                 uint32_t H, uint32_t reduce, void* stream)
{
    if (!n || !d_f0 || !d_f1) return nfail(BM_ERR_INVALID, "bm_net_prepare: null argument");
    if (reduce != 1 && reduce != 2 && reduce != 4) return nfail(BM_ERR_INVALID, "bm_net_prepare: reduce must be 1, 2 or 4");
    const uint32_t w4 = W / reduce / 4, h4 = H / reduce / 4;
    if (b >= n->maxB || (size_t)w4 * h4 > (size_t)n->maxh * n->maxw || w4 == 0 || h4 == 0)
        return nfail(BM_ERR_LIMIT, "bm_net_prepare: beyond the network's buffers");
    dim3 blk(32, 8), g((w4 + 31) / 32, (h4 + 7) / 8);
    __nv_bfloat16* dst = n->d_in + (size_t)b * h4 * w4 * NIN;
    if (reduce == 1)
        k_net_input<<<g, blk, 0, (cudaStream_t)stream>>>(d_f0, d_f1, (int)W, (int)H, dst, (int)w4, (int)h4);
    else
        k_net_input_reduced<<<g, blk, 0, (cudaStream_t)stream>>>(d_f0, d_f1, (int)W, dst, (int)w4, (int)h4, (int)reduce,
                                                                  reduce == 2 ? 1 : 2);
    BN_CUDA(cudaGetLastError());
    return BM_OK;
}

bm_status bm_net_prepare(bm_net* n, uint32_t b, const uint8_t* d_f0, const uint8_t* d_f1, uint32_t W, uint32_t H,
                         void* stream)
{
    return bm_net_prepare_reduced(n, b, d_f0, d_f1, W, H, 1, stream);
}

// Raw network input (bf16 NHWC, 32 channels) for tests.
bm_status bm_net_set_input(bm_net* n, const uint16_t* d_in, uint32_t B, uint32_t h, uint32_t w, void* stream)
{
    if (!n || !d_in) return nfail(BM_ERR_INVALID, "bm_net_set_input: null");
    bm_status s = check_dims(n, B, h, w);
    if (s != BM_OK) return s;
    BN_CUDA(cudaMemcpyAsync(n->d_in, d_in, (size_t)B * h * w * NIN * 2, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
    return BM_OK;
}

bm_status bm_net_set_umma(bm_net* n, int mode)
{
    if (!n) return nfail(BM_ERR_INVALID, "bm_net_set_umma: null");
    if (mode < 0 || mode > 2) return nfail(BM_ERR_INVALID, "bm_net_set_umma: mode is 0, 1 or 2");
    if (mode == 0) {
        n->umma = false;
        n->fused = false;
        return BM_OK;
    }
    if (mode == 2 && n->fused_grid_max <= 0)
        return nfail(BM_ERR_CUDA, "bm_net_set_umma: no cooperative launch of the fused network on this device");
    bool ok = true;
    for (int l = 0; ok && l < NL; l++) ok = weight_map(&n->map_wf[l], n->d_wf[l], COUT_P[l]);
    for (int l = 1; ok && l < NL - 1; l++) ok = weight_map(&n->map_wb[l], n->d_wb[l], CIN_P[l]);
    if (!ok) return nfail(BM_ERR_CUDA, "bm_net_set_umma: tensor map encoding unavailable");
    n->umma = true;
    n->fused = mode == 2;
    n->map_B = n->map_h = n->map_w = 0;
    return BM_OK;
}

int bm_net_umma(const bm_net* n) { return !n || !n->umma ? 0 : n->fused ? 2 : 1; }

int bm_net_fused_ctas(const bm_net* n) { return n ? n->fused_grid_max : 0; }

bm_status bm_net_check(bm_net* n, void* stream)
{
    if (!n) return nfail(BM_ERR_INVALID, "bm_net_check: null");
    int h = 0;
    BN_CUDA(cudaMemcpyAsync(&h, n->d_err, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream));
    BN_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
    if (h) {
        BN_CUDA(cudaMemsetAsync(n->d_err, 0, sizeof(int), (cudaStream_t)stream));
        BN_CUDA(cudaStreamSynchronize((cudaStream_t)stream));
        return nfail(BM_ERR_TIMEOUT, h == 1   ? "bm_net: a tensor-core layer's copies did not arrive in time"
                                     : h == 2 ? "bm_net: a tensor-core layer's MMA did not complete in time"
                                              : "bm_net: the fused network's grid barrier gave up");
    }
    return BM_OK;
}

bm_status bm_net_forward(bm_net* n, uint32_t B, uint32_t h, uint32_t w, float* d_out, void* stream)
{
    if (!n) return nfail(BM_ERR_INVALID, "bm_net_forward: null");
    bm_status s = check_dims(n, B, h, w);
    if (s != BM_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    s = forward(n, B, h, w, st);
    if (s != BM_OK) return s;
    if (d_out) BN_CUDA(cudaMemcpyAsync(d_out, n->d_out, (size_t)B * h * w * 3 * 4, cudaMemcpyDeviceToDevice, st));
    return BM_OK;
}

// Forward, loss against d_target ([B][h][w][3]: u, v in quarter-resolution pixels and
// a validity weight), backward into the FP32 gradient (d_grad_out, optional copy),
// and -- when lr > 0 -- one Adam step.  h_loss receives (flow loss, confidence loss,
// fraction of confident labels).
bm_status bm_net_train_step(bm_net* n, uint32_t B, uint32_t h, uint32_t w, const float* d_target, float lr,
                            float* d_grad_out, float* h_loss, void* stream)
{
    if (!n || !d_target) return nfail(BM_ERR_INVALID, "bm_net_train_step: null");
    bm_status s = check_dims(n, B, h, w);
    if (s != BM_OK) return s;
    cudaStream_t st = (cudaStream_t)stream;
    s = forward(n, B, h, w, st);
    if (s != BM_OK) return s;
    const size_t px = (size_t)B * h * w;
    const int Bi = (int)B, hi = (int)h, wi = (int)w;
    BN_CUDA(cudaMemsetAsync(n->d_grad, 0, n->nparam * 4, st));
    BN_CUDA(cudaMemsetAsync(n->d_loss, 0, 4 * 4, st));
    k_net_loss<<<(unsigned)((px + 255) / 256), 256, 0, st>>>(n->d_out, d_target, px, n->d_dy[0], 1.0f / (float)px, 1.0f,
                                                             0.25f, n->d_loss);
    BN_CUDA(cudaGetLastError());
    // layer 5: dY (16 padded channels, 3 real) -> dW5, and dX into the ReLU mask of act[4]
    float* g = n->d_grad;
    BN_CUDA((launch_wgrad<32, 16, 1>(n->d_act[4], n->d_dy[0], 16, Bi, hi, wi, g + n->poff[5],
                                     g + n->poff[5] + layer_w_count(5), 32, 3, st)));
    BN_CUDA((launch_conv<16, 32, EPI_MASK_BF16, 1>(n->d_dy[0], n->d_wb[5], nullptr, n->d_act[4], n->d_dy[1], Bi, hi, wi,
                                                   32, 32, st)));
    int cur = 1;
    for (int l = 4; l >= 1; l--) {
        BN_CUDA(conv_wgrad(l, n->d_act[l - 1], n->d_dy[cur], Bi, hi, wi, g + n->poff[l], g + n->poff[l] + layer_w_count(l),
                           st));
        if (n->umma)
            BN_CUDA((launch_conv_umma<EPI_MASK_BF16, 32>(n->map_dy[cur], n->map_wb[l], nullptr, n->d_act[l - 1],
                                                          n->d_dy[cur ^ 1], Bi, hi, wi, DIL[l], 32, 32, n->d_err, st)));
        else
            BN_CUDA(conv_bwd_data(l, n->d_dy[cur], n->d_wb[l], n->d_act[l - 1], n->d_dy[cur ^ 1], Bi, hi, wi, st));
        cur ^= 1;
    }
    BN_CUDA(conv_wgrad(0, n->d_in, n->d_dy[cur], Bi, hi, wi, g + n->poff[0], g + n->poff[0] + layer_w_count(0), st));
    if (d_grad_out) BN_CUDA(cudaMemcpyAsync(d_grad_out, g, n->nparam * 4, cudaMemcpyDeviceToDevice, st));
    if (lr > 0) {
        n->step++;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.0f / (1.0f - std::pow(b1, (float)n->step)), c2 = 1.0f / (1.0f - std::pow(b2, (float)n->step));
        k_adam<<<(unsigned)((n->nparam + 255) / 256), 256, 0, st>>>(n->d_master, g, n->d_m, n->d_v, n->nparam, lr, b1, b2,
                                                                    1e-8f, c1, c2, 0.0f);
        BN_CUDA(cudaGetLastError());
        s = pack_weights(n, st);
        if (s != BM_OK) return s;
    }
    if (h_loss) {
        BN_CUDA(cudaMemcpyAsync(h_loss, n->d_loss, 3 * 4, cudaMemcpyDeviceToHost, st));
        BN_CUDA(cudaStreamSynchronize(st));
    }
    return BM_OK;
}

}  // extern "C"

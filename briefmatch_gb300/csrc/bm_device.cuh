// bm_device.cuh -- device code shared by the single-pair kernels (bm_kernels.cu)
// and the batched kernels (bm_batch.cu): per-pixel and per-block bodies of every
// stage, so both launch paths run the same arithmetic.  Included only by units
// compiled with -use_fast_math (the reference's flags, CMakeLists.txt:50).
#pragma once

#include <curand_kernel.h>
#include <type_traits>

#include "bm_internal.h"

namespace bmk {
namespace dev {

// util_cuda.h:61
#define BM_PI 3.141592653589793115997963468544

constexpr int TX = 32;  // block width: one warp per row of a tile
constexpr int TY = 8;   // block height

__device__ __forceinline__ int lo16(uint32_t w) { return (int)(int16_t)(w & 0xffffu); }
__device__ __forceinline__ int hi16(uint32_t w) { return (int)(int16_t)(w >> 16); }

template <int NSP>
__device__ __forceinline__ void store_desc(uint32_t* dst, const uint32_t (&w)[NSP])
{
    if constexpr (NSP >= 4) {
#pragma unroll
        for (int k = 0; k < NSP / 4; k++)
            reinterpret_cast<uint4*>(dst)[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
    } else if constexpr (NSP == 2) {
        *reinterpret_cast<uint2*>(dst) = make_uint2(w[0], w[1]);
    } else {
        dst[0] = w[0];
    }
}

template <int NSP>
__device__ __forceinline__ void load_desc(uint32_t (&w)[NSP], const uint32_t* __restrict__ src)
{
    if constexpr (NSP >= 4) {
#pragma unroll
        for (int k = 0; k < NSP / 4; k++) {
            uint4 v = __ldg(reinterpret_cast<const uint4*>(src) + k);
            w[4 * k] = v.x;
            w[4 * k + 1] = v.y;
            w[4 * k + 2] = v.z;
            w[4 * k + 3] = v.w;
        }
    } else if constexpr (NSP == 2) {
        uint2 v = __ldg(reinterpret_cast<const uint2*>(src));
        w[0] = v.x;
        w[1] = v.y;
    } else {
        w[0] = __ldg(src);
    }
}

template <int NSP>
__device__ __forceinline__ int hamming(const uint32_t (&a)[NSP], const uint32_t* __restrict__ pb)
{
    uint32_t b[NSP];
    load_desc<NSP>(b, pb);
    int h = 0;
#pragma unroll
    for (int k = 0; k < NSP; k++) h += __popc(a[k] ^ b[k]);
    return h;
}

__device__ __forceinline__ void rs_normals(const RsArgs& rs, unsigned int id, float& n1, float& n2)
{
    if (rs.mode == BM_RNG_PHILOX) {
        curandStatePhilox4_32_10_t st;
        curand_init(rs.seed, (unsigned long long)id, 2ull * rs.call, &st);
        float2 v = curand_normal2(&st);
        n1 = v.x;
        n2 = v.y;
    } else {
        // The reference state: curand_init(id, 0, 0) (briefmatch_cuda.cu:57) advanced by
        // two uniforms per earlier call (two curand_normal per call, :240-241).
        curandStateXORWOW_t st;
        curand_init((unsigned long long)id, 0ull, 0ull, &st);
        unsigned long long skip = 2ull * rs.call;
        if (skip <= 512ull) {
            for (unsigned long long k = 0; k < skip; k++) (void)curand(&st);
        } else {
            skipahead(skip, &st);
        }
        n1 = curand_normal(&st);
        n2 = curand_normal(&st);
    }
}

// Descriptor loads for the own pixel: read once per level and never again, so
// they are marked evict-first to leave L2 to the gathered descriptors.
template <int NSP>
__device__ __forceinline__ void load_desc_stream(uint32_t (&w)[NSP], const uint32_t* __restrict__ src)
{
    if constexpr (NSP >= 4) {
#pragma unroll
        for (int k = 0; k < NSP / 4; k++) {
            uint4 v = __ldcs(reinterpret_cast<const uint4*>(src) + k);
            w[4 * k] = v.x;
            w[4 * k + 1] = v.y;
            w[4 * k + 2] = v.z;
            w[4 * k + 3] = v.w;
        }
    } else if constexpr (NSP == 2) {
        uint2 v = __ldcs(reinterpret_cast<const uint2*>(src));
        w[0] = v.x;
        w[1] = v.y;
    } else {
        w[0] = __ldcs(src);
    }
}

// Descriptor gather that is issued only when `pred` holds (the words stay zero
// otherwise); written as predicated PTX loads so that several gathers of one
// thread are in flight together instead of waiting behind each other's branches.
template <int NSP>
__device__ __forceinline__ void gather_desc_pred(uint32_t (&w)[NSP], const uint32_t* __restrict__ src, bool pred)
{
    const int pr = pred ? 1 : 0;
#pragma unroll
    for (int k = 0; k < NSP; k++) w[k] = 0;
    if constexpr (NSP >= 4) {
#pragma unroll
        for (int k = 0; k < NSP / 4; k++)
            asm("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t@p ld.global.nc.v4.u32 {%0, %1, %2, %3}, [%5];\n\t}"
                : "+r"(w[4 * k]), "+r"(w[4 * k + 1]), "+r"(w[4 * k + 2]), "+r"(w[4 * k + 3])
                : "r"(pr), "l"(src + 4 * k));
    } else if constexpr (NSP == 2) {
        asm("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %2, 0;\n\t@p ld.global.nc.v2.u32 {%0, %1}, [%3];\n\t}"
            : "+r"(w[0]), "+r"(w[1])
            : "r"(pr), "l"(src));
    } else {
        asm("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %1, 0;\n\t@p ld.global.nc.u32 %0, [%2];\n\t}"
            : "+r"(w[0])
            : "r"(pr), "l"(src));
    }
}

typedef unsigned long long f2x;  // two packed floats (low = first)

__device__ __forceinline__ f2x pk2(float a, float b) { f2x r; asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b)); return r; }
__device__ __forceinline__ float lo2(f2x v) { return __uint_as_float((unsigned int)(v & 0xffffffffull)); }
__device__ __forceinline__ float hi2(f2x v) { return __uint_as_float((unsigned int)(v >> 32)); }
__device__ __forceinline__ f2x add2(f2x a, f2x b) { f2x d; asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }
__device__ __forceinline__ f2x sub2(f2x a, f2x b) { f2x d; asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }
__device__ __forceinline__ f2x mul2(f2x a, f2x b) { f2x d; asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b)); return d; }
__device__ __forceinline__ f2x fma2(f2x a, f2x b, f2x c)
{
    f2x d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ f2x ex2_2(f2x a) { return pk2(exp2f(lo2(a)), exp2f(hi2(a))); }


// ---------------------------------------------------------------------------
// Lanczos-3 up-sampling (util_cuda.cu:126-158): output pixel (x, y).  The weights
// are tabulated per output column/row with the reference's expression; the 6x6
// accumulation runs in the reference's order (i outer, j inner).
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ float upsample_val(const T* __restrict__ in, int sxi, int syi,
                                              const float* __restrict__ lx, const int* __restrict__ ix,
                                              const float* __restrict__ ly, const int* __restrict__ iy, int x, int y)
{
    int x1 = ix[x], y1 = iy[y];
    float Ly[6];
    int row[6];
#pragma unroll
    for (int b = 0; b < 6; b++) {
        Ly[b] = ly[y * 6 + b];
        row[b] = min(syi - 1, max(0, y1 - 2 + b)) * sxi;
    }
    float v = 0.0f, w = 0.0f;
#pragma unroll
    for (int a = 0; a < 6; a++) {
        float Lx = lx[x * 6 + a];
        int ci = min(sxi - 1, max(0, x1 - 2 + a));
#pragma unroll
        for (int b = 0; b < 6; b++) {
            w += Lx * Ly[b];
            v += float(in[ci + row[b]]) * Lx * Ly[b];
        }
    }
    return v / w;
}

template <typename T>
__device__ __forceinline__ void upsample_px(const T* __restrict__ in, float* __restrict__ out, int sxi, int syi,
                                            int sxo, const float* __restrict__ lx, const int* __restrict__ ix,
                                            const float* __restrict__ ly, const int* __restrict__ iy, int x, int y)
{
    out[x + (size_t)y * sxo] = upsample_val<T>(in, sxi, syi, lx, ix, ly, iy, x, y);
}

// ---------------------------------------------------------------------------
// BRIEF descriptors (briefmatch_cuda.cu:82-124).
// Interior pixels (at least rmax from every border, rmax = the largest |offset|)
// read the image at the precomputed linear offsets `off` with no clamping -- the
// reference's clamped reads give the same addresses there; samples past N carry
// offset 0 and give 0 bits.  Border pixels clamp each coordinate as the reference.
// A warp reads 32 consecutive pixels at one offset: one coalesced L1 request.
// ---------------------------------------------------------------------------
template <int NSP, typename OffArray>
__device__ __forceinline__ void features_interior_px(const float* __restrict__ I, uint32_t* __restrict__ F, int sx,
                                                     int x, int y, const OffArray& off)
{
    const float* base = I + (size_t)y * sx + x;
    uint32_t word[NSP];
#pragma unroll
    for (int wd = 0; wd < NSP; wd++) {
        uint32_t acc = 0;
#pragma unroll
        for (int b = 0; b < 32; b++) {
            const int2 o = off[wd * 32 + b];
            const float i1 = __ldg(base + o.x);
            const float i2 = __ldg(base + o.y);
            if (i1 > i2) acc |= 1u << b;
        }
        word[wd] = acc;
    }
    store_desc<NSP>(F + ((size_t)y * sx + x) * NSP, word);
}

// A strip of PX pixels at x, x+TX, ..., x+(PX-1)*TX of one row, in an image whose
// every sample point of those pixels is addressable (an edge-replicated margin at
// least as wide as the largest offset: the reads then equal the reference's
// per-coordinate clamped reads).  `base` points at pixel x, `room` = sx - x; the
// strip's pixels share each offset's address arithmetic (the others are immediate
// displacements of TX pixels).
template <int NSP, int PX, typename OffArray>
__device__ __forceinline__ void features_strip_px(const float* __restrict__ base, uint32_t* __restrict__ F, int room,
                                                  const OffArray& off)
{
    uint32_t word[PX][NSP];
#pragma unroll
    for (int wd = 0; wd < NSP; wd++) {
        uint32_t acc[PX];
#pragma unroll
        for (int k = 0; k < PX; k++) acc[k] = 0;
#pragma unroll
        for (int b = 0; b < 32; b++) {
            const int2 o = off[wd * 32 + b];
            const float* p1 = base + o.x;
            const float* p2 = base + o.y;
#pragma unroll
            for (int k = 0; k < PX; k++) {
                if (k == 0 || k * TX < room) {
                    const float i1 = __ldg(p1 + k * TX);
                    const float i2 = __ldg(p2 + k * TX);
                    if (i1 > i2) acc[k] |= 1u << b;
                }
            }
        }
#pragma unroll
        for (int k = 0; k < PX; k++) word[k][wd] = acc[k];
    }
#pragma unroll
    for (int k = 0; k < PX; k++)
        if (k == 0 || k * TX < room) store_desc<NSP>(F + (size_t)k * TX * NSP, word[k]);
}

template <int NSP>
__device__ __forceinline__ void features_border_px(const float* __restrict__ I, uint32_t* __restrict__ F, int sx,
                                                   int sy, int N, const int4* __restrict__ s_pat, int x, int y)
{
    const float* base = I + (size_t)y * sx + x;
    uint32_t word[NSP];
#pragma unroll
    for (int wd = 0; wd < NSP; wd++) {
        const int s0 = wd * 32;
        const int cnt = min(32, N - s0);
        uint32_t acc = 0;
#pragma unroll 4
        for (int b = 0; b < cnt; b++) {
            int4 q = s_pat[s0 + b];
            int ox1 = max(-x, min(sx - x - 1, q.x));
            int oy1 = max(-y, min(sy - y - 1, q.y));
            int ox2 = max(-x, min(sx - x - 1, q.z));
            int oy2 = max(-y, min(sy - y - 1, q.w));
            float i1 = __ldg(base + ox1 + (long)oy1 * sx);
            float i2 = __ldg(base + ox2 + (long)oy2 * sx);
            acc |= (i1 > i2 ? 1u : 0u) << b;
        }
        word[wd] = acc;
    }
    store_desc<NSP>(F + ((size_t)y * sx + x) * NSP, word);
}

// True when every pixel of the TX x TY tile at (bx, by) lies rmax or more inside.
__device__ __forceinline__ bool tile_interior(int bx, int by, int sx, int sy, int rmax)
{
    return (bx - rmax >= 0) && (bx + TX - 1 + rmax < sx) && (by - rmax >= 0) && (by + TY - 1 + rmax < sy);
}

// ---------------------------------------------------------------------------
// PatchMatch (briefmatch_cuda.cu:126-246).
// ---------------------------------------------------------------------------
// Zero or temporal initialisation (briefmatch_cuda.cu:149-184); temporal init reads
// the previous field from flow_prev (a snapshot) and writes flow_out.
template <int NSP>
__device__ __forceinline__ void init_px(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                        const uint32_t* __restrict__ flow_prev, uint32_t* __restrict__ flow_out,
                                        uint16_t* __restrict__ cost, int sx, int sy, int first, int x, int y)
{
    const long n = (long)sx * sy;
    const long pix = x + (long)y * sx;
    int nx = 0, ny = 0;
    if (!first) {
        uint32_t own = flow_prev[pix];
        long q = pix + lo16(own) + (long)hi16(own) * sx;
        uint32_t t = (q >= 0 && q < n) ? flow_prev[q] : 0u;
        nx = min(max(lo16(t), -x), sx - x - 1);
        ny = min(max(hi16(t), -y), sy - y - 1);
    }
    uint32_t f1[NSP];
    load_desc<NSP>(f1, F1 + pix * NSP);
    cost[pix] = (uint16_t)hamming<NSP>(f1, F2 + (pix + nx + (long)ny * sx) * NSP);
    flow_out[pix] = pack_flow(nx, ny);
}

// Seeded initialisation: first the plain initialisation (zero vector, or the
// temporal candidate when !first, exactly as init_px), then the network's proposal
// for this pixel -- pred is [h4][w4][3] (u, v in quarter-resolution input pixels,
// confidence logit) -- where its confidence logit reaches logit_min; the proposal
// replaces the plain vector only if its Hamming cost is strictly lower.
template <int NSP>
__device__ __forceinline__ void seed_px(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                        const uint32_t* __restrict__ flow_prev, uint32_t* __restrict__ flow_out,
                                        uint16_t* __restrict__ cost, int sx, int sy, int first, int x, int y,
                                        const float* __restrict__ pred, int w4, int h4, float scale_x, float scale_y,
                                        float inv_x, float inv_y, float logit_min)
{
    const long n = (long)sx * sy;
    const long pix = x + (long)y * sx;
    int nx = 0, ny = 0;
    if (!first) {
        uint32_t own = flow_prev[pix];
        long q = pix + lo16(own) + (long)hi16(own) * sx;
        uint32_t t = (q >= 0 && q < n) ? flow_prev[q] : 0u;
        nx = min(max(lo16(t), -x), sx - x - 1);
        ny = min(max(hi16(t), -y), sy - y - 1);
    }
    uint32_t f1[NSP];
    load_desc<NSP>(f1, F1 + pix * NSP);
    int h = hamming<NSP>(f1, F2 + (pix + nx + (long)ny * sx) * NSP);
    // quarter-resolution cell of this up-sampled pixel (scale = up-sampled px per
    // quarter-resolution px, inv = its reciprocal from the host, so the cell index
    // is one IEEE add and multiply: no approximate division)
    const int qx = min(w4 - 1, max(0, (int)((x + 0.5f) * inv_x)));
    const int qy = min(h4 - 1, max(0, (int)((y + 0.5f) * inv_y)));
    const float* pr = pred + ((size_t)qy * w4 + qx) * 3;
    if (pr[2] >= logit_min) {
        const int sxv = min(max(__float2int_rn(pr[0] * scale_x), -x), sx - x - 1);
        const int syv = min(max(__float2int_rn(pr[1] * scale_y), -y), sy - y - 1);
        if (sxv != nx || syv != ny) {
            const int hs = hamming<NSP>(f1, F2 + (pix + sxv + (long)syv * sx) * NSP);
            if (hs < h) {
                h = hs;
                nx = sxv;
                ny = syv;
            }
        }
    }
    cost[pix] = (uint16_t)h;
    flow_out[pix] = pack_flow(nx, ny);
}

// One jump-flood level at step p (briefmatch_cuda.cu:206-219) for pixel (x, y).
// Neighbours are read from flow_in (the previous level's field) and the result is
// written to flow_out, so the outcome does not depend on the schedule.  All
// neighbour reads are issued together, then all candidate descriptors are gathered
// together, and only then are the candidates accepted in the reference's order
// (d = -1, +1; vertical then horizontal; strictly lower cost wins, insert()
// :126-147).  Candidates equal to the current vector (the reference's own skip) or
// to an earlier candidate cannot change a decision, so their gathers are elided.
// With RS the iteration's random-search candidate (:237-243) is evaluated last; it
// reads only this pixel's own state, so fusing it into the last level gives the
// reference's result.
// INLAUNCH: the field and cost were written by an earlier phase of the same launch
// (the persistent batched kernel); they are then read through L2 (ld.global.cg),
// never through the non-coherent read-only path.
template <bool INLAUNCH>
__device__ __forceinline__ uint32_t field_load(const uint32_t* p)
{
    if constexpr (INLAUNCH)
        return __ldcg(p);
    else
        return __ldg(p);
}

template <int NSP, bool RS, bool INLAUNCH = false>
__device__ __forceinline__ void jump_px(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                        const uint32_t* flow_in, uint32_t* flow_out, uint16_t* cost, int sx, int sy,
                                        int p, int pd, int doubleProp, const RsArgs& rs, int x, int y)
{
    constexpr int NC = RS ? 5 : 4;
    const long n = (long)sx * sy;
    const long pix = x + (long)y * sx;
    const uint32_t own = field_load<INLAUNCH>(flow_in + pix);
    const int h0 = INLAUNCH ? (int)__ldcg(cost + pix) : (int)cost[pix];

    uint32_t cand[NC];
    bool live[NC];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int d = (c < 2) ? -1 : 1;
        const int xy = c & 1;
        const bool active = d > 0 || doubleProp;
        const long doff = xy ? (long)pd * p * d : (long)sx * pd * p * d;
        const long q = pix + doff;
        const uint32_t nb = (active && q >= 0 && q < n) ? field_load<INLAUNCH>(flow_in + q) : 0u;
        const int nx = min(max(lo16(nb), -x), sx - x - 1);
        const int ny = min(max(hi16(nb), -y), sy - y - 1);
        cand[c] = pack_flow(nx, ny);
        live[c] = active;
    }
    if constexpr (RS) {
        float n1, n2;
        rs_normals(rs, (unsigned int)pix, n1, n2);
        const int nx = min(max((int)round(rs.dist * n1), -x), sx - x - 1);
        const int ny = min(max((int)round(rs.dist * n2), -y), sy - y - 1);
        cand[NC - 1] = pack_flow(nx, ny);
        live[NC - 1] = true;
    }
#pragma unroll
    for (int c = 0; c < NC; c++) {
        bool dup = cand[c] == own;
#pragma unroll
        for (int k = 0; k < c; k++) dup = dup || (live[k] && cand[k] == cand[c]);
        live[c] = live[c] && !dup;
    }

    uint32_t f1[NSP];
    load_desc_stream<NSP>(f1, F1 + pix * NSP);
    // predicated gathers, all in flight at once
    uint32_t g[NC][NSP];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        const long t = pix + lo16(cand[c]) + (long)hi16(cand[c]) * sx;
        gather_desc_pred<NSP>(g[c], F2 + t * NSP, live[c]);
    }
    int hc[NC];
#pragma unroll
    for (int c = 0; c < NC; c++) {
        int acc = 0;
#pragma unroll
        for (int k = 0; k < NSP; k++) acc += __popc(f1[k] ^ g[c][k]);
        hc[c] = live[c] ? acc : 0x7fffffff;
    }
    int h = h0;
    uint32_t best = own;
#pragma unroll
    for (int c = 0; c < NC; c++)
        if (hc[c] < h) {
            h = hc[c];
            best = cand[c];
        }
    flow_out[pix] = best;
    if (h != h0) cost[pix] = (uint16_t)h;
}

// Local refinement step of the seeded schedule (no reference counterpart): the
// pixel's own vector moved by r up-sampled pixels left, right, up and down (clamped
// into the image), in that order, each kept only when strictly cheaper than the
// best so far.  Reads flow_in (a snapshot) and writes flow_out, like a jump level.
template <int NSP>
__device__ __forceinline__ void local_px(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                         const uint32_t* __restrict__ flow_in, uint32_t* __restrict__ flow_out,
                                         uint16_t* __restrict__ cost, int sx, int sy, int r, int x, int y)
{
    const long pix = x + (long)y * sx;
    const uint32_t own = __ldg(flow_in + pix);
    const int h0 = (int)cost[pix];
    const int ox = lo16(own), oy = hi16(own);
    uint32_t cand[4];
    bool live[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int dx = c == 0 ? -r : (c == 1 ? r : 0);
        const int dy = c == 2 ? -r : (c == 3 ? r : 0);
        const int nx = min(max(ox + dx, -x), sx - x - 1);
        const int ny = min(max(oy + dy, -y), sy - y - 1);
        cand[c] = pack_flow(nx, ny);
        bool dup = cand[c] == own;
#pragma unroll
        for (int k = 0; k < c; k++) dup = dup || cand[k] == cand[c];
        live[c] = !dup;
    }
    uint32_t f1[NSP];
    load_desc_stream<NSP>(f1, F1 + pix * NSP);
    uint32_t g[4][NSP];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const long t = pix + lo16(cand[c]) + (long)hi16(cand[c]) * sx;
        gather_desc_pred<NSP>(g[c], F2 + t * NSP, live[c]);
    }
    int h = h0;
    uint32_t best = own;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        int acc = 0;
#pragma unroll
        for (int k = 0; k < NSP; k++) acc += __popc(f1[k] ^ g[c][k]);
        if (live[c] && acc < h) {
            h = acc;
            best = cand[c];
        }
    }
    flow_out[pix] = best;
    if (h != h0) cost[pix] = (uint16_t)h;
}

// ---------------------------------------------------------------------------
// Down-sampling (briefmatch.cpp:296-324) for input-resolution pixel (x, y):
// int16 -> float, Gaussian H then V evaluated only where the nearest-neighbour
// decimation samples (source index tables nnx/nny), scaled by (mx, my).  Each
// pass keeps the reference's float rounding and fused multiply-adds.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void downsample_px(const uint32_t* __restrict__ flow, float* __restrict__ U,
                                              float* __restrict__ V, int sx, int sy, int sx_in,
                                              const float* __restrict__ taps, int P, float mx, float my,
                                              const unsigned int* __restrict__ nnx, const unsigned int* __restrict__ nny,
                                              int x, int y)
{
    const unsigned int x1 = nnx[x], y1 = nny[y];
    const size_t o = (size_t)x + (size_t)y * sx_in;
    if (x1 >= (unsigned)sx || y1 >= (unsigned)sy) {
        U[o] = 0.0f;
        V[o] = 0.0f;
        return;
    }
    const int ks2 = P / 2;
    float su = 0, sv = 0;
    for (int i = 0; i < P; i++) {
        const int yy = min(sy - 1, max(0, (int)y1 + i - ks2));
        const uint32_t* row = flow + (size_t)yy * sx;
        float hu = 0, hv = 0;
        for (int k = 0; k < P; k++) {
            const uint32_t f = __ldg(row + min(sx - 1, max(0, (int)x1 + k - ks2)));
            const float tk = taps[k];
            hu += tk * float(lo16(f));
            hv += tk * float(hi16(f));
        }
        su += taps[i] * hu;
        sv += taps[i] * hv;
    }
    U[o] = su * mx;
    V[o] = sv * my;
}

// ---------------------------------------------------------------------------
// 1-D median (util_cuda.cu:75-111) of the two outputs at linear indices p and
// p + step (the second only when `second`): each window is fsize samples at linear
// offsets -ks .. fsize-1-ks (ks = fsize/2), guard 0 outside the plane, and the median
// is the (ks+1)-th smallest.  The two windows share the fsize-1 samples S between
// them; with a the first output's own sample and b the second's, the (ks+1)-th
// smallest of S + {a} is min(max(a, S(ks-1)), S(ks)), S(i) the (i+1)-th smallest of
// S, so one partial selection (positions 0..ks, in registers padded with +inf up to
// FS-1) serves both outputs.
// ---------------------------------------------------------------------------
template <int FS>
__device__ __forceinline__ void median2_px(const float* __restrict__ in, float* __restrict__ out, long p, long step,
                                           long n, int fsize, bool second)
{
    const int ks = fsize / 2;
    auto sample = [&](long idx) { return (idx >= 0 && idx < n) ? __ldg(in + idx) : 0.0f; };
    const float a = sample(p - (long)ks * step);
    const float b = second ? sample(p + (long)(fsize - ks) * step) : 0.0f;
    if (fsize == 1) {
        out[p] = a;
        if (second) out[p + step] = b;
        return;
    }
    float v[FS - 1];
#pragma unroll
    for (int k = 0; k < FS - 1; k++)
        v[k] = (k < fsize - 1) ? sample(p + (long)(k - ks + 1) * step) : __int_as_float(0x7f800000);
#pragma unroll
    for (int i = 0; i < (FS + 1) / 2; i++) {
        if (i <= ks) {
#pragma unroll
            for (int j = i + 1; j < FS - 1; j++) {
                const float x = v[i], y = v[j];
                v[i] = fminf(x, y);
                v[j] = fmaxf(x, y);
            }
        }
    }
    float lo = v[0], hi = v[1];
#pragma unroll
    for (int i = 1; i < (FS + 1) / 2; i++)
        if (i == ks) {
            lo = v[i - 1];
            hi = v[i];
        }
    out[p] = fminf(fmaxf(a, lo), hi);
    if (second) out[p + step] = fminf(fmaxf(b, lo), hi);
}

// ---------------------------------------------------------------------------
// Cross-trilateral filter (briefmatch_cuda.cu:248-297), one block of TX x TRI_TY
// threads filtering the TX x TRI_BY outputs whose top-left pixel is (bx0, by0).
// Each thread owns four vertically adjacent outputs, held as two pairs in packed
// f32x2 registers, so every neighbourhood sample it reads from shared memory is
// used four times and every arithmetic instruction serves two outputs.  The
// (2s + TX) x (2s + TRI_BY) neighbourhood is staged in shared memory with
// clamp-to-edge addressing.  The three Gaussians are one exp2 of the summed
// exponents cE*(du^2 + dv^2) + cI*dI^2 + cS*j^2 = r*(du'^2 + dv'^2 + dI'^2 + j^2*cS/r)
// with du' = kE*u - kE*uc: kE is the power of two nearest sqrt(cE) (so kE*uc is
// exact and du' is the scaled difference rounded once -- a rounded centre would
// tilt every weight of the window the same way), r = cE/kE^2, kI = sqrt(cI/r).
// Each scaled difference is one FMA against the centre's negated scaled value, the
// squared terms accumulate by FMA onto the row term, one multiply by r, one exp2:
// seven FP32 operations per tap and output before the three accumulations.  The
// column factor exp2(-cS*i^2) is applied once per column (the inner loop runs down
// a column); row terms outside the window are +inf (weight 0).
// `smem` must hold tri_smem_bytes(s).
// ---------------------------------------------------------------------------
constexpr int TRI_R = 4;                // outputs per thread (two f32x2 pairs)
constexpr int TRI_TY = 8;               // thread rows per block
constexpr int TRI_BY = TRI_TY * TRI_R;  // output rows per block (32x32 outputs)

__host__ __device__ inline size_t tri_smem_bytes(int s)
{
    return (size_t)(2 * s + TRI_R - 1) * sizeof(float4) + (size_t)(TX + 2 * s) * (TRI_BY + 2 * s) * 3 * sizeof(float);
}

__device__ __forceinline__ f2x ex2n_2(f2x a) { return pk2(exp2f(-lo2(a)), exp2f(-hi2(a))); }

__device__ __forceinline__ void trilateral_block(const float* __restrict__ U, const float* __restrict__ V,
                                                 const float* __restrict__ Um, const float* __restrict__ Vm,
                                                 const float* __restrict__ I, float* __restrict__ Uo,
                                                 float* __restrict__ Vo, int sx, int sy, int s, float cE, float cI,
                                                 float cS, int bx0, int by0, float4* smem4)
{
    const int TW = TX + 2 * s, TH = TRI_BY + 2 * s;
    const int NR = 2 * s + TRI_R - 1;        // source rows a thread walks per column
    float4* rowf = smem4;                    // [NR] row terms j^2*cS for outputs r=0..3
    float2* suv = reinterpret_cast<float2*>(smem4 + NR);
    float* sI = reinterpret_cast<float*>(suv + TW * TH);
    const int x0 = bx0 - s, y0 = by0 - s;
    const int tid = threadIdx.y * TX + threadIdx.x;
    // kE: the power of two nearest sqrt(cE) (exact scaling), r_ the remaining factor
    const float kE = exp2f(rintf(0.5f * __log2f(cE))), r_ = cE / (kE * kE);
    const float kI = sqrtf(cI / r_), cS_r = cS / r_;
    for (int k = tid; k < TW * TH; k += TX * TRI_TY) {
        const int r = k / TW, c = k - r * TW;
        const int gx = min(sx - 1, max(0, x0 + c)), gy = min(sy - 1, max(0, y0 + r));
        const size_t g = (size_t)gx + (size_t)gy * sx;
        suv[k] = make_float2(__ldg(U + g), __ldg(V + g));
        sI[k] = __ldg(I + g);
    }
    for (int m = tid; m < NR; m += TX * TRI_TY) {
        float t[TRI_R];
#pragma unroll
        for (int r = 0; r < TRI_R; r++) {
            const int j = m - r - s;  // vertical offset of this source row for output r
            t[r] = (j >= -s && j < s) ? (float)(j * j) * cS_r : __int_as_float(0x7f800000);
        }
        rowf[m] = make_float4(t[0], t[1], t[2], t[3]);
    }
    __syncthreads();

    const int x = bx0 + threadIdx.x;
    const int yb = by0 + threadIdx.y * TRI_R;
    if (x >= sx || yb >= sy) return;
    float umc[TRI_R], vmc[TRI_R], Ic[TRI_R];
#pragma unroll
    for (int r = 0; r < TRI_R; r++) {
        const int yy = min(sy - 1, yb + r);
        const size_t o = (size_t)x + (size_t)yy * sx;
        umc[r] = -kE * __ldg(Um + o);
        vmc[r] = -kE * __ldg(Vm + o);
        Ic[r] = -kI * sI[(threadIdx.y * TRI_R + r + s) * TW + threadIdx.x + s];
    }
    const f2x umA = pk2(umc[0], umc[1]), umB = pk2(umc[2], umc[3]);
    const f2x vmA = pk2(vmc[0], vmc[1]), vmB = pk2(vmc[2], vmc[3]);
    const f2x IA = pk2(Ic[0], Ic[1]), IB = pk2(Ic[2], Ic[3]);
    const f2x kEE = pk2(kE, kE), kII = pk2(kI, kI), rr = pk2(r_, r_);
    f2x ufA = 0, ufB = 0, vfA = 0, vfB = 0, WA = 0, WB = 0;  // 0 bits = (0.0f, 0.0f)
    const int row0 = threadIdx.y * TRI_R;
    // NC source columns (i .. i + NC - 1) per step: NC times the independent
    // accumulation chains of a one-column walk, to keep the FMA pipe fed between the
    // exp2s (three columns with the row loop unrolled four times measured fastest;
    // the last 2s mod 3 columns go one at a time)
    auto columns = [&](int i, auto ncols) {
        constexpr int NC = decltype(ncols)::value;
        const float2* col = suv + row0 * TW + threadIdx.x + s + i;
        const float* colI = sI + row0 * TW + threadIdx.x + s + i;
        f2x cuA[NC], cuB[NC], cvA[NC], cvB[NC], cwA[NC], cwB[NC];
#pragma unroll
        for (int c = 0; c < NC; c++) cuA[c] = cuB[c] = cvA[c] = cvB[c] = cwA[c] = cwB[c] = 0;
        // source row m lies in output r's window when 0 <= m - r < 2s: pair A (outputs
        // 0, 1) has none of its rows past m = 2s, pair B (outputs 2, 3) none before
        // m = 2; those evaluations would add exact zeros and are skipped
        auto tap = [&](int m, int c, auto doA, auto doB) {
            const float2 uv = col[m * TW + c];
            const float i1 = colI[m * TW + c];
            const float4 rf = rowf[m];
            const f2x uu = pk2(uv.x, uv.x), vv = pk2(uv.y, uv.y), ii = pk2(i1, i1);
            if constexpr (decltype(doA)::value) {
                const f2x du = fma2(uu, kEE, umA), dv = fma2(vv, kEE, vmA), dI = fma2(ii, kII, IA);
                const f2x q = fma2(dI, dI, fma2(dv, dv, fma2(du, du, pk2(rf.x, rf.y))));
                const f2x w = ex2n_2(mul2(q, rr));
                cuA[c] = fma2(w, uu, cuA[c]);
                cvA[c] = fma2(w, vv, cvA[c]);
                cwA[c] = add2(cwA[c], w);
            }
            if constexpr (decltype(doB)::value) {
                const f2x du = fma2(uu, kEE, umB), dv = fma2(vv, kEE, vmB), dI = fma2(ii, kII, IB);
                const f2x q = fma2(dI, dI, fma2(dv, dv, fma2(du, du, pk2(rf.z, rf.w))));
                const f2x w = ex2n_2(mul2(q, rr));
                cuB[c] = fma2(w, uu, cuB[c]);
                cvB[c] = fma2(w, vv, cvB[c]);
                cwB[c] = add2(cwB[c], w);
            }
        };
        static_assert(TRI_R == 4, "the row split below assumes two output pairs");
        using yes = std::true_type;
        using no = std::false_type;
#pragma unroll
        for (int c = 0; c < NC; c++) {
            tap(0, c, yes{}, no{});
            tap(1, c, yes{}, no{});
        }
#pragma unroll 4
        for (int m = 2; m <= 2 * s; m++) {
#pragma unroll
            for (int c = 0; c < NC; c++) tap(m, c, yes{}, yes{});
        }
#pragma unroll
        for (int c = 0; c < NC; c++) {
            tap(2 * s + 1, c, no{}, yes{});
            tap(2 * s + 2, c, no{}, yes{});
        }
#pragma unroll
        for (int c = 0; c < NC; c++) {
            const float wi = exp2f(-(float)((i + c) * (i + c)) * cS);
            const f2x wi2 = pk2(wi, wi);
            ufA = fma2(wi2, cuA[c], ufA);
            ufB = fma2(wi2, cuB[c], ufB);
            vfA = fma2(wi2, cvA[c], vfA);
            vfB = fma2(wi2, cvB[c], vfB);
            WA = fma2(wi2, cwA[c], WA);
            WB = fma2(wi2, cwB[c], WB);
        }
    };
    int i = -s;
    for (; i + 3 <= s; i += 3) columns(i, std::integral_constant<int, 3>{});
    for (; i < s; i++) columns(i, std::integral_constant<int, 1>{});
    const float uf[TRI_R] = {lo2(ufA), hi2(ufA), lo2(ufB), hi2(ufB)};
    const float vf[TRI_R] = {lo2(vfA), hi2(vfA), lo2(vfB), hi2(vfB)};
    const float W[TRI_R] = {lo2(WA), hi2(WA), lo2(WB), hi2(WB)};
#pragma unroll
    for (int r = 0; r < TRI_R; r++) {
        if (yb + r < sy) {
            const size_t o = (size_t)x + (size_t)(yb + r) * sx;
            const float Wc = fmaxf(1e-5f, W[r]);
            Uo[o] = uf[r] / Wc;
            Vo[o] = vf[r] / Wc;
        }
    }
}

// Exponent scales of the trilateral weights: exp(-d/(2 sigma2)) = exp2(-d * c)
// with intensities divided by 255 folded into cI.
struct TriCoef {
    float cE, cI, cS;
};
__host__ __device__ inline TriCoef tri_coef(float sigmaEPE2, float sigmaI2, float sigmaS2)
{
    const float LOG2E = 1.4426950408889634f;
    TriCoef t;
    t.cE = LOG2E / (2.0f * sigmaEPE2);
    t.cI = LOG2E / (2.0f * sigmaI2 * 255.0f * 255.0f);
    t.cS = LOG2E / (2.0f * sigmaS2);
    return t;
}

}  // namespace dev
}  // namespace bmk

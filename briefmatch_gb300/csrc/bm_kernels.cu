// bm_kernels.cu -- sm_103a kernels of the BriefMatch flow engine.
//
// This unit is compiled with -use_fast_math, the flags the reference kernels are
// built with (CMakeLists.txt:50), so that expressions whose rounding the reference
// fixes (Lanczos weights, the nearest-neighbour index of the down-sampler, the
// curand normals) produce the same bits as the reference build.
//
// Layouts (all row-major, x fastest):
//   descriptors  uint32 [sx*sy][nsp], nsp = ceil(N/32) rounded up to a power of two,
//                padding words zero -- one pixel's descriptor is one or more uint4
//   flow         uint32 per pixel, int16 nx in the low half, int16 ny in the high half
//   cost         uint16 per pixel, the Hamming distance of the current candidate
//                (the reference's D is cost/N)
#include <curand_kernel.h>

#include "bm_internal.h"

namespace bmk {

namespace {

// util_cuda.h:61
#define BM_PI 3.141592653589793115997963468544

constexpr int TX = 32;  // block width: one warp per row of a tile
constexpr int TY = 8;   // block height

__device__ __forceinline__ int lo16(uint32_t w) { return (int)(int16_t)(w & 0xffffu); }
__device__ __forceinline__ int hi16(uint32_t w) { return (int)(int16_t)(w >> 16); }

inline dim3 grid2d(int w, int h) { return dim3((w + TX - 1) / TX, (h + TY - 1) / TY); }

// Tile visited by this block.  Full-frame passes alternate their visiting order
// (raster, then reverse raster): a pass that follows one in the other direction
// starts on the tiles its predecessor touched last, which are still in L2.
__device__ __forceinline__ int2 block_tile(int rev)
{
    int bx = blockIdx.x, by = blockIdx.y;
    if (rev) {
        bx = gridDim.x - 1 - bx;
        by = gridDim.y - 1 - by;
    }
    return make_int2(bx * TX, by * TY);
}

// ---------------------------------------------------------------------------
// Lanczos-3 up-sampling (util_cuda.cu:126-158).
// The weights depend on x only (resp. y only), so they are tabulated once per
// output column/row with the reference's expression; the 6x6 accumulation then
// runs in the reference's order (i outer, j inner) with the same contractions.
// ---------------------------------------------------------------------------
__global__ void k_lanczos_tables(float* __restrict__ w, int* __restrict__ idx, int n_in, int n_out)
{
    int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n_out) return;
    float xp = x * float(n_in) / n_out;
    int x1 = floor(xp);
    int a = 3;
    for (int k = 0; k < 6; k++) {
        int i = x1 - a + 1 + k;
        float xx = BM_PI * (xp - i);
        float L = a * sin(xx) * sin(xx / a) / (xx * xx);
        if (L != L) L = 1;
        w[x * 6 + k] = L;
    }
    idx[x] = x1;
}

template <typename T>
__global__ void __launch_bounds__(256) k_upsample(const T* __restrict__ in, float* __restrict__ out,
                                                  int sxi, int syi, int sxo, int syo,
                                                  const float* __restrict__ lx, const int* __restrict__ ix,
                                                  const float* __restrict__ ly, const int* __restrict__ iy)
{
    int x = blockIdx.x * TX + threadIdx.x;
    int y = blockIdx.y * TY + threadIdx.y;
    if (x >= sxo || y >= syo) return;
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
    out[x + (size_t)y * sxo] = v / w;
}

__global__ void k_u8_to_f32(const uint8_t* __restrict__ in, float* __restrict__ out, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

// ---------------------------------------------------------------------------
// BRIEF descriptors (briefmatch_cuda.cu:82-124).
// The sampling pattern (int-truncated offsets, 4 per sample) is staged in shared
// memory.  Blocks whose pixels stay at least rmax (the largest |offset|) away from
// the border read the image at precomputed linear offsets with no clamping; the
// clamped reads of the reference give the same addresses there.  Border blocks
// clamp each coordinate as the reference does.  A warp reads 32 consecutive
// pixels at the same offset, so each sample is one coalesced L1 request.
// ---------------------------------------------------------------------------
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

template <int NSP>
__global__ void __launch_bounds__(256) k_features(const float* __restrict__ I, uint32_t* __restrict__ F,
                                                  int sx, int sy, int N, const int4* __restrict__ pat, int rmax,
                                                  const __grid_constant__ PatternOffsets po, int rev)
{
    __shared__ int4 s_pat[BM_PATCH_MAX / 4];
    const int2 t0 = block_tile(rev);
    const int bx = t0.x, by = t0.y;
    const int x = bx + threadIdx.x, y = by + threadIdx.y;
    const bool interior = (bx - rmax >= 0) && (bx + TX - 1 + rmax < sx) && (by - rmax >= 0) && (by + TY - 1 + rmax < sy);
    uint32_t word[NSP];
    if (interior) {
        // Every sample reads base + a linear offset held in the kernel's parameter
        // space; the loop is fully unrolled so each offset is an immediate operand.
        // Samples past N carry offset 0 and produce 0 bits.
        const float* base = I + (size_t)y * sx + x;
#pragma unroll
        for (int wd = 0; wd < NSP; wd++) {
            uint32_t acc = 0;
#pragma unroll
            for (int b = 0; b < 32; b++) {
                const int2 o = po.off[wd * 32 + b];
                const float i1 = __ldg(base + o.x);
                const float i2 = __ldg(base + o.y);
                if (i1 > i2) acc |= 1u << b;
            }
            word[wd] = acc;
        }
    } else {
        const int tid = threadIdx.y * TX + threadIdx.x;
        for (int k = tid; k < N; k += TX * TY) s_pat[k] = pat[k];
        __syncthreads();
        if (x >= sx || y >= sy) return;
        const float* base = I + (size_t)y * sx + x;
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
    }
    if (x >= sx || y >= sy) return;
    store_desc<NSP>(F + ((size_t)y * sx + x) * NSP, word);
}

// ---------------------------------------------------------------------------
// PatchMatch (briefmatch_cuda.cu:126-246).
// One launch per jump-flood level.  Every pixel reads its neighbours from the
// level's input field and writes the output field (a snapshot per level), so the
// result does not depend on the schedule.  insert() accepts a candidate iff its
// Hamming distance is strictly lower; candidates equal to the current one (the
// reference's own skip) or to one already evaluated in this level are skipped,
// which leaves every decision unchanged.
// ---------------------------------------------------------------------------
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

template <int NSP>
__global__ void __launch_bounds__(256) k_initialize(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                                    const uint32_t* __restrict__ flow_prev, uint32_t* __restrict__ flow_out,
                                                    uint16_t* __restrict__ cost, int sx, int sy, int first, int rev)
{
    const int2 t0 = block_tile(rev);
    const int x = t0.x + threadIdx.x, y = t0.y + threadIdx.y;
    if (x >= sx || y >= sy) return;
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

// One jump-flood level.  All neighbour reads are issued together, then all
// candidate descriptors are gathered together, and only then are the candidates
// accepted in the reference's order (strictly lower cost wins).  Evaluating a
// candidate that the reference would skip (equal to the current vector) or that
// repeats an earlier one cannot change a decision, so those gathers are elided.
// With RS the iteration's random-search candidate (briefmatch_cuda.cu:237-243) is
// evaluated last; it reads nothing but this pixel's own state, so fusing it into
// the last level gives the reference's result.
template <int NSP, bool RS>
__global__ void __launch_bounds__(256) k_jump_level(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                                    const uint32_t* __restrict__ flow_in, uint32_t* __restrict__ flow_out,
                                                    uint16_t* __restrict__ cost, int sx, int sy,
                                                    int p, int pd, int doubleProp, RsArgs rs, int rev)
{
    constexpr int NC = RS ? 5 : 4;
    const int2 t0 = block_tile(rev);
    const int x = t0.x + threadIdx.x, y = t0.y + threadIdx.y;
    if (x >= sx || y >= sy) return;
    const long n = (long)sx * sy;
    const long pix = x + (long)y * sx;
    const uint32_t own = __ldg(flow_in + pix);
    const int h0 = cost[pix];

    uint32_t cand[NC];
    bool live[NC];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int d = (c < 2) ? -1 : 1;
        const int xy = c & 1;
        const bool active = d > 0 || doubleProp;
        const long doff = xy ? (long)pd * p * d : (long)sx * pd * p * d;
        const long q = pix + doff;
        const uint32_t nb = (active && q >= 0 && q < n) ? __ldg(flow_in + q) : 0u;
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

template <int NSP>
__global__ void __launch_bounds__(256) k_random_search(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                                       uint32_t* __restrict__ flow, uint16_t* __restrict__ cost,
                                                       int sx, int sy, RsArgs rs)
{
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= sx || y >= sy) return;
    const long pix = x + (long)y * sx;
    const uint32_t own = flow[pix];
    const int cx = lo16(own), cy = hi16(own);
    float n1, n2;
    rs_normals(rs, (unsigned int)pix, n1, n2);
    const int nx = min(max((int)round(rs.dist * n1), -x), sx - x - 1);
    const int ny = min(max((int)round(rs.dist * n2), -y), sy - y - 1);
    if (nx == cx && ny == cy) return;
    uint32_t f1[NSP];
    load_desc<NSP>(f1, F1 + pix * NSP);
    const int hc = hamming<NSP>(f1, F2 + (pix + nx + (long)ny * sx) * NSP);
    if (hc < cost[pix]) {
        cost[pix] = (uint16_t)hc;
        flow[pix] = pack_flow(nx, ny);
    }
}

__global__ void k_normals(float2* __restrict__ out, int sx, int sy, RsArgs rs)
{
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= sx || y >= sy) return;
    const long pix = x + (long)y * sx;
    float n1, n2;
    rs_normals(rs, (unsigned int)pix, n1, n2);
    out[pix] = make_float2(n1, n2);
}

// ---------------------------------------------------------------------------
// Down-sampling (briefmatch.cpp:296-324): int16 -> float, Gaussian H then V,
// nearest-neighbour decimation, scaling.  Only the pixels the decimation keeps
// are filtered; each keeps the reference's per-pass float rounding.
// ---------------------------------------------------------------------------
// resizeNN's source index, util_cuda.cu:165-166 (sxi = up-sampled size, sxo = input size),
// tabulated per output column / row with the reference's expression.
__global__ void k_nn_table(unsigned int* __restrict__ idx, int n_up, int n_in)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n_in) return;
    unsigned int x1 = round(x * float(n_up) / n_in);
    idx[x] = x1;
}

__global__ void __launch_bounds__(256) k_downsample(const uint32_t* __restrict__ flow, float* __restrict__ U,
                                                    float* __restrict__ V, int sx, int sy, int sx_in, int sy_in,
                                                    const float* __restrict__ taps, int P, float mx, float my,
                                                    const unsigned int* __restrict__ nnx,
                                                    const unsigned int* __restrict__ nny)
{
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= sx_in || y >= sy_in) return;
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

// CUDA_convert, util_cuda.cu:174-183, for both components when no resampling is needed.
__global__ void k_flow_to_planes(const uint32_t* __restrict__ flow, float* __restrict__ U, float* __restrict__ V,
                                 size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t f = flow[i];
    U[i] = (float)lo16(f);
    V[i] = (float)hi16(f);
}

// ---------------------------------------------------------------------------
// 1-D median (util_cuda.cu:75-111): linear-index window, guard 0 outside the
// plane.  The window is held in registers (padded with +inf up to FS) and the
// first ks+1 positions are sorted as in the reference; v[ks] is the median.
// ---------------------------------------------------------------------------
template <int FS>
__global__ void __launch_bounds__(256) k_median_pass(const float* __restrict__ inU, const float* __restrict__ inV,
                                                     float* __restrict__ outU, float* __restrict__ outV,
                                                     int dir, int fsize, int sx, int sy)
{
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= sx || y >= sy) return;
    const float* in = blockIdx.z ? inV : inU;
    float* out = blockIdx.z ? outV : outU;
    const long n = (long)sx * sy;
    const long base = x + (long)y * sx;
    const long step = dir ? 1 : sx;
    const int ks = fsize / 2;
    float v[FS];
#pragma unroll
    for (int k = 0; k < FS; k++) {
        if (k < fsize) {
            const long idx = base + (long)(k - ks) * step;
            v[k] = (idx >= 0 && idx < n) ? __ldg(in + idx) : 0.0f;
        } else {
            v[k] = __int_as_float(0x7f800000);
        }
    }
#pragma unroll
    for (int i = 0; i < (FS + 1) / 2; i++) {
        if (i <= ks) {
#pragma unroll
            for (int j = i + 1; j < FS; j++) {
                const float a = v[i], b = v[j];
                v[i] = fminf(a, b);
                v[j] = fmaxf(a, b);
            }
        }
    }
    float r = v[0];
#pragma unroll
    for (int i = 1; i < (FS + 1) / 2; i++)
        if (i == ks) r = v[i];
    out[base] = r;
}

// ---------------------------------------------------------------------------
// Cross-trilateral filter (briefmatch_cuda.cu:248-297).
// A block of 32x4 threads filters 32x16 output pixels; each thread owns four
// vertically adjacent outputs, held as two pairs in packed f32x2 registers, so
// every neighbourhood sample it reads from shared memory is used four times and
// every arithmetic instruction serves two outputs.  The (2s+32)^2 neighbourhood
// is staged in shared memory with clamp-to-edge addressing.
// The three Gaussians are one exp2 of the summed exponents; the column factor
// exp2(-cS*i^2) is applied once per column (the inner loop runs down a column).
// Row factors outside the window are -inf, which gives weight 0.
// ---------------------------------------------------------------------------
typedef unsigned long long f2x;  // two packed floats (low = first)

__device__ __forceinline__ f2x pk2(float a, float b) { f2x r; asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b)); return r; }
__device__ __forceinline__ float lo2(f2x v) { float a, b; asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); return a; }
__device__ __forceinline__ float hi2(f2x v) { float a, b; asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); return b; }
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

constexpr int TRI_R = 4;              // outputs per thread (two f32x2 pairs)
constexpr int TRI_TY = 4;             // thread rows per block
constexpr int TRI_BY = TRI_TY * TRI_R;  // output rows per block (32x16 outputs: ~3 blocks per SM at s=24)

__global__ void __launch_bounds__(TX * TRI_TY) k_trilateral_x2(const float* __restrict__ U, const float* __restrict__ V,
                                                       const float* __restrict__ Um, const float* __restrict__ Vm,
                                                       const float* __restrict__ I, float* __restrict__ Uo,
                                                       float* __restrict__ Vo, int sx, int sy, int s,
                                                       float cE, float cI, float cS)
{
    extern __shared__ float4 smem4[];
    const int TW = TX + 2 * s, TH = TRI_BY + 2 * s;
    const int NR = 2 * s + TRI_R - 1;        // source rows a thread walks per column
    float4* rowf = smem4;                    // [NR] exponents of the row factor for outputs r=0..3
    float2* suv = reinterpret_cast<float2*>(smem4 + NR);
    float* sI = reinterpret_cast<float*>(suv + TW * TH);
    const int x0 = blockIdx.x * TX - s, y0 = blockIdx.y * TRI_BY - s;
    const int tid = threadIdx.y * TX + threadIdx.x;
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
            t[r] = (j >= -s && j < s) ? -(float)(j * j) * cS : -__int_as_float(0x7f800000);
        }
        rowf[m] = make_float4(t[0], t[1], t[2], t[3]);
    }
    __syncthreads();

    const int x = blockIdx.x * TX + threadIdx.x;
    const int yb = blockIdx.y * TRI_BY + threadIdx.y * TRI_R;
    if (x >= sx || yb >= sy) return;
    float umc[TRI_R], vmc[TRI_R], Ic[TRI_R];
#pragma unroll
    for (int r = 0; r < TRI_R; r++) {
        const int yy = min(sy - 1, yb + r);
        const size_t o = (size_t)x + (size_t)yy * sx;
        umc[r] = __ldg(Um + o);
        vmc[r] = __ldg(Vm + o);
        Ic[r] = sI[(threadIdx.y * TRI_R + r + s) * TW + threadIdx.x + s];
    }
    const f2x umA = pk2(umc[0], umc[1]), umB = pk2(umc[2], umc[3]);
    const f2x vmA = pk2(vmc[0], vmc[1]), vmB = pk2(vmc[2], vmc[3]);
    const f2x IA = pk2(Ic[0], Ic[1]), IB = pk2(Ic[2], Ic[3]);
    const f2x nE = pk2(-cE, -cE), nI = pk2(-cI, -cI);
    f2x ufA = 0, ufB = 0, vfA = 0, vfB = 0, WA = 0, WB = 0;  // 0 bits = (0.0f, 0.0f)
    const int row0 = threadIdx.y * TRI_R;
    for (int i = -s; i < s; i++) {
        const float2* col = suv + row0 * TW + threadIdx.x + s + i;
        const float* colI = sI + row0 * TW + threadIdx.x + s + i;
        f2x cuA = 0, cuB = 0, cvA = 0, cvB = 0, cwA = 0, cwB = 0;
#pragma unroll 4
        for (int m = 0; m < NR; m++) {
            const float2 uv = col[m * TW];
            const float i1 = colI[m * TW];
            const float4 rf = rowf[m];
            const f2x uu = pk2(uv.x, uv.x), vv = pk2(uv.y, uv.y), ii = pk2(i1, i1);
            f2x du = sub2(uu, umA), dv = sub2(vv, vmA), dI = sub2(ii, IA);
            f2x e = fma2(dv, dv, mul2(du, du));
            f2x arg = fma2(mul2(dI, dI), nI, fma2(e, nE, pk2(rf.x, rf.y)));
            f2x w = ex2_2(arg);
            cuA = fma2(w, uu, cuA);
            cvA = fma2(w, vv, cvA);
            cwA = add2(cwA, w);
            du = sub2(uu, umB);
            dv = sub2(vv, vmB);
            dI = sub2(ii, IB);
            e = fma2(dv, dv, mul2(du, du));
            arg = fma2(mul2(dI, dI), nI, fma2(e, nE, pk2(rf.z, rf.w)));
            w = ex2_2(arg);
            cuB = fma2(w, uu, cuB);
            cvB = fma2(w, vv, cvB);
            cwB = add2(cwB, w);
        }
        const float wi = exp2f(-(float)(i * i) * cS);
        const f2x wi2 = pk2(wi, wi);
        ufA = fma2(wi2, cuA, ufA);
        ufB = fma2(wi2, cuB, ufB);
        vfA = fma2(wi2, cvA, vfA);
        vfB = fma2(wi2, cvB, vfB);
        WA = fma2(wi2, cwA, WA);
        WB = fma2(wi2, cwB, WB);
    }
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

__global__ void __launch_bounds__(256) k_trilateral_global(const float* __restrict__ U, const float* __restrict__ V,
                                                           const float* __restrict__ Um, const float* __restrict__ Vm,
                                                           const float* __restrict__ I, float* __restrict__ Uo,
                                                           float* __restrict__ Vo, int sx, int sy, int s,
                                                           float cE, float cI, float cS)
{
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= sx || y >= sy) return;
    const size_t o = (size_t)x + (size_t)y * sx;
    const float um0 = Um[o], vm0 = Vm[o], I0 = I[o];
    float uf = 0.0f, vf = 0.0f, W = 0.0f;
    for (int i = -s; i < s; i++) {
        const int gx = min(sx - 1, max(0, x + i));
        const float si = (float)(i * i) * cS;
        for (int j = -s; j < s; j++) {
            const size_t g = (size_t)gx + (size_t)min(sy - 1, max(0, y + j)) * sx;
            const float u1 = __ldg(U + g), v1 = __ldg(V + g);
            const float dI = __ldg(I + g) - I0;
            const float du = u1 - um0, dv = v1 - vm0;
            const float e = du * du + dv * dv;
            const float sp = si + (float)(j * j) * cS;
            const float w = exp2f(fmaf(e, -cE, fmaf(dI * dI, -cI, -sp)));
            uf = fmaf(w, u1, uf);
            vf = fmaf(w, v1, vf);
            W += w;
        }
    }
    const float Wc = fmaxf(1e-5f, W);
    Uo[o] = uf / Wc;
    Vo[o] = vf / Wc;
}

// ---------------------------------------------------------------------------
// Reference-layout export/import (briefmatch.h:139-141).
// ---------------------------------------------------------------------------
__global__ void k_export_field(const uint32_t* __restrict__ flow, const uint16_t* __restrict__ cost,
                               int16_t* __restrict__ nx, int16_t* __restrict__ ny, float* __restrict__ dist,
                               size_t n, int N)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t f = flow[i];
    if (nx) nx[i] = (int16_t)lo16(f);
    if (ny) ny[i] = (int16_t)hi16(f);
    // featDist's return value, briefmatch_cuda.cu:79
    if (dist) dist[i] = float((int)cost[i]) / N;
}

__global__ void k_import_field(const int16_t* __restrict__ nx, const int16_t* __restrict__ ny,
                               const uint16_t* __restrict__ cost_in, uint32_t* __restrict__ flow,
                               uint16_t* __restrict__ cost, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flow[i] = pack_flow(nx[i], ny[i]);
    if (cost_in) cost[i] = cost_in[i];
}

}  // namespace

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
cudaError_t lanczos_tables(float* w, int* idx, int n_in, int n_out, cudaStream_t st)
{
    k_lanczos_tables<<<(n_out + 127) / 128, 128, 0, st>>>(w, idx, n_in, n_out);
    return cudaGetLastError();
}

cudaError_t upsample_f32(const float* in, float* out, int sxi, int syi, int sxo, int syo,
                         const float* lx, const int* ix, const float* ly, const int* iy, cudaStream_t st)
{
    k_upsample<float><<<grid2d(sxo, syo), dim3(TX, TY), 0, st>>>(in, out, sxi, syi, sxo, syo, lx, ix, ly, iy);
    return cudaGetLastError();
}

cudaError_t upsample_u8(const uint8_t* in, float* out, int sxi, int syi, int sxo, int syo,
                        const float* lx, const int* ix, const float* ly, const int* iy, cudaStream_t st)
{
    k_upsample<uint8_t><<<grid2d(sxo, syo), dim3(TX, TY), 0, st>>>(in, out, sxi, syi, sxo, syo, lx, ix, ly, iy);
    return cudaGetLastError();
}

cudaError_t u8_to_f32(const uint8_t* in, float* out, size_t n, cudaStream_t st)
{
    k_u8_to_f32<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(in, out, n);
    return cudaGetLastError();
}

#define BM_DISPATCH_NSP(nsp, ...)                          \
    switch (nsp) {                                         \
    case 1: { constexpr int NSP = 1; __VA_ARGS__; } break;   \
    case 2: { constexpr int NSP = 2; __VA_ARGS__; } break;   \
    case 4: { constexpr int NSP = 4; __VA_ARGS__; } break;   \
    case 8: { constexpr int NSP = 8; __VA_ARGS__; } break;   \
    case 16: { constexpr int NSP = 16; __VA_ARGS__; } break; \
    default: return cudaErrorInvalidValue;                 \
    }

cudaError_t features(const float* up, uint32_t* F, int sx, int sy, int N, int nsp,
                     const int4* pat, int rmax, const PatternOffsets& po, int rev, cudaStream_t st)
{
    BM_DISPATCH_NSP(nsp, k_features<NSP><<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(up, F, sx, sy, N, pat, rmax, po, rev));
    return cudaGetLastError();
}

cudaError_t initialize(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_prev,
                       uint32_t* flow_out, uint16_t* cost, int sx, int sy, int nsp, int first, int rev,
                       cudaStream_t st)
{
    BM_DISPATCH_NSP(nsp, k_initialize<NSP><<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(F1, F2, flow_prev, flow_out, cost, sx, sy, first, rev));
    return cudaGetLastError();
}

cudaError_t jump_level(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_in,
                       uint32_t* flow_out, uint16_t* cost, int sx, int sy, int nsp,
                       int p, int pd, int doubleProp, const RsArgs& rs, int rev, cudaStream_t st)
{
    if (rs.enabled) {
        BM_DISPATCH_NSP(nsp, k_jump_level<NSP, true><<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(F1, F2, flow_in, flow_out, cost, sx, sy, p, pd, doubleProp, rs, rev));
    } else {
        BM_DISPATCH_NSP(nsp, k_jump_level<NSP, false><<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(F1, F2, flow_in, flow_out, cost, sx, sy, p, pd, doubleProp, rs, rev));
    }
    return cudaGetLastError();
}

cudaError_t random_search(const uint32_t* F1, const uint32_t* F2, uint32_t* flow, uint16_t* cost,
                          int sx, int sy, int nsp, const RsArgs& rs, cudaStream_t st)
{
    BM_DISPATCH_NSP(nsp, k_random_search<NSP><<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(F1, F2, flow, cost, sx, sy, rs));
    return cudaGetLastError();
}

cudaError_t normals(float2* out, int sx, int sy, const RsArgs& rs, cudaStream_t st)
{
    k_normals<<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(out, sx, sy, rs);
    return cudaGetLastError();
}

cudaError_t nn_table(unsigned int* idx, int n_up, int n_in, cudaStream_t st)
{
    k_nn_table<<<(n_in + 127) / 128, 128, 0, st>>>(idx, n_up, n_in);
    return cudaGetLastError();
}

cudaError_t downsample(const uint32_t* flow, float* U, float* V, int sx, int sy, int sx_in, int sy_in,
                       const float* taps, int P, float mx, float my, const unsigned int* nnx,
                       const unsigned int* nny, cudaStream_t st)
{
    k_downsample<<<grid2d(sx_in, sy_in), dim3(TX, TY), 0, st>>>(flow, U, V, sx, sy, sx_in, sy_in, taps, P, mx, my,
                                                                nnx, nny);
    return cudaGetLastError();
}

cudaError_t flow_to_planes(const uint32_t* flow, float* U, float* V, size_t n, cudaStream_t st)
{
    k_flow_to_planes<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(flow, U, V, n);
    return cudaGetLastError();
}

cudaError_t median_pass(const float* inU, const float* inV, float* outU, float* outV,
                        int dir, int fsize, int sx, int sy, cudaStream_t st)
{
    dim3 g = grid2d(sx, sy);
    g.z = 2;
#define BM_MED(FSV) k_median_pass<FSV><<<g, dim3(TX, TY), 0, st>>>(inU, inV, outU, outV, dir, fsize, sx, sy)
    if (fsize <= 9) BM_MED(9);
    else if (fsize <= 13) BM_MED(13);
    else if (fsize <= 15) BM_MED(15);
    else if (fsize <= 23) BM_MED(23);
    else if (fsize <= 31) BM_MED(31);
    else if (fsize <= BM_MAX_MEDIAN) BM_MED(BM_MAX_MEDIAN);
    else return cudaErrorInvalidValue;
#undef BM_MED
    return cudaGetLastError();
}

cudaError_t trilateral(const float* U, const float* V, const float* Um, const float* Vm,
                       const float* I, float* Uo, float* Vo, int sx, int sy, int s,
                       float sigmaEPE2, float sigmaI2, float sigmaS2, cudaStream_t st)
{
    const float LOG2E = 1.4426950408889634f;
    // exp(-d/(2 sigma)) = exp2(-d * log2(e) / (2 sigma)); intensities are divided by 255.
    const float cE = LOG2E / (2.0f * sigmaEPE2);
    const float cI = LOG2E / (2.0f * sigmaI2 * 255.0f * 255.0f);
    const float cS = LOG2E / (2.0f * sigmaS2);
    const size_t smem = (size_t)(2 * s + TRI_R - 1) * sizeof(float4) +
                        (size_t)(TX + 2 * s) * (TRI_BY + 2 * s) * 3 * sizeof(float);
    if (smem <= 220 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(k_trilateral_x2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        dim3 g((sx + TX - 1) / TX, (sy + TRI_BY - 1) / TRI_BY);
        k_trilateral_x2<<<g, dim3(TX, TRI_TY), smem, st>>>(U, V, Um, Vm, I, Uo, Vo, sx, sy, s, cE, cI, cS);
    } else {
        k_trilateral_global<<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(U, V, Um, Vm, I, Uo, Vo, sx, sy, s, cE, cI, cS);
    }
    return cudaGetLastError();
}

cudaError_t export_field(const uint32_t* flow, const uint16_t* cost, int16_t* nx, int16_t* ny,
                         float* dist, size_t n, int N, cudaStream_t st)
{
    k_export_field<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(flow, cost, nx, ny, dist, n, N);
    return cudaGetLastError();
}

cudaError_t import_field(const int16_t* nx, const int16_t* ny, const uint16_t* cost_in,
                         uint32_t* flow, uint16_t* cost, size_t n, cudaStream_t st)
{
    k_import_field<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(nx, ny, cost_in, flow, cost, n);
    return cudaGetLastError();
}

}  // namespace bmk

// bm_kernels.cu -- sm_103a kernels of the BriefMatch flow engine, single frame pair.
//
// This unit is compiled with -use_fast_math, the flags the reference kernels are
// built with (CMakeLists.txt:50), so that expressions whose rounding the reference
// fixes (Lanczos weights, the nearest-neighbour index of the down-sampler, the
// curand normals) produce the same bits as the reference build.  The per-pixel
// bodies live in bm_device.cuh, shared with the batched kernels.
//
// Layouts (all row-major, x fastest):
//   descriptors  uint32 [sx*sy][nsp], nsp = ceil(N/32) rounded up to a power of two,
//                padding words zero -- one pixel's descriptor is one or more uint4
//   flow         uint32 per pixel, int16 nx in the low half, int16 ny in the high half
//   cost         uint16 per pixel, the Hamming distance of the current candidate
//                (the reference's D is cost/N)
#include <climits>
#include <mutex>

#include "bm_device.cuh"

namespace bmk {

namespace {

using namespace dev;

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

// Lanczos weight tables (util_cuda.cu:134-151): per output column (or row) the six
// weights with the reference's expression and the first tap index.
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
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= sxo || y >= syo) return;
    upsample_px<T>(in, out, sxi, syi, sxo, lx, ix, ly, iy, x, y);
}

// Up-sampling into an edge-replicated image: the output covers (sxo + 2m) x
// (syo + 2m) pixels at row pitch `pitch`; a pixel of the margin holds the value of
// the nearest image pixel (each coordinate clamped), computed by the same Lanczos
// expression, so every read of the margin equals a clamped read of the image.
// Each thread computes UP_R output rows of one column (a block covers
// TX x (TY * UP_R) outputs).  The rows share the column's six
// weights and source columns, and rows whose Lanczos windows start on the same
// source row share the products input * Lx: they are formed once per window (36
// multiplies) and each output then takes its 36 multiply-adds onto them in the
// reference's order (util_cuda.cu:140-152: over source columns, then rows;
// v += (in * Lx) * Ly as one rounded product and an FMA, w += Lx * Ly as an FMA), so
// every value equals upsample_val's bit for bit.
constexpr int UP_R = 8;
__global__ void __launch_bounds__(TX * TY) k_upsample_pad_rows(const uint8_t* __restrict__ in, float* __restrict__ out,
                                                               int pitch, int m, int sxi, int syi, int sxo, int syo,
                                                               const float* __restrict__ lx, const int* __restrict__ ix,
                                                               const float* __restrict__ ly, const int* __restrict__ iy)
{
    const int X = blockIdx.x * TX + threadIdx.x;
    const int Y0 = (blockIdx.y * TY + threadIdx.y) * UP_R;
    if (X >= sxo + 2 * m || Y0 >= syo + 2 * m) return;
    const int x = min(sxo - 1, max(0, X - m));
    float Lx[6];
    int col[6];
    const int x1 = __ldg(ix + x);
#pragma unroll
    for (int a = 0; a < 6; a++) {
        Lx[a] = __ldg(lx + x * 6 + a);
        col[a] = min(sxi - 1, max(0, x1 - 2 + a));
    }
    float P[6][6];  // P[a][b] = in[row b of the window][col a] * Lx[a]
    int win = INT_MIN;
#pragma unroll
    for (int r = 0; r < UP_R; r++) {
        const int Y = Y0 + r;
        if (Y >= syo + 2 * m) break;
        const int y = min(syo - 1, max(0, Y - m));
        const int y1 = __ldg(iy + y);
        if (y1 != win) {  // uniform across the warp (one output row per warp)
            win = y1;
#pragma unroll
            for (int b = 0; b < 6; b++) {
                const uint8_t* src = in + (size_t)min(syi - 1, max(0, y1 - 2 + b)) * sxi;
#pragma unroll
                for (int a = 0; a < 6; a++) P[a][b] = __fmul_rn((float)__ldg(src + col[a]), Lx[a]);
            }
        }
        float Ly[6];
#pragma unroll
        for (int b = 0; b < 6; b++) Ly[b] = __ldg(ly + y * 6 + b);
        float v = 0.0f, w = 0.0f;
#pragma unroll
        for (int a = 0; a < 6; a++)
#pragma unroll
            for (int b = 0; b < 6; b++) {
                w = __fmaf_rn(Lx[a], Ly[b], w);
                v = __fmaf_rn(P[a][b], Ly[b], v);
            }
        out[X + (size_t)Y * pitch] = v / w;
    }
}

__global__ void k_u8_to_f32(const uint8_t* __restrict__ in, float* __restrict__ out, size_t n)
{
    size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}


// BRIEF descriptors: interior tiles read the linear offsets from the kernel's
// parameter space (fully unrolled, immediate operands); border tiles stage the
// pattern in shared memory and clamp.
template <int NSP>
__global__ void __launch_bounds__(256) k_features(const float* __restrict__ I, uint32_t* __restrict__ F,
                                                  int sx, int sy, int N, const int4* __restrict__ pat, int rmax,
                                                  const __grid_constant__ PatternOffsets po, int rev)
{
    __shared__ int4 s_pat[BM_PATCH_MAX / 4];
    const int2 t0 = block_tile(rev);
    const int x = t0.x + threadIdx.x, y = t0.y + threadIdx.y;
    if (tile_interior(t0.x, t0.y, sx, sy, rmax)) {
        features_interior_px<NSP>(I, F, sx, x, y, po.off);
    } else {
        const int tid = threadIdx.y * TX + threadIdx.x;
        for (int k = tid; k < N; k += TX * TY) s_pat[k] = pat[k];
        __syncthreads();
        if (x >= sx || y >= sy) return;
        features_border_px<NSP>(I, F, sx, sy, N, s_pat, x, y);
    }
}

// BRIEF descriptors from an edge-replicated image (k_upsample_pad_rows) whose margin is
// at least the pattern's largest offset: every pixel reads at the linear offsets
// (no clamping, no border tiles); each thread computes feat_px<NSP>() pixels TX apart
// (two up to 128-bit descriptors, where sharing each offset's address arithmetic
// pays; one for longer ones, whose descriptor words would cost occupancy).
template <int NSP>
__host__ __device__ constexpr int feat_px() { return NSP <= 4 ? 2 : 1; }
template <int NSP>
__global__ void __launch_bounds__(256) k_features_pad(const float* __restrict__ I, uint32_t* __restrict__ F,
                                                      int pitch, int sx, int sy,
                                                      const __grid_constant__ PatternOffsets po, int rev)
{
    int bx = blockIdx.x, by = blockIdx.y;
    if (rev) {
        bx = gridDim.x - 1 - bx;
        by = gridDim.y - 1 - by;
    }
    const int x = bx * (TX * feat_px<NSP>()) + threadIdx.x, y = by * TY + threadIdx.y;
    if (x >= sx || y >= sy) return;
    features_strip_px<NSP, feat_px<NSP>()>(I + (size_t)y * pitch + x, F + ((size_t)y * sx + x) * NSP, sx - x, po.off);
}

template <int NSP>
__global__ void __launch_bounds__(256) k_initialize(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                                    const uint32_t* __restrict__ flow_prev, uint32_t* __restrict__ flow_out,
                                                    uint16_t* __restrict__ cost, int sx, int sy, int first, int rev)
{
    const int2 t0 = block_tile(rev);
    const int x = t0.x + threadIdx.x, y = t0.y + threadIdx.y;
    if (x >= sx || y >= sy) return;
    init_px<NSP>(F1, F2, flow_prev, flow_out, cost, sx, sy, first, x, y);
}

template <int NSP>
__global__ void __launch_bounds__(256) k_seed(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                              const uint32_t* __restrict__ flow_prev, uint32_t* __restrict__ flow_out,
                                              uint16_t* __restrict__ cost, int sx, int sy, int first,
                                              const float* __restrict__ pred, int w4, int h4, float scale_x,
                                              float scale_y, float inv_x, float inv_y, float logit_min)
{
    const int x = blockIdx.x * TX + threadIdx.x, y = blockIdx.y * TY + threadIdx.y;
    if (x >= sx || y >= sy) return;
    seed_px<NSP>(F1, F2, flow_prev, flow_out, cost, sx, sy, first, x, y, pred, w4, h4, scale_x, scale_y, inv_x, inv_y,
                 logit_min);
}

template <int NSP, bool RS>
__global__ void __launch_bounds__(256) k_jump_level(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                                    const uint32_t* __restrict__ flow_in, uint32_t* __restrict__ flow_out,
                                                    uint16_t* __restrict__ cost, int sx, int sy,
                                                    int p, int pd, int doubleProp, RsArgs rs, int rev)
{
    const int2 t0 = block_tile(rev);
    const int x = t0.x + threadIdx.x, y = t0.y + threadIdx.y;
    if (x >= sx || y >= sy) return;
    jump_px<NSP, RS>(F1, F2, flow_in, flow_out, cost, sx, sy, p, pd, doubleProp, rs, x, y);
}

template <int NSP>
__global__ void __launch_bounds__(256) k_local_step(const uint32_t* __restrict__ F1, const uint32_t* __restrict__ F2,
                                                    const uint32_t* __restrict__ flow_in, uint32_t* __restrict__ flow_out,
                                                    uint16_t* __restrict__ cost, int sx, int sy, int r, int rev)
{
    const int2 t0 = block_tile(rev);
    const int x = t0.x + threadIdx.x, y = t0.y + threadIdx.y;
    if (x >= sx || y >= sy) return;
    local_px<NSP>(F1, F2, flow_in, flow_out, cost, sx, sy, r, x, y);
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
    downsample_px(flow, U, V, sx, sy, sx_in, taps, P, mx, my, nnx, nny, x, y);
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


// Separable 1-D median, both components in one launch (blockIdx.z).  Each thread
// computes two outputs adjacent along the filter direction (median2_px): down a
// column (dir 0) the rows y and y+1; along the rows (dir 1) the linear indices 2t and
// 2t+1 (the reference's window runs over linear indices, so a pair may span a row
// end).
template <int FS>
__global__ void __launch_bounds__(256) k_median_pass(const float* __restrict__ inU, const float* __restrict__ inV,
                                                     float* __restrict__ outU, float* __restrict__ outV,
                                                     int dir, int fsize, int sx, int sy)
{
    static_assert(FS % 2 == 1, "median register windows are odd");
    const float* in = blockIdx.z ? inV : inU;
    float* out = blockIdx.z ? outV : outU;
    const long n = (long)sx * sy;
    if (dir) {
        const long p = 2 * ((long)blockIdx.x * (TX * TY) + threadIdx.y * TX + threadIdx.x);
        if (p >= n) return;
        median2_px<FS>(in, out, p, 1, n, fsize, p + 1 < n);
    } else {
        const int x = blockIdx.x * TX + threadIdx.x, y = 2 * (blockIdx.y * TY + threadIdx.y);
        if (x >= sx || y >= sy) return;
        median2_px<FS>(in, out, x + (long)y * sx, sx, n, fsize, y + 1 < sy);
    }
}

__global__ void __launch_bounds__(TX * TRI_TY) k_trilateral_x2(const float* __restrict__ U, const float* __restrict__ V,
                                                               const float* __restrict__ Um, const float* __restrict__ Vm,
                                                               const float* __restrict__ I, float* __restrict__ Uo,
                                                               float* __restrict__ Vo, int sx, int sy, int s,
                                                               float cE, float cI, float cS)
{
    extern __shared__ float4 smem4[];
    trilateral_block(U, V, Um, Vm, I, Uo, Vo, sx, sy, s, cE, cI, cS, blockIdx.x * TX, blockIdx.y * TRI_BY, smem4);
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

cudaError_t upsample_u8_pad(const uint8_t* in, float* out, int pitch, int m, int sxi, int syi, int sxo, int syo,
                            const float* lx, const int* ix, const float* ly, const int* iy, cudaStream_t st)
{
    if (m < 0 || pitch < sxo + 2 * m) return cudaErrorInvalidValue;
    const dim3 g((sxo + 2 * m + TX - 1) / TX, (syo + 2 * m + TY * UP_R - 1) / (TY * UP_R));
    k_upsample_pad_rows<<<g, dim3(TX, TY), 0, st>>>(in, out, pitch, m, sxi, syi, sxo, syo, lx, ix, ly, iy);
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

cudaError_t features_pad(const float* up, int pitch, uint32_t* F, int sx, int sy, int nsp,
                         const PatternOffsets& po, int rev, cudaStream_t st)
{
    BM_DISPATCH_NSP(nsp, {
        const int w = TX * feat_px<NSP>();
        k_features_pad<NSP><<<dim3((sx + w - 1) / w, (sy + TY - 1) / TY), dim3(TX, TY), 0, st>>>(up, F, pitch, sx, sy,
                                                                                                 po, rev);
    });
    return cudaGetLastError();
}

cudaError_t initialize(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_prev,
                       uint32_t* flow_out, uint16_t* cost, int sx, int sy, int nsp, int first, int rev,
                       cudaStream_t st)
{
    BM_DISPATCH_NSP(nsp, k_initialize<NSP><<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(F1, F2, flow_prev, flow_out, cost, sx, sy, first, rev));
    return cudaGetLastError();
}

cudaError_t seed_field(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_prev, uint32_t* flow_out,
                       uint16_t* cost, int sx, int sy, int nsp, int first, const float* pred, int w4, int h4,
                       float scale_x, float scale_y, float logit_min, cudaStream_t st)
{
    // host IEEE reciprocals: the device cell lookup multiplies by them
    const float inv_x = 1.0f / scale_x, inv_y = 1.0f / scale_y;
    BM_DISPATCH_NSP(nsp, k_seed<NSP><<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(F1, F2, flow_prev, flow_out, cost, sx, sy, first, pred, w4, h4, scale_x, scale_y, inv_x, inv_y, logit_min));
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

cudaError_t local_step(const uint32_t* F1, const uint32_t* F2, const uint32_t* flow_in, uint32_t* flow_out,
                       uint16_t* cost, int sx, int sy, int nsp, int r, int rev, cudaStream_t st)
{
    BM_DISPATCH_NSP(nsp, k_local_step<NSP><<<grid2d(sx, sy), dim3(TX, TY), 0, st>>>(F1, F2, flow_in, flow_out, cost, sx, sy, r, rev));
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
    const long n = (long)sx * sy;
    const dim3 g = dir ? dim3((unsigned)((n + 2 * TX * TY - 1) / (2 * TX * TY)), 1, 2)
                       : dim3((sx + TX - 1) / TX, (sy + 2 * TY - 1) / (2 * TY), 2);
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

// The trilateral kernel's dynamic shared-memory opt-in, raised only when a larger
// window than any before needs it (so launches after the first of a size make no
// attribute call and can be captured in a graph).  The opt-in only ever grows, under
// a lock: contexts created on several host threads never lower it below what another
// thread's launch was checked against.
cudaError_t ensure_trilateral_smem(int s)
{
    static std::mutex mu;
    static int granted[64] = {0};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    const int need = (int)tri_smem_bytes(s);
    std::lock_guard<std::mutex> lock(mu);
    if (need <= granted[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(k_trilateral_x2, cudaFuncAttributeMaxDynamicSharedMemorySize, need);
    if (e == cudaSuccess) granted[dev] = need;
    return e;
}

cudaError_t trilateral(const float* U, const float* V, const float* Um, const float* Vm,
                       const float* I, float* Uo, float* Vo, int sx, int sy, int s,
                       float sigmaEPE2, float sigmaI2, float sigmaS2, cudaStream_t st)
{
    const TriCoef tc = tri_coef(sigmaEPE2, sigmaI2, sigmaS2);
    const float cE = tc.cE, cI = tc.cI, cS = tc.cS;
    const size_t smem = tri_smem_bytes(s);
    if (smem <= 220 * 1024) {
        cudaError_t e = ensure_trilateral_smem(s);
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

// bm_batch.cu -- many frame pairs of uneven size in one pass.
//
// A batch packs every pair's buffers into one device arena and describes each pair
// (geometry, derived constants, buffer addresses) in a device table.  Every stage
// runs as one launch over the union of all pairs' tiles; a block finds its pair by
// binary search over per-stage tile prefix sums.  The matching phase (initialisation
// and every jump-flood level of every iteration) can instead run as one persistent
// cooperative launch whose blocks meet at a bounded grid barrier between levels.
// A whole batch step can be captured in a CUDA graph and replayed.  Which schedule
// runs is chosen by bm_batch_autotune, which times the candidates on the batch
// itself and caches the winner per batch shape in a JSON file.
//
// Each pair is computed exactly as a fresh single-pair context would: the first
// frame primes, the second is matched with zero initialisation and the random
// stream positions 0..iterations-1.  The per-pixel bodies are bm_device.cuh's.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "bm_device.cuh"

namespace {

using namespace bmk;
using namespace bmk::dev;

// One pair of the batch as the kernels see it.
struct PairDev {
    int sx, sy, sx_in, sy_in;
    int P, fsize, tri_s, rmax;
    float dist, mx, my, cE, cI, cS;
    int first_up_tile_x;   // tiles per row on the up-sampled grid
    int first_in_tile_x;   // tiles per row at input resolution (32x8)
    int first_tri_tile_x;  // tiles per row for the trilateral filter (TX x TRI_BY)
    const uint8_t* frame[2];
    float* guide;          // frame 0 as float (the trilateral guide)
    float* up;             // up-sampled frame: dense sx*sy, or edge-replicated (below)
    int up_margin;         // margin the up buffer has room for: (sx+2m)*(sy+2m) floats
    uint32_t* F[2];
    uint32_t* flow[2];
    uint16_t* cost;
    float* flow_in;        // U then V
    float* flow_med;
    float* flow_out;
    float* tmp;
    const int4* pat;
    const int2* off;
    const float* taps;
    const float* lx;
    const int* ix;
    const float* ly;
    const int* iy;
    const unsigned int* nnx;
    const unsigned int* nny;
};

// The pairs [lo, hi) (internal order) that one launch covers: a "wave".
struct BatchDev {
    const PairDev* pairs;
    const unsigned int* pre_up;   // [count+1] exclusive prefix of up-sampled-grid tiles
    const unsigned int* pre_in;   // input-resolution 32x8 tiles
    const unsigned int* pre_tri;  // trilateral TX x TRI_BY tiles
    int lo, hi;
    int N;
};

// Bounded grid barrier for the persistent launch (all blocks co-resident by the
// cooperative launch).  A block that waits longer than `limit` polls sets the error
// word and every block leaves at its next barrier.  `arrived` and `generation` are
// cleared before every wave's launch, `error` and `where` once per step.
struct GridSync {
    unsigned int arrived;
    unsigned int generation;
    unsigned int error;
    unsigned int where;
};

__device__ __forceinline__ bool grid_sync(GridSync* gs, unsigned int nblocks, unsigned long long limit,
                                          unsigned int tag)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        ok = 1;
        volatile unsigned int* vgen = &gs->generation;
        volatile unsigned int* verr = &gs->error;
        const unsigned int gen = *vgen;
        __threadfence();
        const unsigned int a = atomicAdd(&gs->arrived, 1u);
        if (a == nblocks - 1) {
            atomicExch(&gs->arrived, 0u);
            __threadfence();
            atomicAdd(&gs->generation, 1u);
        } else {
            unsigned long long it = 0;
            while (*vgen == gen) {
                if (*verr || ++it > limit) {
                    atomicExch(&gs->error, 1u);
                    atomicMax(&gs->where, tag);
                    ok = 0;
                    break;
                }
                __nanosleep(100);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Pair of the wave [wlo, whi) that owns tile `tile` (a global tile index).
__device__ __forceinline__ int find_pair(const unsigned int* __restrict__ pre, int wlo, int whi, unsigned int tile)
{
    int lo = wlo, hi = whi - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(pre + mid) <= tile)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// ---------------------------------------------------------------------------
// Batched stages: blockIdx.x enumerates the union of all pairs' tiles.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_b_guide(BatchDev bd)
{
    const unsigned int tile = bd.pre_in[bd.lo] + blockIdx.x;
    const int i = find_pair(bd.pre_in, bd.lo, bd.hi, tile);
    const PairDev& P = bd.pairs[i];
    const unsigned int t = tile - bd.pre_in[i];
    const int x = (int)(t % P.first_in_tile_x) * TX + threadIdx.x, y = (int)(t / P.first_in_tile_x) * TY + threadIdx.y;
    if (x >= P.sx_in || y >= P.sy_in) return;
    const size_t o = (size_t)y * P.sx_in + x;
    P.guide[o] = (float)P.frame[0][o];
}

__global__ void __launch_bounds__(256) k_b_upsample(BatchDev bd, int which)
{
    const unsigned int tile = bd.pre_up[bd.lo] + blockIdx.x;
    const int i = find_pair(bd.pre_up, bd.lo, bd.hi, tile);
    const PairDev& P = bd.pairs[i];
    const unsigned int t = tile - bd.pre_up[i];
    const int x = (int)(t % P.first_up_tile_x) * TX + threadIdx.x, y = (int)(t / P.first_up_tile_x) * TY + threadIdx.y;
    if (x >= P.sx || y >= P.sy) return;
    if (P.sx == P.sx_in && P.sy == P.sy_in)
        P.up[(size_t)y * P.sx + x] = (float)P.frame[which][(size_t)y * P.sx + x];
    else
        upsample_px<uint8_t>(P.frame[which], P.up, P.sx_in, P.sy_in, P.sx, P.lx, P.ix, P.ly, P.iy, x, y);
}

// Tile `tile` of the up-sampled grids, visited in reverse order when rev is set.
__device__ __forceinline__ bool up_tile(const BatchDev& bd, unsigned int tile, int& i, int& x, int& y)
{
    i = find_pair(bd.pre_up, bd.lo, bd.hi, tile);
    const PairDev& P = bd.pairs[i];
    const unsigned int t = tile - bd.pre_up[i];
    x = (int)(t % P.first_up_tile_x) * TX + threadIdx.x;
    y = (int)(t / P.first_up_tile_x) * TY + threadIdx.y;
    return x < P.sx && y < P.sy;
}

template <int NSP>
__global__ void __launch_bounds__(256) k_b_initialize(BatchDev bd, int cur, int rev)
{
    const unsigned int base = bd.pre_up[bd.lo], total = bd.pre_up[bd.hi] - base;
    const unsigned int tile = base + (rev ? total - 1 - blockIdx.x : blockIdx.x);
    int i, x, y;
    if (!up_tile(bd, tile, i, x, y)) return;
    const PairDev& P = bd.pairs[i];
    init_px<NSP>(P.F[0], P.F[1], P.flow[cur], P.flow[cur ^ 1], P.cost, P.sx, P.sy, 1, x, y);
}

template <int NSP, bool RS>
__global__ void __launch_bounds__(256) k_b_jump(BatchDev bd, int cur, int p, int pd, int doubleProp, RsArgs rs, int rev)
{
    const unsigned int base = bd.pre_up[bd.lo], total = bd.pre_up[bd.hi] - base;
    const unsigned int tile = base + (rev ? total - 1 - blockIdx.x : blockIdx.x);
    int i, x, y;
    if (!up_tile(bd, tile, i, x, y)) return;
    const PairDev& P = bd.pairs[i];
    RsArgs r = rs;
    r.dist = P.dist;
    jump_px<NSP, RS>(P.F[0], P.F[1], P.flow[cur], P.flow[cur ^ 1], P.cost, P.sx, P.sy, p, pd, doubleProp, r, x, y);
}

struct MatchPlan {
    int iterations, jfMax, doubleProp, rng;
    unsigned long long seed;
    unsigned long long spin_limit;
    int snake;
};

// Initialisation and every jump-flood level of every iteration in one launch.
// Each phase walks the union of up-sampled tiles with a grid-stride loop, then all
// blocks meet at the grid barrier before the next phase reads the new field.
template <int NSP>
__global__ void __launch_bounds__(256) k_b_match_persistent(BatchDev bd, MatchPlan plan, GridSync* gs)
{
    const unsigned int base = bd.pre_up[bd.lo], total = bd.pre_up[bd.hi] - base;
    int cur = 0;
    unsigned int phase = 0;
    for (unsigned int k = blockIdx.x; k < total; k += gridDim.x) {
        int i, x, y;
        if (up_tile(bd, base + k, i, x, y)) {
            const PairDev& P = bd.pairs[i];
            init_px<NSP>(P.F[0], P.F[1], P.flow[0], P.flow[1], P.cost, P.sx, P.sy, 1, x, y);
        }
    }
    cur = 1;
    if (!grid_sync(gs, gridDim.x, plan.spin_limit, ++phase)) return;
    int pd = -1;
    for (int it = 0; it < plan.iterations; it++) {
        int levels = 0;
        for (int s = plan.jfMax; s > 0; s /= 2) levels++;
        int lvl = 0;
        for (int s = plan.jfMax; s > 0; s /= 2, lvl++) {
            const bool last = lvl == levels - 1;
            const int rev = plan.snake ? (int)(phase & 1u) : 0;
            RsArgs rs;
            rs.enabled = last ? 1 : 0;
            rs.mode = plan.rng;
            rs.seed = plan.seed;
            rs.call = (unsigned long long)it;
            for (unsigned int k = blockIdx.x; k < total; k += gridDim.x) {
                const unsigned int tile = base + (rev ? total - 1 - k : k);
                int i, x, y;
                if (!up_tile(bd, tile, i, x, y)) continue;
                const PairDev& P = bd.pairs[i];
                rs.dist = P.dist;
                if (last)
                    jump_px<NSP, true, true>(P.F[0], P.F[1], P.flow[cur], P.flow[cur ^ 1], P.cost, P.sx, P.sy, s, pd,
                                             plan.doubleProp, rs, x, y);
                else
                    jump_px<NSP, false, true>(P.F[0], P.F[1], P.flow[cur], P.flow[cur ^ 1], P.cost, P.sx, P.sy, s,
                                              pd, plan.doubleProp, rs, x, y);
            }
            cur ^= 1;
            if (!grid_sync(gs, gridDim.x, plan.spin_limit, ++phase)) return;
        }
        pd = -pd;
    }
}

__global__ void __launch_bounds__(256) k_b_downsample(BatchDev bd, int cur)
{
    const unsigned int tile = bd.pre_in[bd.lo] + blockIdx.x;
    const int i = find_pair(bd.pre_in, bd.lo, bd.hi, tile);
    const PairDev& P = bd.pairs[i];
    const unsigned int t = tile - bd.pre_in[i];
    const int x = (int)(t % P.first_in_tile_x) * TX + threadIdx.x, y = (int)(t / P.first_in_tile_x) * TY + threadIdx.y;
    if (x >= P.sx_in || y >= P.sy_in) return;
    const size_t ni = (size_t)P.sx_in * P.sy_in;
    if (P.sx == P.sx_in && P.sy == P.sy_in) {
        const uint32_t f = P.flow[cur][(size_t)y * P.sx + x];
        P.flow_in[(size_t)y * P.sx_in + x] = (float)lo16(f);
        P.flow_in[ni + (size_t)y * P.sx_in + x] = (float)hi16(f);
        return;
    }
    downsample_px(P.flow[cur], P.flow_in, P.flow_in + ni, P.sx, P.sy, P.sx_in, P.taps, P.P, P.mx, P.my, P.nnx, P.nny,
                  x, y);
}

// Self-test of the bounded barrier: `blocks` blocks wait for `expect` arrivals.
__global__ void k_barrier_selftest(GridSync* gs, unsigned int expect, unsigned long long limit)
{
    grid_sync(gs, expect, limit, 1);
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

struct bm_batch {
    std::vector<bm_params> prm;
    uint32_t count = 0;
    uint32_t N = 0, nsp = 1, iterations = 0, jfMax = 0;
    int doubleProp = 1, filter = 1, rng = BM_RNG_XORWOW;
    unsigned long long seed = 0;
    cudaStream_t own_stream = nullptr, stream = nullptr;
    char* arena = nullptr;
    size_t arena_bytes = 0;
    std::vector<PairDev> pairs;   // host copy (device addresses)
    PairDev* d_pairs = nullptr;
    unsigned int* d_pre = nullptr;   // 3 prefix arrays of count+1
    std::vector<unsigned int> pre_up, pre_in, pre_tri;
    GridSync* d_sync = nullptr;
    size_t frames_offset = 0, frames_bytes = 0;   // packed input frames inside the arena
    size_t flows_offset = 0, flows_bytes = 0;     // packed refined flows (U,V per pair)
    std::vector<size_t> frame_off, flow_off;
    std::vector<uint32_t> order;   // internal index -> caller's pair index (ascending working set)
    std::vector<uint32_t> pos;     // caller's pair index -> internal index
    std::vector<size_t> ws;        // working set of each pair (internal order), bytes
    std::vector<PatternOffsets> pattern_off;  // per pair (internal order), for the per-pair descriptor launches
    std::vector<PatternOffsets> pattern_off_pad;  // the same for the edge-replicated up-sampled image
    int max_fsize = 1, max_tri_s = 0;
    size_t tri_smem = 0;
    int coop_blocks_per_sm = 0, num_sms = 0;
    bm_batch_schedule sched{};
    cudaGraphExec_t graph_exec = nullptr;
    cudaGraph_t graph = nullptr;
    bool graph_valid = false;
    uint64_t launches = 0;
    // learned proposal (bm_batch_set_proposal): per-pair schedule only
    bm_net* net = nullptr;
    float net_logit_min = 0.0f;
    uint32_t net_iterations = 0, net_jfMax = 0;
    uint32_t net_reduce = 1;   // bm_batch_set_proposal_reduce: cells of 4 * net_reduce input pixels
    uint32_t local_steps = 0, local_radius = 1;   // bm_batch_set_local_steps
    float* d_pred = nullptr;   // [h4][w4][3] of the pair being seeded (pairs run in stream order)
    // concurrent branches of the per-pair schedule (bm_batch_schedule.streams):
    // streams forked from and joined back into the batch stream, and for a proposal
    // one network copy and prediction buffer per extra branch
    std::vector<cudaStream_t> branch;
    std::vector<cudaEvent_t> branch_done;
    cudaEvent_t fork_ev = nullptr;
    std::vector<bm_net*> net_copy;
    std::vector<float*> pred_copy;
};

namespace {

bm_status bfail(bm_status st, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    bmk::set_error_text(buf);
    return st;
}

#define BB_CUDA(call)                                                                                     \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return bfail(BM_ERR_CUDA, "%s (%s:%d)", cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

BatchDev batch_dev(const bm_batch* b, int lo, int hi)
{
    BatchDev bd;
    bd.pairs = b->d_pairs;
    bd.pre_up = b->d_pre;
    bd.pre_in = b->d_pre + (b->count + 1);
    bd.pre_tri = b->d_pre + 2 * (b->count + 1);
    bd.lo = lo;
    bd.hi = hi;
    bd.N = (int)b->N;
    return bd;
}

// Consecutive runs of pairs (internal order: ascending working set) whose working
// sets add up to at most `budget` bytes; a pair larger than the budget is a wave of
// its own.  budget 0: one wave.
std::vector<std::pair<int, int>> make_waves(const bm_batch* b, uint64_t budget)
{
    std::vector<std::pair<int, int>> w;
    if (budget == 0) {
        w.push_back({0, (int)b->count});
        return w;
    }
    int lo = 0;
    uint64_t acc = 0;
    for (int j = 0; j < (int)b->count; j++) {
        if (j > lo && acc + b->ws[j] > budget) {
            w.push_back({lo, j});
            lo = j;
            acc = 0;
        }
        acc += b->ws[j];
    }
    w.push_back({lo, (int)b->count});
    return w;
}

#define BB_NSP(nsp, ...)                                            \
    switch (nsp) {                                                  \
    case 1: { constexpr int NSP = 1; __VA_ARGS__; } break;          \
    case 2: { constexpr int NSP = 2; __VA_ARGS__; } break;          \
    case 4: { constexpr int NSP = 4; __VA_ARGS__; } break;          \
    case 8: { constexpr int NSP = 8; __VA_ARGS__; } break;          \
    case 16: { constexpr int NSP = 16; __VA_ARGS__; } break;        \
    default: return bfail(BM_ERR_INVALID, "bad descriptor stride"); \
    }

bm_status enqueue_wave(bm_batch* b, const bm_batch_schedule& s, int lo, int hi);

// Enqueue one batch step on b->stream (no synchronisation): every wave runs the
// whole pipeline before the next starts.
bm_status enqueue_step(bm_batch* b, const bm_batch_schedule& s)
{
    // The persistent form's barrier word: its error and phase fields start clear once
    // per step and stay set across the step's waves (each wave resets only the arrival
    // count and generation), so a barrier that gave up in any wave reaches check_sync.
    if (s.persistent && !s.per_pair) BB_CUDA(cudaMemsetAsync(b->d_sync, 0, sizeof(GridSync), b->stream));
    for (const auto& w : make_waves(b, s.wave_bytes)) {
        bm_status st = enqueue_wave(b, s, w.first, w.second);
        if (st != BM_OK) return st;
    }
    return BM_OK;
}

// One pair through the single-pair kernels (parameters in the launch, as a plain
// context runs it), into the batch's buffers.
bm_status enqueue_pair(bm_batch* b, const bm_batch_schedule& s, int j, cudaStream_t st, bm_net* net, float* d_pred)
{
    const PairDev& d = b->pairs[j];
    const size_t ni = (size_t)d.sx_in * d.sy_in;
    const bool resample = d.sx != d.sx_in || d.sy != d.sy_in;
    BB_CUDA(u8_to_f32(d.frame[0], d.guide, ni, st));
    int rev = 0;
    // descriptors from the edge-replicated up-sampled image while the pair's pattern
    // fits the margin its buffer was laid out with; from the dense image otherwise
    const bool padded = resample && d.rmax <= d.up_margin;
    const int pitch = d.sx + 2 * d.up_margin;
    for (int which = 0; which < 2; which++) {
        if (padded) {
            BB_CUDA(upsample_u8_pad(d.frame[which], d.up, pitch, d.up_margin, d.sx_in, d.sy_in, d.sx, d.sy, d.lx, d.ix,
                                    d.ly, d.iy, st));
            BB_CUDA(features_pad(d.up + (size_t)d.up_margin * pitch + d.up_margin, pitch, d.F[which], d.sx, d.sy,
                                 (int)b->nsp, b->pattern_off_pad[j], rev, st));
        } else {
            if (resample)
                BB_CUDA(upsample_u8(d.frame[which], d.up, d.sx_in, d.sy_in, d.sx, d.sy, d.lx, d.ix, d.ly, d.iy, st));
            else
                BB_CUDA(u8_to_f32(d.frame[which], d.up, ni, st));
            BB_CUDA(features(d.up, d.F[which], d.sx, d.sy, (int)b->N, (int)b->nsp, d.pat, d.rmax, b->pattern_off[j], rev,
                             st));
        }
        rev ^= s.snake ? 1 : 0;
    }
    int cur = 0;
    uint32_t iterations = b->iterations, jfMax = b->jfMax;
    if (net) {
        // the proposal for this pair, then the seeded initialisation (bm_seed's rule)
        const uint32_t red = b->net_reduce;
        const uint32_t w4 = (uint32_t)d.sx_in / red / 4, h4 = (uint32_t)d.sy_in / red / 4;
        bm_status nst = bm_net_prepare_reduced(net, 0, d.frame[0], d.frame[1], (uint32_t)d.sx_in, (uint32_t)d.sy_in, red,
                                               st);
        if (nst == BM_OK) nst = bm_net_forward(net, 1, h4, w4, d_pred, st);
        if (nst != BM_OK) return nst;
        const float cell = 4.0f * (float)red;
        const float scx = cell * (float)d.sx / (float)d.sx_in, scy = cell * (float)d.sy / (float)d.sy_in;
        BB_CUDA(seed_field(d.F[0], d.F[1], d.flow[cur], d.flow[cur ^ 1], d.cost, d.sx, d.sy, (int)b->nsp, 1, d_pred,
                           (int)w4, (int)h4, scx, scy, b->net_logit_min, st));
        iterations = b->net_iterations;
        if (b->net_jfMax) jfMax = b->net_jfMax;
        b->launches += 8;
        rev ^= s.snake ? 1 : 0;
        cur ^= 1;
        int r = (int)b->local_radius;
        for (uint32_t k = 0; k < b->local_steps; k++) {
            BB_CUDA(local_step(d.F[0], d.F[1], d.flow[cur], d.flow[cur ^ 1], d.cost, d.sx, d.sy, (int)b->nsp, r, rev, st));
            rev ^= s.snake ? 1 : 0;
            cur ^= 1;
            r = r > 1 ? r / 2 : 1;
        }
        b->launches += b->local_steps;
    } else {
        BB_CUDA(initialize(d.F[0], d.F[1], d.flow[cur], d.flow[cur ^ 1], d.cost, d.sx, d.sy, (int)b->nsp, 1, rev, st));
        rev ^= s.snake ? 1 : 0;
        cur ^= 1;
    }
    int pd = -1;
    int levels = 0;
    for (int q = (int)jfMax; q > 0; q /= 2) levels++;
    for (uint32_t it = 0; it < iterations; it++) {
        int lvl = 0;
        for (int q = (int)jfMax; q > 0; q /= 2, lvl++) {
            RsArgs rs;
            rs.enabled = lvl == levels - 1;
            rs.mode = b->rng;
            rs.seed = b->seed;
            rs.call = it;
            rs.dist = d.dist;
            BB_CUDA(jump_level(d.F[0], d.F[1], d.flow[cur], d.flow[cur ^ 1], d.cost, d.sx, d.sy, (int)b->nsp, q, pd,
                               b->doubleProp, rs, rev, st));
            rev ^= s.snake ? 1 : 0;
            cur ^= 1;
        }
        pd = -pd;
    }
    if (resample) {
        BB_CUDA(downsample(d.flow[cur], d.flow_in, d.flow_in + ni, d.sx, d.sy, d.sx_in, d.sy_in, d.taps, d.P, d.mx,
                           d.my, d.nnx, d.nny, st));
    } else {
        BB_CUDA(flow_to_planes(d.flow[cur], d.flow_in, d.flow_in + ni, ni, st));
    }
    b->launches += 6 + (uint64_t)iterations * levels - (net ? 1 : 0);
    return BM_OK;
}

bm_status enqueue_refine(bm_batch* b, int lo, int hi);
bm_status enqueue_refine_pair(bm_batch* b, int j, cudaStream_t st);

// The per-pair schedule over pairs [lo, hi).  With k > 1 streams the pairs are
// dealt to k branches (largest first, each to the branch with the least work so
// far) that fork from the batch stream and join back into it; each pair's whole
// pipeline, refinement included, stays on its branch.
bm_status enqueue_per_pair(bm_batch* b, const bm_batch_schedule& s, int lo, int hi)
{
    const int k = std::min<int>((int)s.streams, (int)b->branch.size() + 1);
    if (k <= 1) {
        for (int j = lo; j < hi; j++) {
            bm_status st = enqueue_pair(b, s, j, b->stream, b->net, b->d_pred);
            if (st != BM_OK) return st;
        }
        return enqueue_refine(b, lo, hi);
    }
    std::vector<cudaStream_t> bs(k);
    bs[0] = b->stream;
    for (int i = 1; i < k; i++) bs[i] = b->branch[i - 1];
    BB_CUDA(cudaEventRecord(b->fork_ev, b->stream));
    for (int i = 1; i < k; i++) BB_CUDA(cudaStreamWaitEvent(bs[i], b->fork_ev, 0));
    std::vector<uint64_t> load(k, 0);
    std::vector<std::vector<int>> deal(k);
    for (int j = hi - 1; j >= lo; j--) {
        const int i = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[i] += b->ws[j];
        deal[i].push_back(j);
    }
    for (int i = 0; i < k; i++) {
        bm_net* net = b->net ? (i == 0 ? b->net : b->net_copy[i - 1]) : nullptr;
        float* pred = i == 0 ? b->d_pred : (b->net ? b->pred_copy[i - 1] : nullptr);
        for (int j : deal[i]) {
            bm_status st = enqueue_pair(b, s, j, bs[i], net, pred);
            if (st == BM_OK) st = enqueue_refine_pair(b, j, bs[i]);
            if (st != BM_OK) return st;
        }
    }
    for (int i = 1; i < k; i++) {
        BB_CUDA(cudaEventRecord(b->branch_done[i - 1], bs[i]));
        BB_CUDA(cudaStreamWaitEvent(b->stream, b->branch_done[i - 1], 0));
    }
    return BM_OK;
}

bm_status enqueue_wave(bm_batch* b, const bm_batch_schedule& s, int lo, int hi)
{
    if (s.per_pair) return enqueue_per_pair(b, s, lo, hi);
    const BatchDev bd = batch_dev(b, lo, hi);
    const unsigned int t_up = b->pre_up[hi] - b->pre_up[lo], t_in = b->pre_in[hi] - b->pre_in[lo];
    cudaStream_t st = b->stream;
    const dim3 blk(TX, TY);
    k_b_guide<<<t_in, blk, 0, st>>>(bd);
    BB_CUDA(cudaGetLastError());
    // descriptors: one launch per pair so each reads its sample offsets from the
    // parameter space (the single-pair kernel)
    for (int which = 0; which < 2; which++) {
        k_b_upsample<<<t_up, blk, 0, st>>>(bd, which);
        BB_CUDA(cudaGetLastError());
        for (int j = lo; j < hi; j++) {
            const PairDev& d = b->pairs[j];
            BB_CUDA(features(d.up, d.F[which], d.sx, d.sy, (int)b->N, (int)b->nsp, d.pat, d.rmax, b->pattern_off[j],
                             which, st));
        }
    }
    b->launches += 3 + 2 * (hi - lo);
    int cur = 0;
    if (s.persistent) {
        BB_CUDA(cudaMemsetAsync(b->d_sync, 0, offsetof(GridSync, error), st));  // arrived, generation
        MatchPlan plan;
        plan.iterations = (int)b->iterations;
        plan.jfMax = (int)b->jfMax;
        plan.doubleProp = b->doubleProp;
        plan.rng = b->rng;
        plan.seed = b->seed;
        plan.spin_limit = s.spin_limit ? s.spin_limit : (1ull << 24);
        plan.snake = s.snake;
        const int bps = std::max(1, std::min((int)s.blocks_per_sm, b->coop_blocks_per_sm));
        const unsigned int grid = std::min<unsigned int>((unsigned)(bps * b->num_sms), t_up);
        GridSync* gs = b->d_sync;
        void* args[] = {(void*)&bd, (void*)&plan, (void*)&gs};
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(grid);
        cfg.blockDim = blk;
        cfg.stream = st;
        cudaLaunchAttribute attr;
        attr.id = cudaLaunchAttributeCooperative;
        attr.val.cooperative = 1;
        cfg.attrs = &attr;
        cfg.numAttrs = 1;
        cudaError_t e = cudaSuccess;
        BB_NSP(b->nsp, (e = cudaLaunchKernelExC(&cfg, (const void*)k_b_match_persistent<NSP>, args)));
        BB_CUDA(e);
        b->launches += 1;
        int levels = 0;
        for (int q = (int)b->jfMax; q > 0; q /= 2) levels++;
        cur = (1 + (int)b->iterations * levels) & 1;
    } else {
        int rev = 0;
        BB_NSP(b->nsp, (k_b_initialize<NSP><<<t_up, blk, 0, st>>>(bd, cur, rev)));
        BB_CUDA(cudaGetLastError());
        b->launches++;
        cur ^= 1;
        int pd = -1;
        for (uint32_t it = 0; it < b->iterations; it++) {
            int levels = 0;
            for (int q = (int)b->jfMax; q > 0; q /= 2) levels++;
            int lvl = 0;
            for (int q = (int)b->jfMax; q > 0; q /= 2, lvl++) {
                rev = s.snake ? rev ^ 1 : 0;
                RsArgs rs;
                rs.enabled = lvl == levels - 1;
                rs.mode = b->rng;
                rs.seed = b->seed;
                rs.call = it;
                rs.dist = 0;
                if (rs.enabled) {
                    BB_NSP(b->nsp, (k_b_jump<NSP, true><<<t_up, blk, 0, st>>>(bd, cur, q, pd, b->doubleProp, rs, rev)));
                } else {
                    BB_NSP(b->nsp, (k_b_jump<NSP, false><<<t_up, blk, 0, st>>>(bd, cur, q, pd, b->doubleProp, rs, rev)));
                }
                BB_CUDA(cudaGetLastError());
                b->launches++;
                cur ^= 1;
            }
            pd = -pd;
        }
    }
    k_b_downsample<<<t_in, blk, 0, st>>>(bd, cur);
    BB_CUDA(cudaGetLastError());
    b->launches++;
    return enqueue_refine(b, lo, hi);
}

// Refinement: one launch per pair and stage, each sized to its pair (median window,
// trilateral window and shared memory).
bm_status enqueue_refine_pair(bm_batch* b, int j, cudaStream_t st)
{
    const PairDev& d = b->pairs[j];
    const bm_params& p = b->prm[b->order[j]];
    const size_t ni = (size_t)d.sx_in * d.sy_in;
    if (b->filter) {
        const int fs = d.fsize == 0 ? 1 : d.fsize;
        BB_CUDA(median_pass(d.flow_in, d.flow_in + ni, d.tmp, d.tmp + ni, 1, fs, d.sx_in, d.sy_in, st));
        BB_CUDA(median_pass(d.tmp, d.tmp + ni, d.flow_med, d.flow_med + ni, 0, fs, d.sx_in, d.sy_in, st));
        BB_CUDA(trilateral(d.flow_in, d.flow_in + ni, d.flow_med, d.flow_med + ni, d.guide, d.flow_out,
                           d.flow_out + ni, d.sx_in, d.sy_in, d.tri_s, p.sEPE * p.sEPE, p.sI * p.sI, p.sS * p.sS,
                           st));
        b->launches += 3;
    } else {
        BB_CUDA(cudaMemcpyAsync(d.flow_out, d.flow_in, 2 * ni * sizeof(float), cudaMemcpyDeviceToDevice, st));
    }
    return BM_OK;
}

bm_status enqueue_refine(bm_batch* b, int lo, int hi)
{
    for (int j = lo; j < hi; j++) {
        bm_status st = enqueue_refine_pair(b, j, b->stream);
        if (st != BM_OK) return st;
    }
    return BM_OK;
}

// Branch streams, events and (with a proposal) network copies for k - 1 extra
// branches; created outside any capture.
bm_status ensure_branches(bm_batch* b, int k)
{
    if (k > 8) return bfail(BM_ERR_LIMIT, "bm_batch: at most 8 concurrent streams");
    if (!b->fork_ev) BB_CUDA(cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming));
    while ((int)b->branch.size() < k - 1) {
        cudaStream_t st = nullptr;
        cudaEvent_t ev = nullptr;
        BB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        b->branch.push_back(st);
        BB_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
        b->branch_done.push_back(ev);
    }
    if (b->net) {
        size_t cells = 0;
        uint32_t mh = 0, mw = 0;
        for (const auto& p : b->prm) {
            cells = std::max(cells, (size_t)(p.sx_in / 4) * (p.sy_in / 4));
            mh = std::max(mh, p.sy_in / 4);
            mw = std::max(mw, p.sx_in / 4);
        }
        std::vector<float> params(bm_net_param_count());
        if ((int)b->net_copy.size() < k - 1) {
            bm_status st = bm_net_get_params(b->net, params.data(), params.size());
            if (st != BM_OK) return st;
        }
        while ((int)b->net_copy.size() < k - 1) {
            bm_net* n = nullptr;
            bm_status st = bm_net_create(1, mh, mw, &n);
            if (st == BM_OK) st = bm_net_set_params(n, params.data(), params.size());
            if (st != BM_OK) {
                if (n) bm_net_destroy(n);
                return st;
            }
            b->net_copy.push_back(n);
            float* pr = nullptr;
            if (bmk::device_malloc((void**)&pr, cells * 3 * sizeof(float)) != cudaSuccess)
                return bfail(BM_ERR_NOMEM, "bm_batch: prediction buffer allocation failed");
            b->pred_copy.push_back(pr);
        }
    }
    return BM_OK;
}

void drop_net_copies(bm_batch* b)
{
    for (bm_net* n : b->net_copy) bm_net_destroy(n);
    for (float* p : b->pred_copy) bmk::device_free(p);
    b->net_copy.clear();
    b->pred_copy.clear();
}

void destroy_graph(bm_batch* b)
{
    if (b->graph_exec) cudaGraphExecDestroy(b->graph_exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->graph_exec = nullptr;
    b->graph = nullptr;
    b->graph_valid = false;
}

bm_status capture_graph(bm_batch* b)
{
    destroy_graph(b);
    BB_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    bm_status st = enqueue_step(b, b->sched);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (st != BM_OK) {
        if (g) cudaGraphDestroy(g);
        return st;
    }
    if (e != cudaSuccess) return bfail(BM_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    b->graph = g;
    e = cudaGraphInstantiate(&b->graph_exec, g, 0);
    if (e != cudaSuccess) {
        destroy_graph(b);
        return bfail(BM_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    b->graph_valid = true;
    return BM_OK;
}

bm_status check_sync(bm_batch* b)
{
    if (!b->sched.persistent || b->sched.per_pair) return BM_OK;
    GridSync h;
    BB_CUDA(cudaMemcpyAsync(&h, b->d_sync, sizeof(h), cudaMemcpyDeviceToHost, b->stream));
    BB_CUDA(cudaStreamSynchronize(b->stream));
    if (h.error) return bfail(BM_ERR_TIMEOUT, "batched matching: a grid barrier timed out (phase %u)", h.where);
    return BM_OK;
}

std::string shape_key(const bm_batch* b)
{
    unsigned long long px = 0;
    for (const auto& p : b->prm) px += (unsigned long long)p.sx * p.sy;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, dev);
    std::ostringstream ss;
    ss << prop.name << "|pairs=" << b->count << "|N=" << b->N << "|it=" << b->iterations << "|jf=" << b->jfMax
       << "|upMpx=" << (px + 500000) / 1000000;
    if (b->net)
        ss << "|seeded=" << b->net_iterations << "/" << b->net_jfMax << "/ls" << b->local_steps << "r" << b->local_radius
           << "/x" << b->net_reduce;
    return ss.str();
}

}  // namespace

extern "C" {

bm_status bm_batch_create(const bm_params* pairs, uint32_t count, bm_batch** out)
{
    if (!pairs || !out || count == 0) return bfail(BM_ERR_INVALID, "bm_batch_create: empty batch");
    *out = nullptr;
    const bm_params& p0 = pairs[0];
    for (uint32_t i = 0; i < count; i++) {
        const bm_params& p = pairs[i];
        if (p.N != p0.N || p.iterations != p0.iterations || p.jfMax != p0.jfMax || p.doubleProp != p0.doubleProp ||
            p.filter != p0.filter || p.rng != p0.rng || p.seed != p0.seed)
            return bfail(BM_ERR_INVALID, "bm_batch_create: pair %u differs in N/iterations/jfMax/doubleProp/filter/rng",
                         i);
        if (p.N < 1 || p.N > BM_PATCH_MAX / 4 || p.fsize > BM_MAX_MEDIAN || p.sx == 0 || p.sy == 0 || p.sx_in == 0 ||
            p.sy_in == 0 || p.sx > 32767 || p.sy > 32767)
            return bfail(BM_ERR_LIMIT, "bm_batch_create: pair %u has parameters beyond the limits", i);
        if (std::ceil(p.sigma * 3) * 2 + 1 > BM_CONST_KERNEL_SIZE)
            return bfail(BM_ERR_LIMIT, "bm_batch_create: pair %u: Gaussian down-sampling filter too large", i);
    }
    bm_batch* b = new bm_batch();
    b->prm.assign(pairs, pairs + count);
    b->count = count;
    b->N = p0.N;
    b->nsp = feature_stride(p0.N);
    b->iterations = p0.iterations;
    b->jfMax = p0.jfMax;
    b->doubleProp = p0.doubleProp ? 1 : 0;
    b->filter = p0.filter ? 1 : 0;
    b->rng = (int)p0.rng;
    b->seed = p0.seed;
    b->sched.persistent = 0;
    b->sched.blocks_per_sm = 0;
    b->sched.snake = 1;
    b->sched.use_graph = 1;
    b->sched.spin_limit = 1ull << 24;
    b->sched.wave_bytes = 0;
    b->sched.per_pair = 0;
    {
        std::vector<size_t> ws_api(count);
        for (uint32_t i = 0; i < count; i++) {
            const size_t n = (size_t)pairs[i].sx * pairs[i].sy, ni = (size_t)pairs[i].sx_in * pairs[i].sy_in;
            ws_api[i] = n * (8 * (size_t)b->nsp + 14) + ni * 38;
        }
        b->order.resize(count);
        for (uint32_t i = 0; i < count; i++) b->order[i] = i;
        std::stable_sort(b->order.begin(), b->order.end(), [&](uint32_t a, uint32_t c) { return ws_api[a] < ws_api[c]; });
        b->pos.resize(count);
        b->ws.resize(count);
        for (uint32_t j = 0; j < count; j++) {
            b->pos[b->order[j]] = j;
            b->ws[j] = ws_api[b->order[j]];
        }
    }

    // layout
    struct Off {
        size_t frame[2], guide, up, F[2], flow[2], cost, fin, fmed, fout, tmp, pat, off, taps, lx, ix, ly, iy, nnx, nny;
    };
    std::vector<Off> offs(count);
    size_t cursor = 0;
    auto take = [&](size_t bytes) {
        const size_t o = cursor;
        cursor += align256(bytes);
        return o;
    };
    // packed inputs first (pair-major, frame 0 then frame 1) and packed outputs next,
    // so the e2e path moves each with one copy
    b->frames_offset = 0;
    b->frame_off.resize(2 * (size_t)count);
    size_t fcur = 0;
    for (uint32_t i = 0; i < count; i++)
        for (int k = 0; k < 2; k++) {
            b->frame_off[2 * i + k] = fcur;
            fcur += (size_t)pairs[i].sx_in * pairs[i].sy_in;
        }
    b->frames_bytes = fcur;
    cursor = align256(fcur);
    b->flows_offset = cursor;
    b->flow_off.resize(count);
    size_t ocur = 0;
    for (uint32_t i = 0; i < count; i++) {
        b->flow_off[i] = ocur;
        ocur += 2 * (size_t)pairs[i].sx_in * pairs[i].sy_in * sizeof(float);
    }
    b->flows_bytes = ocur;
    cursor += align256(ocur);
    // the up-sampled image of a re-sampled pair has room for an edge-replicated margin
    // as wide as its default pattern's largest offset (per-pair schedule)
    std::vector<int> margin(count, 0);
    {
        std::vector<float> pat(4 * (size_t)b->N);
        for (uint32_t i = 0; i < count; i++) {
            const bm_params& p = pairs[i];
            if (p.sx == p.sx_in && p.sy == p.sy_in) continue;
            bm_make_pattern(&p, 0, pat.data());
            for (float v : pat) margin[i] = std::max(margin[i], std::abs((int)v));
        }
    }
    for (uint32_t i = 0; i < count; i++) {
        const bm_params& p = pairs[i];
        const size_t n = (size_t)p.sx * p.sy, ni = (size_t)p.sx_in * p.sy_in;
        Off& o = offs[i];
        o.guide = take(ni * 4);
        o.up = take((p.sx + 2 * (size_t)margin[i]) * (p.sy + 2 * (size_t)margin[i]) * 4);
        o.F[0] = take(n * b->nsp * 4);
        o.F[1] = take(n * b->nsp * 4);
        o.flow[0] = take(n * 4);
        o.flow[1] = take(n * 4);
        o.cost = take(n * 2);
        o.fin = take(2 * ni * 4);
        o.fmed = take(2 * ni * 4);
        o.tmp = take(2 * ni * 4);
        o.pat = take((BM_PATCH_MAX / 4) * sizeof(int4));
        o.off = take((BM_PATCH_MAX / 4) * sizeof(int2));
        o.taps = take(BM_CONST_KERNEL_SIZE * 4);
        o.lx = take((size_t)p.sx * 6 * 4);
        o.ix = take((size_t)p.sx * 4);
        o.ly = take((size_t)p.sy * 6 * 4);
        o.iy = take((size_t)p.sy * 4);
        o.nnx = take((size_t)p.sx_in * 4);
        o.nny = take((size_t)p.sy_in * 4);
    }
    b->arena_bytes = cursor;
    cudaError_t e = bmk::device_malloc((void**)&b->arena, b->arena_bytes);
    if (e != cudaSuccess) {
        delete b;
        return bfail(BM_ERR_NOMEM, "bm_batch_create: cudaMalloc of %zu bytes failed: %s", cursor, cudaGetErrorString(e));
    }
    e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        bmk::device_free(b->arena);
        delete b;
        return bfail(BM_ERR_CUDA, "bm_batch_create: %s", cudaGetErrorString(e));
    }
    b->stream = b->own_stream;
    auto fail_clean = [&](bm_status st) {
        bm_batch_destroy(b);
        return st;
    };
    if (cudaMemsetAsync(b->arena, 0, b->arena_bytes, b->stream) != cudaSuccess)
        return fail_clean(bfail(BM_ERR_CUDA, "bm_batch_create: clearing the arena failed"));
    // tiles and descriptors
    b->pairs.resize(count);
    b->pre_up.assign(count + 1, 0);
    b->pre_in.assign(count + 1, 0);
    b->pre_tri.assign(count + 1, 0);
    std::vector<float> pattern(4 * (size_t)b->N);
    for (uint32_t j = 0; j < count; j++) {
        const uint32_t i = b->order[j];  // caller's index of internal pair j
        const bm_params& p = pairs[i];
        const Off& o = offs[i];
        PairDev& d = b->pairs[j];
        d.sx = (int)p.sx;
        d.sy = (int)p.sy;
        d.sx_in = (int)p.sx_in;
        d.sy_in = (int)p.sy_in;
        float taps[BM_CONST_KERNEL_SIZE];
        uint32_t P = 0;
        bm_gauss_taps(p.sigma, taps, &P);
        d.P = (int)P;
        d.fsize = (int)p.fsize;
        d.tri_s = (int)std::ceil(2.5 * (double)std::sqrt(p.sS * p.sS));
        d.dist = std::sqrt(std::ceil((float)p.sx * 0.5f / 3.0f));
        d.mx = (float)p.sx_in / (float)p.sx;
        d.my = (float)p.sy_in / (float)p.sy;
        const TriCoef tc = tri_coef(p.sEPE * p.sEPE, p.sI * p.sI, p.sS * p.sS);
        d.cE = tc.cE;
        d.cI = tc.cI;
        d.cS = tc.cS;
        d.first_up_tile_x = (d.sx + TX - 1) / TX;
        d.first_in_tile_x = (d.sx_in + TX - 1) / TX;
        d.first_tri_tile_x = (d.sx_in + TX - 1) / TX;
        b->pre_up[j + 1] = b->pre_up[j] + (unsigned)(d.first_up_tile_x * ((d.sy + TY - 1) / TY));
        b->pre_in[j + 1] = b->pre_in[j] + (unsigned)(d.first_in_tile_x * ((d.sy_in + TY - 1) / TY));
        b->pre_tri[j + 1] = b->pre_tri[j] + (unsigned)(d.first_tri_tile_x * ((d.sy_in + TRI_BY - 1) / TRI_BY));
        char* A = b->arena;
        d.frame[0] = reinterpret_cast<const uint8_t*>(A + b->frames_offset + b->frame_off[2 * i]);
        d.frame[1] = reinterpret_cast<const uint8_t*>(A + b->frames_offset + b->frame_off[2 * i + 1]);
        d.flow_out = reinterpret_cast<float*>(A + b->flows_offset + b->flow_off[i]);
        d.guide = reinterpret_cast<float*>(A + o.guide);
        d.up = reinterpret_cast<float*>(A + o.up);
        d.up_margin = margin[i];
        d.F[0] = reinterpret_cast<uint32_t*>(A + o.F[0]);
        d.F[1] = reinterpret_cast<uint32_t*>(A + o.F[1]);
        d.flow[0] = reinterpret_cast<uint32_t*>(A + o.flow[0]);
        d.flow[1] = reinterpret_cast<uint32_t*>(A + o.flow[1]);
        d.cost = reinterpret_cast<uint16_t*>(A + o.cost);
        d.flow_in = reinterpret_cast<float*>(A + o.fin);
        d.flow_med = reinterpret_cast<float*>(A + o.fmed);
        d.tmp = reinterpret_cast<float*>(A + o.tmp);
        d.pat = reinterpret_cast<const int4*>(A + o.pat);
        d.off = reinterpret_cast<const int2*>(A + o.off);
        d.taps = reinterpret_cast<const float*>(A + o.taps);
        d.lx = reinterpret_cast<const float*>(A + o.lx);
        d.ix = reinterpret_cast<const int*>(A + o.ix);
        d.ly = reinterpret_cast<const float*>(A + o.ly);
        d.iy = reinterpret_cast<const int*>(A + o.iy);
        d.nnx = reinterpret_cast<const unsigned int*>(A + o.nnx);
        d.nny = reinterpret_cast<const unsigned int*>(A + o.nny);
        b->max_fsize = std::max(b->max_fsize, (int)p.fsize);
        b->max_tri_s = std::max(b->max_tri_s, d.tri_s);
        if (cudaMemcpyAsync((void*)d.taps, taps, P * sizeof(float), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
            lanczos_tables((float*)d.lx, (int*)d.ix, d.sx_in, d.sx, b->stream) != cudaSuccess ||
            lanczos_tables((float*)d.ly, (int*)d.iy, d.sy_in, d.sy, b->stream) != cudaSuccess ||
            nn_table((unsigned int*)d.nnx, d.sx, d.sx_in, b->stream) != cudaSuccess ||
            nn_table((unsigned int*)d.nny, d.sy, d.sy_in, b->stream) != cudaSuccess)
            return fail_clean(bfail(BM_ERR_CUDA, "bm_batch_create: table set-up failed"));
        bm_make_pattern(&p, 0, pattern.data());
        bm_status st = bm_batch_set_pattern(b, i, pattern.data(), 4 * b->N);
        if (st != BM_OK) return fail_clean(st);
    }
    b->tri_smem = tri_smem_bytes(b->max_tri_s);
    if (b->filter && b->tri_smem > 220 * 1024)
        return fail_clean(bfail(BM_ERR_LIMIT, "bm_batch_create: spatial window %d too large for the batched filter",
                                b->max_tri_s));
    if (bmk::device_malloc((void**)&b->d_pairs, count * sizeof(PairDev)) != cudaSuccess ||
        bmk::device_malloc((void**)&b->d_pre, 3 * (count + 1) * sizeof(unsigned int)) != cudaSuccess ||
        bmk::device_malloc((void**)&b->d_sync, sizeof(GridSync)) != cudaSuccess)
        return fail_clean(bfail(BM_ERR_NOMEM, "bm_batch_create: descriptor allocation failed"));
    std::vector<unsigned int> pre;
    pre.insert(pre.end(), b->pre_up.begin(), b->pre_up.end());
    pre.insert(pre.end(), b->pre_in.begin(), b->pre_in.end());
    pre.insert(pre.end(), b->pre_tri.begin(), b->pre_tri.end());
    if (cudaMemcpyAsync(b->d_pairs, b->pairs.data(), count * sizeof(PairDev), cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(b->d_pre, pre.data(), pre.size() * sizeof(unsigned int), cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess ||
        cudaMemsetAsync(b->d_sync, 0, sizeof(GridSync), b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
        return fail_clean(bfail(BM_ERR_CUDA, "bm_batch_create: descriptor upload failed"));
    if (b->filter && ensure_trilateral_smem(b->max_tri_s) != cudaSuccess)
        return fail_clean(bfail(BM_ERR_CUDA, "bm_batch_create: shared-memory opt-in failed"));
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev);
    int occ = 0;
    cudaError_t oe = cudaSuccess;
    switch (b->nsp) {
    case 1: oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_b_match_persistent<1>, TX * TY, 0); break;
    case 2: oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_b_match_persistent<2>, TX * TY, 0); break;
    case 4: oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_b_match_persistent<4>, TX * TY, 0); break;
    case 8: oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_b_match_persistent<8>, TX * TY, 0); break;
    default: oe = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_b_match_persistent<16>, TX * TY, 0); break;
    }
    if (oe != cudaSuccess) return fail_clean(bfail(BM_ERR_CUDA, "occupancy query: %s", cudaGetErrorString(oe)));
    b->coop_blocks_per_sm = occ;
    b->sched.blocks_per_sm = (uint32_t)occ;
    *out = b;
    return BM_OK;
}

bm_status bm_batch_destroy(bm_batch* b)
{
    if (!b) return BM_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    destroy_graph(b);
    if (b->arena) bmk::device_free(b->arena);
    if (b->d_pairs) bmk::device_free(b->d_pairs);
    if (b->d_pre) bmk::device_free(b->d_pre);
    if (b->d_sync) bmk::device_free(b->d_sync);
    if (b->d_pred) bmk::device_free(b->d_pred);
    drop_net_copies(b);
    for (cudaStream_t st : b->branch) cudaStreamDestroy(st);
    for (cudaEvent_t ev : b->branch_done) cudaEventDestroy(ev);
    if (b->fork_ev) cudaEventDestroy(b->fork_ev);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return BM_OK;
}

uint32_t bm_batch_count(const bm_batch* b) { return b ? b->count : 0; }

bm_status bm_batch_set_stream(bm_batch* b, void* stream)
{
    if (!b) return bfail(BM_ERR_INVALID, "null batch");
    cudaStream_t s = stream ? (cudaStream_t)stream : b->own_stream;
    if (s != b->stream) {
        // work already queued on the old stream finishes before the new one's
        BB_CUDA(cudaStreamSynchronize(b->stream));
        destroy_graph(b);
    }
    b->stream = s;
    return BM_OK;
}

bm_status bm_batch_set_pattern(bm_batch* b, uint32_t pair, const float* h_pattern, uint32_t count)
{
    if (!b || !h_pattern || pair >= b->count) return bfail(BM_ERR_INVALID, "bm_batch_set_pattern: bad argument");
    if (count != 4 * b->N) return bfail(BM_ERR_INVALID, "bm_batch_set_pattern: expected 4*N values");
    std::vector<int4> pat(b->N);
    std::vector<int2> off(BM_PATCH_MAX / 4, make_int2(0, 0)), off_pad(BM_PATCH_MAX / 4, make_int2(0, 0));
    int rmax = 0;
    const uint32_t j = b->pos[pair];
    PairDev& d = b->pairs[j];
    const int sx = d.sx, pitch = d.sx + 2 * d.up_margin;
    for (uint32_t s = 0; s < b->N; s++) {
        int v[4];
        for (int k = 0; k < 4; k++) {
            v[k] = (int)h_pattern[4 * s + k];
            rmax = std::max(rmax, std::abs(v[k]));
        }
        pat[s] = make_int4(v[0], v[1], v[2], v[3]);
        off[s] = make_int2(v[0] + v[1] * sx, v[2] + v[3] * sx);
        off_pad[s] = make_int2(v[0] + v[1] * pitch, v[2] + v[3] * pitch);
    }
    d.rmax = rmax;
    if (b->pattern_off.size() != b->count) b->pattern_off.resize(b->count);
    if (b->pattern_off_pad.size() != b->count) b->pattern_off_pad.resize(b->count);
    std::memcpy(b->pattern_off[j].off, off.data(), sizeof(b->pattern_off[j].off));
    std::memcpy(b->pattern_off_pad[j].off, off_pad.data(), sizeof(b->pattern_off_pad[j].off));
    BB_CUDA(cudaMemcpyAsync((void*)d.pat, pat.data(), b->N * sizeof(int4), cudaMemcpyHostToDevice, b->stream));
    BB_CUDA(cudaMemcpyAsync((void*)d.off, off.data(), off.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
    if (b->d_pairs)
        BB_CUDA(cudaMemcpyAsync(b->d_pairs + j, &d, sizeof(PairDev), cudaMemcpyHostToDevice, b->stream));
    BB_CUDA(cudaStreamSynchronize(b->stream));
    return BM_OK;
}

bm_status bm_batch_frame_ptr(bm_batch* b, uint32_t pair, uint32_t which, uint8_t** d_ptr)
{
    if (!b || !d_ptr || pair >= b->count || which > 1) return bfail(BM_ERR_INVALID, "bm_batch_frame_ptr: bad argument");
    *d_ptr = reinterpret_cast<uint8_t*>(b->arena + b->frames_offset + b->frame_off[2 * pair + which]);
    return BM_OK;
}

bm_status bm_batch_load_frames(bm_batch* b, const uint8_t* packed, size_t bytes, int on_device)
{
    if (!b || !packed) return bfail(BM_ERR_INVALID, "bm_batch_load_frames: null argument");
    if (bytes != b->frames_bytes)
        return bfail(BM_ERR_INVALID, "bm_batch_load_frames: expected %zu bytes, got %zu", b->frames_bytes, bytes);
    BB_CUDA(cudaMemcpyAsync(b->arena + b->frames_offset, packed, bytes,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, b->stream));
    return BM_OK;
}

size_t bm_batch_frames_bytes(const bm_batch* b) { return b ? b->frames_bytes : 0; }
size_t bm_batch_flows_bytes(const bm_batch* b) { return b ? b->flows_bytes : 0; }

bm_status bm_batch_read_flows(bm_batch* b, float* packed, size_t bytes, int on_device)
{
    if (!b || !packed) return bfail(BM_ERR_INVALID, "bm_batch_read_flows: null argument");
    if (bytes != b->flows_bytes)
        return bfail(BM_ERR_INVALID, "bm_batch_read_flows: expected %zu bytes, got %zu", b->flows_bytes, bytes);
    BB_CUDA(cudaMemcpyAsync(packed, b->arena + b->flows_offset, bytes,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, b->stream));
    if (!on_device) BB_CUDA(cudaStreamSynchronize(b->stream));
    return BM_OK;
}

bm_status bm_batch_flow_ptr(bm_batch* b, uint32_t pair, float** d_u, float** d_v)
{
    if (!b || pair >= b->count || !d_u || !d_v) return bfail(BM_ERR_INVALID, "bm_batch_flow_ptr: bad argument");
    const PairDev& d = b->pairs[b->pos[pair]];
    const size_t ni = (size_t)d.sx_in * d.sy_in;
    *d_u = d.flow_out;
    *d_v = d.flow_out + ni;
    return BM_OK;
}

bm_status bm_batch_set_schedule(bm_batch* b, const bm_batch_schedule* s)
{
    if (!b || !s) return bfail(BM_ERR_INVALID, "bm_batch_set_schedule: null argument");
    if (b->net && !s->per_pair)
        return bfail(BM_ERR_INVALID, "bm_batch_set_schedule: a batch with a proposal runs the per-pair schedule");
    if (s->per_pair && s->streams > 1) {
        if (b->stream) BB_CUDA(cudaStreamSynchronize(b->stream));
        bm_status st = ensure_branches(b, (int)s->streams);
        if (st != BM_OK) return st;
    }
    b->sched = *s;
    if (b->sched.blocks_per_sm == 0 || (int)b->sched.blocks_per_sm > b->coop_blocks_per_sm)
        b->sched.blocks_per_sm = (uint32_t)b->coop_blocks_per_sm;
    destroy_graph(b);
    return BM_OK;
}

bm_status bm_batch_get_schedule(const bm_batch* b, bm_batch_schedule* s)
{
    if (!b || !s) return bfail(BM_ERR_INVALID, "bm_batch_get_schedule: null argument");
    *s = b->sched;
    return BM_OK;
}

bm_status bm_batch_run(bm_batch* b)
{
    if (!b) return bfail(BM_ERR_INVALID, "null batch");
    if (b->sched.use_graph) {
        if (!b->graph_valid) {
            bm_status st = capture_graph(b);
            if (st != BM_OK) return st;
        }
        BB_CUDA(cudaGraphLaunch(b->graph_exec, b->stream));
    } else {
        bm_status st = enqueue_step(b, b->sched);
        if (st != BM_OK) return st;
    }
    return BM_OK;
}

bm_status bm_batch_synchronize(bm_batch* b)
{
    if (!b) return bfail(BM_ERR_INVALID, "null batch");
    BB_CUDA(cudaStreamSynchronize(b->stream));
    return check_sync(b);
}

uint64_t bm_batch_launch_count(const bm_batch* b) { return b ? b->launches : 0; }

bm_status bm_batch_set_local_steps(bm_batch* b, uint32_t count, uint32_t first_radius)
{
    if (!b) return bfail(BM_ERR_INVALID, "null batch");
    if (count > 16 || (count && (first_radius < 1 || first_radius > 256)))
        return bfail(BM_ERR_INVALID, "bm_batch_set_local_steps: at most 16 steps, first radius 1..256");
    b->local_steps = count;
    b->local_radius = count ? first_radius : 1;
    destroy_graph(b);
    return BM_OK;
}

bm_status bm_batch_set_proposal(bm_batch* b, bm_net* net, float conf_threshold, uint32_t iterations, uint32_t jfMax)
{
    if (!b) return bfail(BM_ERR_INVALID, "null batch");
    if (net && !(conf_threshold > 0.0f && conf_threshold < 1.0f))
        return bfail(BM_ERR_INVALID, "bm_batch_set_proposal: confidence threshold must lie in (0, 1)");
    if (net) {
        size_t cells = 0;
        for (const auto& p : b->prm) {
            if (p.sx_in < 4 || p.sy_in < 4) return bfail(BM_ERR_LIMIT, "bm_batch_set_proposal: frame too small");
            cells = std::max(cells, (size_t)(p.sx_in / 4) * (p.sy_in / 4));
        }
        if (!b->d_pred && bmk::device_malloc((void**)&b->d_pred, cells * 3 * sizeof(float)) != cudaSuccess)
            return bfail(BM_ERR_NOMEM, "bm_batch_set_proposal: prediction buffer allocation failed");
        b->sched.per_pair = 1;
        b->sched.persistent = 0;
    }
    if (b->stream) BB_CUDA(cudaStreamSynchronize(b->stream));
    drop_net_copies(b);
    b->net = net;
    b->net_logit_min = net ? std::log(conf_threshold / (1.0f - conf_threshold)) : 0.0f;
    b->net_iterations = iterations;
    b->net_jfMax = jfMax;
    destroy_graph(b);
    if (net && b->sched.streams > 1) return ensure_branches(b, (int)b->sched.streams);
    return BM_OK;
}

bm_status bm_batch_set_proposal_reduce(bm_batch* b, uint32_t reduce)
{
    if (!b) return bfail(BM_ERR_INVALID, "null batch");
    if (reduce != 1 && reduce != 2 && reduce != 4)
        return bfail(BM_ERR_INVALID, "bm_batch_set_proposal_reduce: reduce must be 1, 2 or 4");
    for (const auto& p : b->prm)
        if (p.sx_in < 4 * reduce || p.sy_in < 4 * reduce)
            return bfail(BM_ERR_LIMIT, "bm_batch_set_proposal_reduce: frame too small");
    if (b->stream) BB_CUDA(cudaStreamSynchronize(b->stream));
    b->net_reduce = reduce;
    destroy_graph(b);
    return BM_OK;
}

// Times each candidate schedule on this batch (after one untimed run each) and keeps
// the fastest; with cache_path, a previous choice for the same shape is reused and
// new choices are appended (one JSON object per line: {"key": ..., schedule, "ms"}).
bm_status bm_batch_autotune(bm_batch* b, const char* cache_path, int reps, char* report, size_t report_len)
{
    if (!b) return bfail(BM_ERR_INVALID, "null batch");
    const std::string key = shape_key(b);
    if (cache_path) {
        std::ifstream in(cache_path);
        std::string line, hit;
        while (std::getline(in, line))
            if (line.find("\"key\": \"" + key + "\"") != std::string::npos) hit = line;
        if (!hit.empty()) {
            bm_batch_schedule s = b->sched;
            unsigned long long v;
            auto grab = [&](const char* name, unsigned long long& dst) {
                const std::string k = std::string("\"") + name + "\": ";
                const size_t pos = hit.find(k);
                if (pos == std::string::npos) return false;
                dst = std::strtoull(hit.c_str() + pos + k.size(), nullptr, 10);
                return true;
            };
            bool ok = true;
            ok &= grab("persistent", v) && ((s.persistent = (uint32_t)v), true);
            ok &= grab("blocks_per_sm", v) && ((s.blocks_per_sm = (uint32_t)v), true);
            ok &= grab("snake", v) && ((s.snake = (uint32_t)v), true);
            ok &= grab("use_graph", v) && ((s.use_graph = (uint32_t)v), true);
            ok &= grab("wave_bytes", v) && ((s.wave_bytes = v), true);
            ok &= grab("per_pair", v) && ((s.per_pair = (uint32_t)v), true);
            if (grab("streams", v)) s.streams = (uint32_t)v;
            if (ok) {
                bm_batch_set_schedule(b, &s);
                if (report) std::snprintf(report, report_len, "cached: %s", hit.c_str());
                return BM_OK;
            }
        }
    }
    std::vector<bm_batch_schedule> cands;
    const uint64_t MB = 1ull << 20;
    {
        bm_batch_schedule s = b->sched;
        s.per_pair = 1;
        s.persistent = 0;
        s.snake = 1;
        s.use_graph = 1;
        s.wave_bytes = 0;
        cands.push_back(s);
    }
    {
        const bm_batch_schedule base = cands.back();
        for (uint32_t k : {2u, 4u}) {   // pairs on concurrent branches of the graph
            bm_batch_schedule s = base;
            s.streams = k;
            cands.push_back(s);
        }
        bm_batch_schedule s = base;
        s.use_graph = 0;   // per-pair launches without the graph
        cands.push_back(s);
    }
    const uint64_t waves[4] = {0ull, 64 * MB, 96 * MB, 160 * MB};
    for (uint64_t wave : waves) {
        if (b->net) break;   // the proposal runs in the per-pair schedule only
        for (uint32_t persistent = 0; persistent <= 1; persistent++) {
            bm_batch_schedule s = b->sched;
            s.per_pair = 0;
            s.persistent = persistent;
            s.blocks_per_sm = (uint32_t)b->coop_blocks_per_sm;
            s.snake = 1;
            s.use_graph = 1;
            s.wave_bytes = wave;
            cands.push_back(s);
        }
    }
    if (reps < 1) reps = 3;
    double best_ms = 1e30;
    bm_batch_schedule best = b->sched;
    std::ostringstream rep;
    cudaEvent_t e0, e1;
    BB_CUDA(cudaEventCreate(&e0));
    BB_CUDA(cudaEventCreate(&e1));
    for (const auto& s : cands) {
        bm_batch_set_schedule(b, &s);
        bm_status st = bm_batch_run(b);
        if (st == BM_OK) st = bm_batch_synchronize(b);
        if (st != BM_OK) {
            rep << "{per_pair=" << s.per_pair << ",persistent=" << s.persistent << ",wave=" << (s.wave_bytes >> 20)
                << "MB: failed} ";
            continue;
        }
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < reps && st == BM_OK; r++) st = bm_batch_run(b);
        cudaEventRecord(e1, b->stream);
        if (st == BM_OK) st = bm_batch_synchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= reps;
        rep << "{per_pair=" << s.per_pair << ",streams=" << (s.streams > 1 ? s.streams : 1) << ",graph=" << s.use_graph
            << ",persistent=" << s.persistent << ",wave=" << (s.wave_bytes >> 20) << "MB: "
            << (st == BM_OK ? std::to_string(ms) : std::string("failed")) << " ms} ";
        if (st == BM_OK && ms < best_ms) {
            best_ms = ms;
            best = s;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    bm_batch_set_schedule(b, &best);
    if (cache_path) {
        std::ofstream out(cache_path, std::ios::app);
        out << "{\"key\": \"" << key << "\", \"persistent\": " << best.persistent << ", \"blocks_per_sm\": "
            << best.blocks_per_sm << ", \"snake\": " << best.snake << ", \"use_graph\": " << best.use_graph
            << ", \"wave_bytes\": " << best.wave_bytes << ", \"per_pair\": " << best.per_pair
            << ", \"streams\": " << best.streams << ", \"ms\": "
            << best_ms << "}\n";
    }
    if (report)
        std::snprintf(report, report_len, "%s-> per_pair=%u streams=%u graph=%u persistent=%u wave=%lluMB",
                      rep.str().c_str(), best.per_pair, best.streams > 1 ? best.streams : 1, best.use_graph,
                      best.persistent, (unsigned long long)(best.wave_bytes >> 20));
    return BM_OK;
}

bm_status bm_selftest_barrier(uint32_t blocks, uint32_t expect, uint64_t spin_limit, int* timed_out)
{
    if (!timed_out || blocks == 0 || blocks > 64) return bfail(BM_ERR_INVALID, "bm_selftest_barrier: bad argument");
    GridSync* gs = nullptr;
    BB_CUDA(cudaMalloc((void**)&gs, sizeof(GridSync)));  // self-test scratch, not engine state
    cudaMemset(gs, 0, sizeof(GridSync));
    void* args[] = {(void*)&gs, (void*)&expect, (void*)&spin_limit};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)k_barrier_selftest, dim3(blocks), dim3(32), args, 0, 0);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    GridSync h{};
    if (e == cudaSuccess) e = cudaMemcpy(&h, gs, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(gs);  // self-test scratch
    if (e != cudaSuccess) return bfail(BM_ERR_CUDA, "bm_selftest_barrier: %s", cudaGetErrorString(e));
    *timed_out = h.error ? 1 : 0;
    return h.error ? bfail(BM_ERR_TIMEOUT, "grid barrier gave up after %llu polls", (unsigned long long)spin_limit)
                   : BM_OK;
}

}  // extern "C"

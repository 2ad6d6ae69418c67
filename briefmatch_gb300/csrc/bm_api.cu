// bm_api.cu -- the C ABI of the engine: context (buffer ownership as in
// BriefMatch::setup, briefmatch.cpp:72-214), the stage entry points that stand in
// for the reference's CUDA_* launchers, and the one-frame pipeline of
// OFPipeline::processFrame (of_pipeline.cpp:241-333).
//
// Nothing here synchronises the device except calls that hand data back to the
// host; the reference synchronises after every launch (util_cuda.cu:185-275).
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "bm_internal.h"

namespace {

thread_local std::string g_last_error;

bm_status fail(bm_status st, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return st;
}

#define BM_CUDA(call)                                                                        \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return fail(BM_ERR_CUDA, "%s in %s at line %d", cudaGetErrorString(e_), __FILE__, \
                        __LINE__);                                                           \
    } while (0)

// Every kernel launch goes through BM_LAUNCH: it counts launches and, while
// profiling is on, brackets the launch with CUDA events on the context's stream.
#define BM_LAUNCH(ctx, name, call)                               \
    do {                                                         \
        cudaEvent_t a_ = nullptr, b_ = nullptr;                  \
        if ((ctx)->prof_on) prof_begin((ctx), &a_, &b_);         \
        BM_CUDA(call);                                           \
        (ctx)->launches++;                                       \
        if ((ctx)->prof_on) prof_end((ctx), (name), a_, b_);     \
    } while (0)

}  // namespace

void bmk::set_error_text(const char* msg) { g_last_error = msg ? msg : ""; }

struct bm_ctx {
    bm_params prm;
    uint32_t nsp = 1;
    size_t npix = 0, npix_in = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;

    // frames in a ring of three: [cur_frame] receives the next frame, [prev] holds the
    // previous one (a third slot lets a pipelined refinement keep reading its guide)
    uint8_t* d_u8[3] = {nullptr, nullptr, nullptr};
    float* d_frame[3] = {nullptr, nullptr, nullptr};
    int cur_frame = 0;
    int prev_frame() const { return (cur_frame + 2) % 3; }
    float* d_up = nullptr;   // dense up-sampled image (BM_BUF_UP), filled on request
    // working up-sampled image with an edge-replicated margin of up_margin pixels on
    // every side (at least the pattern's largest offset), row pitch up_pitch()
    float* d_upad = nullptr;
    int up_margin = 0;
    bool upad_valid = false;   // d_upad holds the current frame
    int up_pitch() const { return (int)prm.sx + 2 * up_margin; }
    float* upad_origin() const { return d_upad + (size_t)up_margin * up_pitch() + up_margin; }
    uint32_t* d_feat[2] = {nullptr, nullptr};
    int feat1 = 0;                           // d_feat[feat1] is FEAT1, d_feat[feat1^1] FEAT2
    uint32_t* d_flow[2] = {nullptr, nullptr};
    int flow_cur = 0;
    uint16_t* d_cost = nullptr;
    float* d_flow_in = nullptr;    // U then V, npix_in each (one of d_flow_in_buf)
    float* d_flow_in_buf[2] = {nullptr, nullptr};
    int flow_in_slot = 0;
    // pipelined bm_frame (bm_set_pipelined): refinement and output copies of a pair on
    // refine_stream, overlapping the next pair's matching on the context stream
    bool pipelined = false;
    cudaStream_t refine_stream = nullptr;
    cudaEvent_t ev_ready = nullptr;               // context stream: pair down-sampled
    cudaEvent_t ev_frame_free[3] = {};            // refine stream: guide frame slot released
    cudaEvent_t ev_flowin_free[2] = {};           // refine stream: down-sampled flow released
    cudaEvent_t ev_refined = nullptr;             // refine stream: last refinement and copies done
    float* d_flow_med = nullptr;
    float* d_flow_out = nullptr;
    float* d_tmp = nullptr;
    int4* d_pattern = nullptr;
    int pattern_rmax = 0;
    bmk::PatternOffsets pattern_off;       // linear offsets for width sx
    bmk::PatternOffsets pattern_off_pad;   // linear offsets for pitch up_pitch()
    float* d_taps = nullptr;
    float* d_lx = nullptr;
    int* d_ix = nullptr;
    float* d_ly = nullptr;
    int* d_iy = nullptr;
    unsigned int* d_nnx = nullptr;   // resizeNN source column per input column
    unsigned int* d_nny = nullptr;   // resizeNN source row per input row

    float dist = 0;          // random-search radius, briefmatch.cpp:271
    int tri_s = 0;           // trilateral half window, briefmatch_cuda.cu:266
    uint64_t rs_calls = 0;   // random-search calls made so far
    int pass_rev = 0;        // visiting order of the next full-frame pass (alternates)
    bool first_match = true; // BriefMatch::m_firstFrame
    bool primed = false;
    uint64_t launches = 0;

    // learned proposal (bm_set_proposal)
    bm_net* net = nullptr;
    float net_logit_min = 0.0f;
    uint32_t net_iterations = 0, net_jfMax = 0;
    uint32_t net_reduce = 1;   // bm_set_proposal_reduce: cells of 4 * net_reduce input pixels
    uint32_t local_steps = 0, local_radius = 1;   // bm_set_local_steps
    float* d_pred = nullptr;   // [h4][w4][3]
    uint32_t net_w4() const { return prm.sx_in / net_reduce / 4; }
    uint32_t net_h4() const { return prm.sy_in / net_reduce / 4; }
    // with bm_set_proposal_stream(ctx, 1) the network runs on a side stream,
    // concurrently with the frame's up-sampling and descriptors: it starts once both
    // 8-bit frames are on the device (ev_u8) and the seed waits for it (ev_net)
    cudaStream_t net_stream = nullptr;
    cudaEvent_t ev_u8 = nullptr, ev_net = nullptr;
    bool net_pending = false;   // ev_net recorded for this frame, not yet waited on
    bool net_side = false;      // bm_set_proposal_stream (measured slower beside the descriptors)

    // colour coding (bm_colors), allocated on first use
    int* d_color_word = nullptr;    // largest vector length, float bits
    uint8_t* d_rgb = nullptr;       // sx_in*sy_in*3 bytes

    struct ProfRec {
        const char* name;
        cudaEvent_t a, b;
    };
    struct ProfTotal {
        const char* name;
        uint64_t launches;
        double ms;
    };
    bool prof_on = false;
    std::vector<ProfRec> prof_pending;
    std::vector<cudaEvent_t> prof_pool;
    std::vector<ProfTotal> prof_totals;

    uint32_t* feat1_ptr() const { return d_feat[feat1]; }
    uint32_t* feat2_ptr() const { return d_feat[feat1 ^ 1]; }
};

namespace {

cudaEvent_t prof_event(bm_ctx* c)
{
    if (!c->prof_pool.empty()) {
        cudaEvent_t e = c->prof_pool.back();
        c->prof_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    return e;
}

void prof_begin(bm_ctx* c, cudaEvent_t* a, cudaEvent_t* b)
{
    *a = prof_event(c);
    *b = prof_event(c);
    if (*a) cudaEventRecord(*a, c->stream);
}

void prof_end(bm_ctx* c, const char* name, cudaEvent_t a, cudaEvent_t b)
{
    if (!a || !b) return;
    cudaEventRecord(b, c->stream);
    c->prof_pending.push_back({name, a, b});
}

// Fold finished launch records into the per-kernel totals (synchronises the stream).
cudaError_t prof_collect(bm_ctx* c)
{
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess && c->refine_stream) e = cudaStreamSynchronize(c->refine_stream);
    if (e != cudaSuccess) return e;
    for (auto& r : c->prof_pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, r.a, r.b);
        bool found = false;
        for (auto& t : c->prof_totals)
            if (std::strcmp(t.name, r.name) == 0) {
                t.launches++;
                t.ms += ms;
                found = true;
                break;
            }
        if (!found) c->prof_totals.push_back({r.name, 1, (double)ms});
        c->prof_pool.push_back(r.a);
        c->prof_pool.push_back(r.b);
    }
    c->prof_pending.clear();
    return cudaSuccess;
}

template <typename T>
bm_status dev_alloc(T** p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    cudaError_t e = bmk::device_malloc((void**)p, count * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        return fail(BM_ERR_NOMEM, "cudaMalloc of %zu bytes failed: %s", count * sizeof(T), cudaGetErrorString(e));
    }
    return BM_OK;
}

void release(bm_ctx* c)
{
    void* ptrs[] = {c->d_u8[0], c->d_u8[1], c->d_u8[2], c->d_pred, c->d_frame[0], c->d_frame[1], c->d_frame[2], c->d_up, c->d_upad,
                    c->d_feat[0], c->d_feat[1], c->d_flow[0], c->d_flow[1], c->d_cost, c->d_flow_in_buf[0],
                    c->d_flow_in_buf[1], c->d_flow_med, c->d_flow_out,
                    c->d_tmp, c->d_pattern, c->d_taps, c->d_lx, c->d_ix, c->d_ly, c->d_iy,
                    c->d_nnx, c->d_nny, c->d_color_word, c->d_rgb};
    for (void* p : ptrs)
        if (p) bmk::device_free(p);
    for (auto& r : c->prof_pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (cudaEvent_t e : c->prof_pool) cudaEventDestroy(e);
    cudaEvent_t evs[] = {c->ev_ready, c->ev_refined, c->ev_frame_free[0], c->ev_frame_free[1], c->ev_frame_free[2],
                         c->ev_flowin_free[0], c->ev_flowin_free[1], c->ev_u8, c->ev_net};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    if (c->refine_stream) cudaStreamDestroy(c->refine_stream);
    if (c->net_stream) cudaStreamDestroy(c->net_stream);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
}

// The context stream waits for the pipelined refinement queued so far (no-op otherwise).
cudaError_t join_refine(bm_ctx* c)
{
    if (!c->refine_stream) return cudaSuccess;
    return cudaStreamWaitEvent(c->stream, c->ev_refined, 0);
}

bm_status check_ctx(const bm_ctx* c)
{
    if (!c) return fail(BM_ERR_INVALID, "null context");
    return BM_OK;
}

int next_order(bm_ctx* c)
{
    const int r = c->pass_rev;
    c->pass_rev ^= 1;
    return r;
}

bmk::RsArgs rs_args(const bm_ctx* c, bool enabled)
{
    bmk::RsArgs rs;
    rs.enabled = enabled ? 1 : 0;
    rs.mode = (int)c->prm.rng;
    rs.seed = c->prm.seed;
    rs.call = c->rs_calls;
    rs.dist = c->dist;
    return rs;
}

bm_status features_into(bm_ctx* c, const float* d_up, uint32_t* F, bool padded = false)
{
    const bm_params& p = c->prm;
    if (padded) {
        BM_LAUNCH(c, "features", bmk::features_pad(d_up, c->up_pitch(), F, (int)p.sx, (int)p.sy, (int)c->nsp,
                                                   c->pattern_off_pad, next_order(c), c->stream));
        return BM_OK;
    }
    BM_LAUNCH(c, "features", bmk::features(d_up, F, (int)p.sx, (int)p.sy, (int)p.N, (int)c->nsp, c->d_pattern, c->pattern_rmax,
                               c->pattern_off, next_order(c), c->stream));
    return BM_OK;
}

// One jump-flood pass; the random search of this iteration is fused into the last
// level when fuse_rs is set (it reads only the pixel's own state).
bm_status propagate_pass(bm_ctx* c, int pd, bool fuse_rs, uint32_t jfMax)
{
    const bm_params& p = c->prm;
    int levels = 0;
    for (int step = (int)jfMax; step > 0; step /= 2) levels++;
    int lvl = 0;
    for (int step = (int)jfMax; step > 0; step /= 2, lvl++) {
        const bool last = (lvl == levels - 1);
        bmk::RsArgs rs = rs_args(c, fuse_rs && last);
        BM_LAUNCH(c, rs.enabled ? "jump_level_rs" : "jump_level", bmk::jump_level(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur], c->d_flow[c->flow_cur ^ 1],
                                     c->d_cost, (int)p.sx, (int)p.sy, (int)c->nsp, step, pd, p.doubleProp ? 1 : 0, rs,
                                     next_order(c), c->stream));
        c->flow_cur ^= 1;
    }
    if (fuse_rs) {
        if (levels == 0) {
            bmk::RsArgs rs = rs_args(c, true);
            BM_LAUNCH(c, "random_search", bmk::random_search(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur], c->d_cost, (int)p.sx,
                                            (int)p.sy, (int)c->nsp, rs, c->stream));
        }
        c->rs_calls++;
    }
    return BM_OK;
}

// Local refinement steps of the seeded schedule: radius local_radius, then halved
// down to 1 (bm_set_local_steps).
bm_status local_steps_impl(bm_ctx* c)
{
    const bm_params& p = c->prm;
    int r = (int)c->local_radius;
    for (uint32_t k = 0; k < c->local_steps; k++) {
        BM_LAUNCH(c, "local_step", bmk::local_step(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur],
                                                   c->d_flow[c->flow_cur ^ 1], c->d_cost, (int)p.sx, (int)p.sy,
                                                   (int)c->nsp, r, next_order(c), c->stream));
        c->flow_cur ^= 1;
        r = r > 1 ? r / 2 : 1;
    }
    return BM_OK;
}

// BriefMatch::match.  With a proposal network attached (and its prediction in
// d_pred), the initialisation is the seeded one and the iteration count and jump
// maximum are the proposal's.
bm_status match_impl(bm_ctx* c, const float* d_im2, bool seeded, bool padded = false)
{
    const bm_params& p = c->prm;
    bm_status st = features_into(c, d_im2, c->feat2_ptr(), padded);
    if (st != BM_OK) return st;
    const int first = (c->first_match || !p.tInit) ? 1 : 0;
    uint32_t iterations = p.iterations, jfMax = p.jfMax;
    if (seeded) {
        // a cell covers 4 * net_reduce input pixels; its vector is in those units
        const int w4 = (int)c->net_w4(), h4 = (int)c->net_h4();
        const float cell = 4.0f * (float)c->net_reduce;
        const float scx = cell * (float)p.sx / (float)p.sx_in, scy = cell * (float)p.sy / (float)p.sy_in;
        if (c->net_pending) {  // the proposal computed on the side stream
            BM_CUDA(cudaStreamWaitEvent(c->stream, c->ev_net, 0));
            c->net_pending = false;
        }
        BM_LAUNCH(c, "seed", bmk::seed_field(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur], c->d_flow[c->flow_cur ^ 1],
                                             c->d_cost, (int)p.sx, (int)p.sy, (int)c->nsp, first, c->d_pred, w4, h4, scx,
                                             scy, c->net_logit_min, c->stream));
        iterations = c->net_iterations;
        if (c->net_jfMax) jfMax = c->net_jfMax;
        c->flow_cur ^= 1;
        st = local_steps_impl(c);
        if (st != BM_OK) return st;
    } else {
        BM_LAUNCH(c, "initialize", bmk::initialize(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur], c->d_flow[c->flow_cur ^ 1],
                                     c->d_cost, (int)p.sx, (int)p.sy, (int)c->nsp, first, next_order(c), c->stream));
        c->flow_cur ^= 1;
    }
    int pd = -1;
    for (uint32_t it = 0; it < iterations; it++) {
        st = propagate_pass(c, pd, true, jfMax);
        if (st != BM_OK) return st;
        pd = -pd;
    }
    c->first_match = false;
    return BM_OK;
}

bm_status downsample_impl(bm_ctx* c)
{
    const bm_params& p = c->prm;
    float* U = c->d_flow_in;
    float* V = c->d_flow_in + c->npix_in;
    if (p.sx_in != p.sx || p.sy_in != p.sy) {
        const float mx = (float)p.sx_in / (float)p.sx;  // briefmatch.cpp:316-317
        const float my = (float)p.sy_in / (float)p.sy;
        BM_LAUNCH(c, "downsample", bmk::downsample(c->d_flow[c->flow_cur], U, V, (int)p.sx, (int)p.sy, (int)p.sx_in, (int)p.sy_in,
                                     c->d_taps, (int)p.P, mx, my, c->d_nnx, c->d_nny, c->stream));
    } else {
        // briefmatch.cpp:319-323: the converted field is the output
        BM_LAUNCH(c, "flow_to_planes", bmk::flow_to_planes(c->d_flow[c->flow_cur], U, V, c->npix, c->stream));
    }
    return BM_OK;
}

bm_status process_impl(bm_ctx* c, const float* d_prev_in)
{
    const bm_params& p = c->prm;
    const size_t n = c->npix_in;
    float* U = c->d_flow_in;
    float* V = U + n;
    if (p.filter) {
        if (!d_prev_in) return fail(BM_ERR_INVALID, "process: the guide frame is required when filtering");
        const int fs = p.fsize == 0 ? 1 : (int)p.fsize;
        BM_LAUNCH(c, "median_pass", bmk::median_pass(U, V, c->d_tmp, c->d_tmp + n, 1, fs, (int)p.sx_in, (int)p.sy_in, c->stream));
        BM_LAUNCH(c, "median_pass", bmk::median_pass(c->d_tmp, c->d_tmp + n, c->d_flow_med, c->d_flow_med + n, 0, fs, (int)p.sx_in,
                                      (int)p.sy_in, c->stream));
        BM_LAUNCH(c, "trilateral", bmk::trilateral(U, V, c->d_flow_med, c->d_flow_med + n, d_prev_in, c->d_flow_out,
                                     c->d_flow_out + n, (int)p.sx_in, (int)p.sy_in, c->tri_s, p.sEPE * p.sEPE,
                                     p.sI * p.sI, p.sS * p.sS, c->stream));
    } else {
        BM_CUDA(cudaMemcpyAsync(c->d_flow_out, c->d_flow_in, 2 * n * sizeof(float), cudaMemcpyDeviceToDevice, c->stream));
    }
    return BM_OK;
}

bm_status set_pattern_impl(bm_ctx* c, const float* h_pattern)
{
    const uint32_t N = c->prm.N;
    std::vector<int4> pat(N);
    int rmax = 0;
    for (uint32_t s = 0; s < N; s++) {
        // int() truncation as in briefmatch_cuda.cu:110-113
        int v[4];
        for (int k = 0; k < 4; k++) {
            v[k] = (int)h_pattern[4 * s + k];
            rmax = std::max(rmax, std::abs(v[k]));
        }
        pat[s] = make_int4(v[0], v[1], v[2], v[3]);
    }
    // the working up-sampled image's margin must cover the largest offset
    const bm_params& p = c->prm;
    // (the new image is allocated first: if that fails, the previous pattern and
    // working image stay in effect)
    if ((p.sx != p.sx_in || p.sy != p.sy_in) && (!c->d_upad || rmax > c->up_margin)) {
        float* fresh = nullptr;
        const bm_status st = dev_alloc(&fresh, (p.sx + 2 * (size_t)rmax) * (p.sy + 2 * (size_t)rmax));
        if (st != BM_OK) return st;
        const cudaError_t e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) {
            bmk::device_free(fresh);
            return fail(BM_ERR_CUDA, "bm_set_pattern: %s", cudaGetErrorString(e));
        }
        if (c->d_upad) bmk::device_free(c->d_upad);
        c->d_upad = fresh;
        c->up_margin = rmax;
        c->upad_valid = false;
    }
    std::memset(&c->pattern_off, 0, sizeof(c->pattern_off));
    std::memset(&c->pattern_off_pad, 0, sizeof(c->pattern_off_pad));
    const int sx = (int)p.sx, pitch = c->up_pitch();
    for (uint32_t s = 0; s < N; s++) {
        c->pattern_off.off[s] = make_int2(pat[s].x + pat[s].y * sx, pat[s].z + pat[s].w * sx);
        c->pattern_off_pad.off[s] = make_int2(pat[s].x + pat[s].y * pitch, pat[s].z + pat[s].w * pitch);
    }
    BM_CUDA(cudaMemcpyAsync(c->d_pattern, pat.data(), N * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
    BM_CUDA(cudaStreamSynchronize(c->stream));
    c->pattern_rmax = rmax;
    return BM_OK;
}

}  // namespace

extern "C" {

const char* bm_last_error(void) { return g_last_error.c_str(); }

const char* bm_version(void) { return "briefmatch_gb300 0.1 (sm_103a)"; }

bm_status bm_create(const bm_params* prm, bm_ctx** out)
{
    if (!prm || !out) return fail(BM_ERR_INVALID, "bm_create: null argument");
    *out = nullptr;
    const bm_params& p = *prm;
    // briefmatch.cpp:78-96
    if (p.N > BM_PATCH_MAX / 4)
        return fail(BM_ERR_LIMIT, "Feature length exceeds maximum value. Current size is %u and maximum is %d.", p.N,
                    BM_PATCH_MAX / 4);
    if (p.N < 1) return fail(BM_ERR_LIMIT, "Feature length must be at least 1.");
    if (p.fsize > BM_MAX_MEDIAN)
        return fail(BM_ERR_LIMIT, "Median filter size exceeds maximum value. Current size is %u and maximum is %d.",
                    p.fsize, BM_MAX_MEDIAN);
    if (std::ceil(p.sigma * 3) * 2 + 1 > BM_CONST_KERNEL_SIZE)
        return fail(BM_ERR_LIMIT,
                    "Maximum size of Gaussian down-sampling filter exceeded. Currently using sigma = %0.4f and "
                    "maximum is %0.4f.",
                    p.sigma, std::floor((BM_CONST_KERNEL_SIZE - 1.0f) / 2.0f) / 3.0f);
    if (p.sx == 0 || p.sy == 0 || p.sx_in == 0 || p.sy_in == 0)
        return fail(BM_ERR_INVALID, "bm_create: zero image size");
    // the field is int16 (briefmatch.h:140-141)
    if (p.sx > 32767 || p.sy > 32767)
        return fail(BM_ERR_LIMIT, "Up-sampled size %ux%u exceeds the int16 flow range.", p.sx, p.sy);
    if (p.rng != BM_RNG_XORWOW && p.rng != BM_RNG_PHILOX) return fail(BM_ERR_INVALID, "unknown rng %u", p.rng);
    const int tri_s = bmk::trilateral_half_window(p.sEPE, p.sI, p.sS, p.sx_in, p.sy_in);
    if (tri_s == -1) return fail(BM_ERR_INVALID, "bm_create: filter sigmas must be finite and positive");
    if (tri_s == -2)
        return fail(BM_ERR_LIMIT, "bm_create: trilateral window (sS = %g) is wider than twice the %ux%u frame",
                    (double)p.sS, p.sx_in, p.sy_in);

    bm_ctx* c = new bm_ctx();
    c->prm = p;
    c->nsp = bmk::feature_stride(p.N);
    c->npix = (size_t)p.sx * p.sy;
    c->npix_in = (size_t)p.sx_in * p.sy_in;
    float taps[BM_CONST_KERNEL_SIZE];
    uint32_t P = 0;
    bm_status st = bm_gauss_taps(p.sigma, taps, &P);
    if (st != BM_OK) {
        delete c;
        return fail(st, "Gaussian taps could not be built for sigma %f", p.sigma);
    }
    c->prm.P = P;
    c->dist = std::sqrt(std::ceil((float)p.sx * 0.5f / 3.0f));  // briefmatch.cpp:271
    c->tri_s = tri_s;  // briefmatch_cuda.cu:266

#define BM_TRY(x)           \
    do {                    \
        st = (x);           \
        if (st != BM_OK) {  \
            release(c);     \
            delete c;       \
            return st;      \
        }                   \
    } while (0)
    cudaError_t e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return fail(BM_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    c->stream = c->own_stream;
    const size_t n = c->npix, ni = c->npix_in;
    for (int k = 0; k < 3; k++) BM_TRY(dev_alloc(&c->d_u8[k], ni));
    BM_TRY(dev_alloc(&c->d_pred, (size_t)(p.sx_in / 4 + 1) * (p.sy_in / 4 + 1) * 3));
    for (int k = 0; k < 3; k++) BM_TRY(dev_alloc(&c->d_frame[k], ni));
    BM_TRY(dev_alloc(&c->d_up, n));
    BM_TRY(dev_alloc(&c->d_feat[0], n * c->nsp));
    BM_TRY(dev_alloc(&c->d_feat[1], n * c->nsp));
    BM_TRY(dev_alloc(&c->d_flow[0], n));
    BM_TRY(dev_alloc(&c->d_flow[1], n));
    BM_TRY(dev_alloc(&c->d_cost, n));
    BM_TRY(dev_alloc(&c->d_flow_in_buf[0], 2 * ni));
    BM_TRY(dev_alloc(&c->d_flow_in_buf[1], 2 * ni));
    c->d_flow_in = c->d_flow_in_buf[0];
    BM_TRY(dev_alloc(&c->d_flow_med, 2 * ni));
    BM_TRY(dev_alloc(&c->d_flow_out, 2 * ni));
    BM_TRY(dev_alloc(&c->d_tmp, 2 * ni));
    BM_TRY(dev_alloc(&c->d_pattern, BM_PATCH_MAX / 4));
    BM_TRY(dev_alloc(&c->d_taps, BM_CONST_KERNEL_SIZE));
    BM_TRY(dev_alloc(&c->d_lx, (size_t)p.sx * 6));
    BM_TRY(dev_alloc(&c->d_ix, (size_t)p.sx));
    BM_TRY(dev_alloc(&c->d_ly, (size_t)p.sy * 6));
    BM_TRY(dev_alloc(&c->d_iy, (size_t)p.sy));
    BM_TRY(dev_alloc(&c->d_nnx, (size_t)p.sx_in));
    BM_TRY(dev_alloc(&c->d_nny, (size_t)p.sy_in));
#undef BM_TRY
    auto cu = [&](cudaError_t err) -> bool {
        if (err != cudaSuccess) {
            fail(BM_ERR_CUDA, "bm_create: %s", cudaGetErrorString(err));
            release(c);
            delete c;
            return false;
        }
        return true;
    };
    // zeroed descriptors and field: the first pair of a sequence starts from defined state
    if (!cu(cudaMemsetAsync(c->d_feat[0], 0, n * c->nsp * sizeof(uint32_t), c->stream))) return BM_ERR_CUDA;
    if (!cu(cudaMemsetAsync(c->d_feat[1], 0, n * c->nsp * sizeof(uint32_t), c->stream))) return BM_ERR_CUDA;
    if (!cu(cudaMemsetAsync(c->d_flow[0], 0, n * sizeof(uint32_t), c->stream))) return BM_ERR_CUDA;
    if (!cu(cudaMemsetAsync(c->d_flow[1], 0, n * sizeof(uint32_t), c->stream))) return BM_ERR_CUDA;
    if (!cu(cudaMemsetAsync(c->d_cost, 0, n * sizeof(uint16_t), c->stream))) return BM_ERR_CUDA;
    if (!cu(cudaMemsetAsync(c->d_flow_out, 0, 2 * ni * sizeof(float), c->stream))) return BM_ERR_CUDA;
    for (int k = 0; k < 3; k++)
        if (!cu(cudaMemsetAsync(c->d_frame[k], 0, ni * sizeof(float), c->stream))) return BM_ERR_CUDA;
    if (!cu(cudaMemcpyAsync(c->d_taps, taps, P * sizeof(float), cudaMemcpyHostToDevice, c->stream))) return BM_ERR_CUDA;
    if (!cu(bmk::lanczos_tables(c->d_lx, c->d_ix, (int)p.sx_in, (int)p.sx, c->stream))) return BM_ERR_CUDA;
    if (!cu(bmk::lanczos_tables(c->d_ly, c->d_iy, (int)p.sy_in, (int)p.sy, c->stream))) return BM_ERR_CUDA;
    if (!cu(bmk::nn_table(c->d_nnx, (int)p.sx, (int)p.sx_in, c->stream))) return BM_ERR_CUDA;
    if (!cu(bmk::nn_table(c->d_nny, (int)p.sy, (int)p.sy_in, c->stream))) return BM_ERR_CUDA;
    c->launches += 4;
    std::vector<float> pattern(4 * (size_t)p.N);
    bm_make_pattern(&c->prm, 0, pattern.data());
    st = set_pattern_impl(c, pattern.data());
    if (st != BM_OK) {
        release(c);
        delete c;
        return st;
    }
    *out = c;
    return BM_OK;
}

bm_status bm_destroy(bm_ctx* c)
{
    if (!c) return BM_OK;
    cudaStreamSynchronize(c->stream);
    if (c->refine_stream) cudaStreamSynchronize(c->refine_stream);
    release(c);
    delete c;
    return BM_OK;
}

bm_status bm_get_params(const bm_ctx* c, bm_params* out)
{
    if (!c || !out) return fail(BM_ERR_INVALID, "bm_get_params: null argument");
    *out = c->prm;
    return BM_OK;
}

bm_status bm_set_stream(bm_ctx* c, void* stream)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    const cudaStream_t s = stream ? (cudaStream_t)stream : c->own_stream;
    // work already queued on the old stream (buffer clears, pattern upload, frames)
    // finishes before anything queued on the new one
    if (s != c->stream) {
        BM_CUDA(cudaStreamSynchronize(c->stream));
        if (c->refine_stream) BM_CUDA(cudaStreamSynchronize(c->refine_stream));
    }
    c->stream = s;
    return BM_OK;
}

bm_status bm_synchronize(bm_ctx* c)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    BM_CUDA(cudaStreamSynchronize(c->stream));
    if (c->refine_stream) BM_CUDA(cudaStreamSynchronize(c->refine_stream));
    return BM_OK;
}

bm_status bm_set_pipelined(bm_ctx* c, int on)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (on && !c->refine_stream) {
        BM_CUDA(cudaStreamCreateWithFlags(&c->refine_stream, cudaStreamNonBlocking));
        cudaEvent_t* evs[] = {&c->ev_ready, &c->ev_refined, &c->ev_frame_free[0], &c->ev_frame_free[1],
                              &c->ev_frame_free[2], &c->ev_flowin_free[0], &c->ev_flowin_free[1]};
        for (cudaEvent_t* e : evs) BM_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        // nothing of the refinement stream may start before the work queued so far
        BM_CUDA(cudaEventRecord(c->ev_ready, c->stream));
        BM_CUDA(cudaStreamWaitEvent(c->refine_stream, c->ev_ready, 0));
        BM_CUDA(cudaEventRecord(c->ev_refined, c->refine_stream));
    }
    if (!on && c->refine_stream) BM_CUDA(join_refine(c));
    c->pipelined = on != 0;
    return BM_OK;
}

bm_status bm_join(bm_ctx* c)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    BM_CUDA(join_refine(c));
    return BM_OK;
}

bm_status bm_set_pattern(bm_ctx* c, const float* h_pattern, uint32_t count)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!h_pattern) return fail(BM_ERR_INVALID, "bm_set_pattern: null pattern");
    if (count != 4 * c->prm.N)
        return fail(BM_ERR_INVALID, "bm_set_pattern: expected %u values (4*N), got %u", 4 * c->prm.N, count);
    return set_pattern_impl(c, h_pattern);
}

uint32_t bm_feature_stride(const bm_ctx* c) { return c ? c->nsp : 0; }

bm_status bm_read_buffer(bm_ctx* c, bm_buffer_id id, void* dst, size_t bytes, int dst_on_device)
{
    void* src = nullptr;
    size_t cap = 0;
    bm_status st = bm_buffer(c, id, &src, &cap);
    if (st != BM_OK) return st;
    if (!dst) return fail(BM_ERR_INVALID, "bm_read_buffer: null destination");
    if (bytes > cap) return fail(BM_ERR_INVALID, "bm_read_buffer: %zu bytes requested, buffer holds %zu", bytes, cap);
    BM_CUDA(join_refine(c));
    BM_CUDA(cudaMemcpyAsync(dst, src, bytes, dst_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            c->stream));
    if (!dst_on_device) BM_CUDA(cudaStreamSynchronize(c->stream));
    return BM_OK;
}

bm_status bm_write_buffer(bm_ctx* c, bm_buffer_id id, const void* src, size_t bytes, int src_on_device)
{
    void* dst = nullptr;
    size_t cap = 0;
    bm_status st = bm_buffer(c, id, &dst, &cap);
    if (st != BM_OK) return st;
    if (!src) return fail(BM_ERR_INVALID, "bm_write_buffer: null source");
    if (bytes > cap) return fail(BM_ERR_INVALID, "bm_write_buffer: %zu bytes given, buffer holds %zu", bytes, cap);
    BM_CUDA(join_refine(c));
    BM_CUDA(cudaMemcpyAsync(dst, src, bytes, src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                            c->stream));
    if (!src_on_device) BM_CUDA(cudaStreamSynchronize(c->stream));
    return BM_OK;
}

bm_status bm_buffer(bm_ctx* c, bm_buffer_id id, void** d_ptr, size_t* bytes)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!d_ptr) return fail(BM_ERR_INVALID, "bm_buffer: null output");
    const size_t n = c->npix, ni = c->npix_in;
    void* p = nullptr;
    size_t b = 0;
    switch (id) {
    case BM_BUF_FEAT1: p = c->feat1_ptr(); b = n * c->nsp * 4; break;
    case BM_BUF_FEAT2: p = c->feat2_ptr(); b = n * c->nsp * 4; break;
    case BM_BUF_FLOW: p = c->d_flow[c->flow_cur]; b = n * 4; break;
    case BM_BUF_COST: p = c->d_cost; b = n * 2; break;
    case BM_BUF_UP:
        if (c->upad_valid) {   // the dense copy of the working (edge-replicated) image
            const size_t w = (size_t)c->prm.sx * sizeof(float);
            BM_CUDA(cudaMemcpy2DAsync(c->d_up, w, c->upad_origin(), (size_t)c->up_pitch() * sizeof(float), w,
                                      c->prm.sy, cudaMemcpyDeviceToDevice, c->stream));
        }
        p = c->d_up;
        b = n * 4;
        break;
    case BM_BUF_FLOW_IN: p = c->d_flow_in; b = 2 * ni * 4; break;
    case BM_BUF_FLOW_MED: p = c->d_flow_med; b = 2 * ni * 4; break;
    case BM_BUF_FLOW_OUT: p = c->d_flow_out; b = 2 * ni * 4; break;
    case BM_BUF_FRAME: p = c->d_frame[c->cur_frame]; b = ni * 4; break;
    case BM_BUF_FRAME_PREV: p = c->d_frame[c->prev_frame()]; b = ni * 4; break;
    default: return fail(BM_ERR_INVALID, "bm_buffer: unknown id %d", (int)id);
    }
    *d_ptr = p;
    if (bytes) *bytes = b;
    return BM_OK;
}

bm_status bm_upsample(bm_ctx* c, const float* d_in, float* d_out)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!d_in || !d_out) return fail(BM_ERR_INVALID, "bm_upsample: null buffer");
    const bm_params& p = c->prm;
    BM_LAUNCH(c, "upsample_f32", bmk::upsample_f32(d_in, d_out, (int)p.sx_in, (int)p.sy_in, (int)p.sx, (int)p.sy, c->d_lx, c->d_ix,
                                   c->d_ly, c->d_iy, c->stream));
    return BM_OK;
}

bm_status bm_upsample_u8(bm_ctx* c, const uint8_t* d_in, float* d_out)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!d_in || !d_out) return fail(BM_ERR_INVALID, "bm_upsample_u8: null buffer");
    const bm_params& p = c->prm;
    BM_LAUNCH(c, "upsample_u8", bmk::upsample_u8(d_in, d_out, (int)p.sx_in, (int)p.sy_in, (int)p.sx, (int)p.sy, c->d_lx, c->d_ix,
                                  c->d_ly, c->d_iy, c->stream));
    return BM_OK;
}

bm_status bm_features(bm_ctx* c, const float* d_up, int slot)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!d_up) return fail(BM_ERR_INVALID, "bm_features: null image");
    if (slot != 0 && slot != 1) return fail(BM_ERR_INVALID, "bm_features: slot must be 0 or 1");
    return features_into(c, d_up, slot == 0 ? c->feat1_ptr() : c->feat2_ptr());
}

bm_status bm_initialize(bm_ctx* c, int first)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    const bm_params& p = c->prm;
    BM_LAUNCH(c, "initialize", bmk::initialize(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur], c->d_flow[c->flow_cur ^ 1],
                                 c->d_cost, (int)p.sx, (int)p.sy, (int)c->nsp, first ? 1 : 0, next_order(c), c->stream));
    c->flow_cur ^= 1;
    return BM_OK;
}

bm_status bm_propagate(bm_ctx* c, int pd)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    return propagate_pass(c, pd, false, c->prm.jfMax);
}

bm_status bm_random_search(bm_ctx* c)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    const bm_params& p = c->prm;
    bmk::RsArgs rs = rs_args(c, true);
    BM_LAUNCH(c, "random_search", bmk::random_search(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur], c->d_cost, (int)p.sx,
                                    (int)p.sy, (int)c->nsp, rs, c->stream));
    c->rs_calls++;
    return BM_OK;
}

bm_status bm_match(bm_ctx* c, const float* d_im1, const float* d_im2)
{
    (void)d_im1;
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!d_im2) return fail(BM_ERR_INVALID, "bm_match: null frame");
    return match_impl(c, d_im2, false);
}

bm_status bm_downsample(bm_ctx* c)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    BM_CUDA(join_refine(c));
    return downsample_impl(c);
}

bm_status bm_process(bm_ctx* c, const float* d_prev_in)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    BM_CUDA(join_refine(c));
    return process_impl(c, d_prev_in);
}

bm_status bm_swap(bm_ctx* c)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    c->feat1 ^= 1;
    return BM_OK;
}

bm_status bm_convert(bm_ctx* c, float* h_u, float* h_v)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!h_u || !h_v) return fail(BM_ERR_INVALID, "bm_convert: null output");
    BM_CUDA(join_refine(c));
    const size_t b = c->npix_in * sizeof(float);
    BM_CUDA(cudaMemcpyAsync(h_u, c->d_flow_out, b, cudaMemcpyDeviceToHost, c->stream));
    BM_CUDA(cudaMemcpyAsync(h_v, c->d_flow_out + c->npix_in, b, cudaMemcpyDeviceToHost, c->stream));
    BM_CUDA(cudaStreamSynchronize(c->stream));
    return BM_OK;
}

bm_status bm_colors(bm_ctx* c, uint8_t* rgb, int rgb_on_device)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!rgb) return fail(BM_ERR_INVALID, "bm_colors: null output");
    const size_t ni = c->npix_in;
    if (!c->d_color_word) {
        cudaError_t e = bmk::device_malloc((void**)&c->d_color_word, sizeof(int));
        if (e != cudaSuccess) return fail(BM_ERR_NOMEM, "bm_colors: %s", cudaGetErrorString(e));
    }
    uint8_t* out = rgb;
    if (!rgb_on_device) {
        if (!c->d_rgb) {
            cudaError_t e = bmk::device_malloc((void**)&c->d_rgb, 3 * ni);
            if (e != cudaSuccess) return fail(BM_ERR_NOMEM, "bm_colors: %s", cudaGetErrorString(e));
        }
        out = c->d_rgb;
    }
    BM_CUDA(join_refine(c));
    BM_LAUNCH(c, "flow_colors", bmk::flow_colors(c->d_flow_out, c->d_flow_out + ni, ni, c->prm.maxmot,
                                                 c->d_color_word, out, c->stream));
    if (!rgb_on_device) {
        BM_CUDA(cudaMemcpyAsync(rgb, c->d_rgb, 3 * ni, cudaMemcpyDeviceToHost, c->stream));
        BM_CUDA(cudaStreamSynchronize(c->stream));
    }
    return BM_OK;
}

bm_status bm_flow_colors(const float* d_u, const float* d_v, uint32_t width, uint32_t height, float max_motion,
                         uint8_t* d_rgb, void* stream)
{
    if (!d_u || !d_v || !d_rgb) return fail(BM_ERR_INVALID, "bm_flow_colors: null buffer");
    if (!(max_motion > 0) || !(max_motion < 3.0e38f))
        return fail(BM_ERR_INVALID, "bm_flow_colors: max_motion must be a finite positive number");
    const cudaError_t e = bmk::flow_colors(d_u, d_v, (size_t)width * height, max_motion, nullptr, d_rgb,
                                           static_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return fail(BM_ERR_CUDA, "bm_flow_colors: %s", cudaGetErrorString(e));
    return BM_OK;
}

bm_status bm_export_field(bm_ctx* c, int16_t* d_nx, int16_t* d_ny, float* d_dist)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    BM_LAUNCH(c, "export_field", bmk::export_field(c->d_flow[c->flow_cur], c->d_cost, d_nx, d_ny, d_dist, c->npix, (int)c->prm.N,
                                   c->stream));
    return BM_OK;
}

bm_status bm_import_field(bm_ctx* c, const int16_t* d_nx, const int16_t* d_ny, const uint16_t* d_cost)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!d_nx || !d_ny) return fail(BM_ERR_INVALID, "bm_import_field: null field");
    BM_LAUNCH(c, "import_field", bmk::import_field(d_nx, d_ny, d_cost, c->d_flow[c->flow_cur], c->d_cost, c->npix, c->stream));
    return BM_OK;
}

bm_status bm_normals(bm_ctx* c, uint64_t call, float* d_out)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!d_out) return fail(BM_ERR_INVALID, "bm_normals: null output");
    bmk::RsArgs rs = rs_args(c, true);
    rs.call = call;
    BM_LAUNCH(c, "normals", bmk::normals(reinterpret_cast<float2*>(d_out), (int)c->prm.sx, (int)c->prm.sy, rs, c->stream));
    return BM_OK;
}

bm_status bm_nn_indices(bm_ctx* c, uint32_t* h_x, uint32_t* h_y)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!h_x || !h_y) return fail(BM_ERR_INVALID, "bm_nn_indices: null output");
    BM_CUDA(cudaMemcpyAsync(h_x, c->d_nnx, c->prm.sx_in * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    BM_CUDA(cudaMemcpyAsync(h_y, c->d_nny, c->prm.sy_in * sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream));
    BM_CUDA(cudaStreamSynchronize(c->stream));
    return BM_OK;
}

bm_status bm_rng_position(bm_ctx* c, uint64_t* calls)
{
    if (check_ctx(c) || !calls) return fail(BM_ERR_INVALID, "bm_rng_position: null argument");
    *calls = c->rs_calls;
    return BM_OK;
}

bm_status bm_set_rng_position(bm_ctx* c, uint64_t calls)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    c->rs_calls = calls;
    return BM_OK;
}

bm_status bm_set_proposal(bm_ctx* c, bm_net* net, float conf_threshold, uint32_t iterations, uint32_t jfMax)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (net && !(conf_threshold > 0.0f && conf_threshold < 1.0f))
        return fail(BM_ERR_INVALID, "bm_set_proposal: confidence threshold must lie in (0, 1)");
    if (net && (c->prm.sx_in < 4 || c->prm.sy_in < 4)) return fail(BM_ERR_LIMIT, "bm_set_proposal: frame too small");
    if (net && !c->net_stream) {
        cudaError_t e = cudaStreamCreateWithFlags(&c->net_stream, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_u8, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_net, cudaEventDisableTiming);
        if (e != cudaSuccess) return fail(BM_ERR_CUDA, "bm_set_proposal: %s", cudaGetErrorString(e));
    }
    c->net = net;
    c->net_logit_min = net ? std::log(conf_threshold / (1.0f - conf_threshold)) : 0.0f;
    c->net_iterations = iterations;
    c->net_jfMax = jfMax;
    return BM_OK;
}

bm_status bm_set_proposal_reduce(bm_ctx* c, uint32_t reduce)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (reduce != 1 && reduce != 2 && reduce != 4)
        return fail(BM_ERR_INVALID, "bm_set_proposal_reduce: reduce must be 1, 2 or 4");
    if (c->prm.sx_in < 4 * reduce || c->prm.sy_in < 4 * reduce)
        return fail(BM_ERR_LIMIT, "bm_set_proposal_reduce: frame too small");
    c->net_reduce = reduce;
    return BM_OK;
}

bm_status bm_set_proposal_stream(bm_ctx* c, int side)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    c->net_side = side != 0;
    return BM_OK;
}

bm_status bm_set_local_steps(bm_ctx* c, uint32_t count, uint32_t first_radius)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (count > 16 || (count && (first_radius < 1 || first_radius > 256)))
        return fail(BM_ERR_INVALID, "bm_set_local_steps: at most 16 steps, first radius 1..256");
    c->local_steps = count;
    c->local_radius = count ? first_radius : 1;
    return BM_OK;
}

bm_status bm_local_step(bm_ctx* c, uint32_t radius)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (radius < 1 || radius > 256) return fail(BM_ERR_INVALID, "bm_local_step: radius 1..256");
    const bm_params& p = c->prm;
    BM_LAUNCH(c, "local_step", bmk::local_step(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur],
                                               c->d_flow[c->flow_cur ^ 1], c->d_cost, (int)p.sx, (int)p.sy, (int)c->nsp,
                                               (int)radius, next_order(c), c->stream));
    c->flow_cur ^= 1;
    return BM_OK;
}

bm_status bm_seed(bm_ctx* c, int first, const float* d_pred, uint32_t w4, uint32_t h4, float conf_threshold)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!d_pred || w4 == 0 || h4 == 0) return fail(BM_ERR_INVALID, "bm_seed: bad prediction");
    if (!(conf_threshold > 0.0f && conf_threshold < 1.0f))
        return fail(BM_ERR_INVALID, "bm_seed: confidence threshold must lie in (0, 1)");
    const bm_params& p = c->prm;
    const float scx = (float)p.sx / (float)w4, scy = (float)p.sy / (float)h4;
    BM_LAUNCH(c, "seed", bmk::seed_field(c->feat1_ptr(), c->feat2_ptr(), c->d_flow[c->flow_cur], c->d_flow[c->flow_cur ^ 1],
                                         c->d_cost, (int)p.sx, (int)p.sy, (int)c->nsp, first ? 1 : 0, d_pred, (int)w4,
                                         (int)h4, scx, scy, std::log(conf_threshold / (1.0f - conf_threshold)),
                                         c->stream));
    c->flow_cur ^= 1;
    return BM_OK;
}

bm_status bm_reset_sequence(bm_ctx* c)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    c->primed = false;
    c->first_match = true;
    return BM_OK;
}

uint64_t bm_launch_count(const bm_ctx* c) { return c ? c->launches : 0; }

bm_status bm_profile_enable(bm_ctx* c, int on)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    c->prof_on = on != 0;
    return BM_OK;
}

bm_status bm_profile_reset(bm_ctx* c)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    BM_CUDA(prof_collect(c));
    c->prof_totals.clear();
    return BM_OK;
}

bm_status bm_profile_read(bm_ctx* c, bm_kernel_stat* out, uint32_t cap, uint32_t* count)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!count) return fail(BM_ERR_INVALID, "bm_profile_read: null count");
    BM_CUDA(prof_collect(c));
    *count = (uint32_t)c->prof_totals.size();
    if (out)
        for (uint32_t i = 0; i < cap && i < *count; i++) {
            out[i].name = c->prof_totals[i].name;
            out[i].launches = c->prof_totals[i].launches;
            out[i].ms = c->prof_totals[i].ms;
        }
    return BM_OK;
}

bm_status bm_frame(bm_ctx* c, const uint8_t* frame, int frame_on_device, float* u, float* v, int out_on_device)
{
    if (check_ctx(c)) return BM_ERR_INVALID;
    if (!frame) return fail(BM_ERR_INVALID, "bm_frame: null frame");
    const bm_params& p = c->prm;
    const size_t ni = c->npix_in;
    const int slot = c->cur_frame, prev = c->prev_frame();
    // a pipelined refinement two frames back may still read this slot as its guide
    if (c->refine_stream) BM_CUDA(cudaStreamWaitEvent(c->stream, c->ev_frame_free[slot], 0));
    // of_pipeline.cpp:297 (8-bit here: a quarter of the reference's float copy); the
    // frame is kept for the next pair's proposal input
    uint8_t* d_u8 = c->d_u8[slot];
    BM_CUDA(cudaMemcpyAsync(d_u8, frame, ni, frame_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                            c->stream));
    const bool seeded = c->primed && c->net != nullptr;
    if (seeded && c->net_side) {
        // the proposal network on its side stream, from the previous and this frame,
        // while this stream up-samples and describes the frame; match_impl's seed waits
        const uint32_t w4 = c->net_w4(), h4 = c->net_h4();
        BM_CUDA(cudaEventRecord(c->ev_u8, c->stream));
        BM_CUDA(cudaStreamWaitEvent(c->net_stream, c->ev_u8, 0));
        bm_status nst = bm_net_prepare_reduced(c->net, 0, c->d_u8[prev], d_u8, p.sx_in, p.sy_in, c->net_reduce,
                                               c->net_stream);
        if (nst == BM_OK) nst = bm_net_forward(c->net, 1, h4, w4, c->d_pred, c->net_stream);
        if (nst != BM_OK) return nst;
        BM_CUDA(cudaEventRecord(c->ev_net, c->net_stream));
        c->net_pending = true;
        c->launches += 7;
    }
    float* cur = c->d_frame[slot];
    BM_LAUNCH(c, "u8_to_f32", bmk::u8_to_f32(d_u8, cur, ni, c->stream));
    // of_pipeline.cpp:301-310
    const float* up = cur;
    const bool padded = p.sx != p.sx_in || p.sy != p.sy_in;
    if (padded) {
        BM_LAUNCH(c, "upsample_u8", bmk::upsample_u8_pad(d_u8, c->d_upad, c->up_pitch(), c->up_margin, (int)p.sx_in,
                                                         (int)p.sy_in, (int)p.sx, (int)p.sy, c->d_lx, c->d_ix, c->d_ly,
                                                         c->d_iy, c->stream));
        up = c->upad_origin();
        c->upad_valid = true;
    }
    bm_status st;
    bool refine_async = false;
    if (!c->primed) {
        st = features_into(c, up, c->feat2_ptr(), padded);
        if (st != BM_OK) return st;
        BM_CUDA(join_refine(c));
        BM_CUDA(cudaMemsetAsync(c->d_flow_out, 0, 2 * ni * sizeof(float), c->stream));
        c->primed = true;
    } else {
        if (seeded && !c->net_side) {  // the network on the context stream, after up-sampling
            const uint32_t w4 = c->net_w4(), h4 = c->net_h4();
            st = bm_net_prepare_reduced(c->net, 0, c->d_u8[prev], d_u8, p.sx_in, p.sy_in, c->net_reduce, c->stream);
            if (st == BM_OK) st = bm_net_forward(c->net, 1, h4, w4, c->d_pred, c->stream);
            if (st != BM_OK) return st;
            c->launches += 7;
        }
        st = match_impl(c, up, seeded, padded);                   // of_pipeline.cpp:314
        if (st != BM_OK) return st;
        if (c->pipelined) {
            // the down-sampled flow alternates between two buffers; the refinement of
            // the pair before last must have released this one
            c->flow_in_slot ^= 1;
            c->d_flow_in = c->d_flow_in_buf[c->flow_in_slot];
            BM_CUDA(cudaStreamWaitEvent(c->stream, c->ev_flowin_free[c->flow_in_slot], 0));
        }
        st = downsample_impl(c);                                  // :319
        if (st != BM_OK) return st;
        if (c->pipelined) {
            // refinement (:324) and the output copies on the refinement stream, while
            // the context stream goes on with the next frame
            BM_CUDA(cudaEventRecord(c->ev_ready, c->stream));
            BM_CUDA(cudaStreamWaitEvent(c->refine_stream, c->ev_ready, 0));
            const cudaStream_t main = c->stream;
            c->stream = c->refine_stream;
            st = process_impl(c, c->d_frame[prev]);
            cudaError_t e = cudaSuccess;
            if (st == BM_OK) {
                e = cudaEventRecord(c->ev_flowin_free[c->flow_in_slot], c->refine_stream);
                if (e == cudaSuccess) e = cudaEventRecord(c->ev_frame_free[prev], c->refine_stream);
            }
            c->stream = main;
            if (st != BM_OK) return st;
            BM_CUDA(e);
            refine_async = true;
        } else {
            st = process_impl(c, c->d_frame[prev]);               // :324
            if (st != BM_OK) return st;
        }
    }
    // of_pipeline.cpp:331-333
    c->cur_frame = (c->cur_frame + 1) % 3;
    c->feat1 ^= 1;
    const cudaStream_t out_stream = refine_async ? c->refine_stream : c->stream;
    if (u || v) {
        const cudaMemcpyKind kind = out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
        if (u) BM_CUDA(cudaMemcpyAsync(u, c->d_flow_out, ni * sizeof(float), kind, out_stream));
        if (v) BM_CUDA(cudaMemcpyAsync(v, c->d_flow_out + ni, ni * sizeof(float), kind, out_stream));
        if (!out_on_device && !c->pipelined) BM_CUDA(cudaStreamSynchronize(c->stream));
    }
    if (refine_async) BM_CUDA(cudaEventRecord(c->ev_refined, c->refine_stream));
    return BM_OK;
}

}  // extern "C"

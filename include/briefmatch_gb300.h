/*
 * briefmatch_gb300.h -- C ABI of the GB300 BriefMatch flow engine.
 *
 * The engine replaces the reference's kernel layer (kernels/briefmatch_cuda.h:64-93,
 * kernels/util_cuda.h:114-129) and the device-side sequencing of BriefMatch
 * (briefmatch.cpp:72-352) and OFPipeline::processFrame (of_pipeline.cpp:241-333).
 * Each entry point names the reference function it stands in for.
 *
 * Conventions
 *   - Every call returns a bm_status; nothing throws across this boundary.  The
 *     text of the last error on the calling thread is bm_last_error().
 *   - Sizes are size_t / uint32_t; there is no int-sized allocation limit.
 *   - Arguments named d_* are device pointers, h_* host pointers.
 *   - Work is queued on the context's stream (bm_set_stream); calls that return
 *     host data synchronise that stream before returning.
 *   - A context owns its device buffers, its BRIEF sampling pattern and its
 *     down-sampling taps, so several contexts can coexist in one process (the
 *     reference keeps these in process-wide __constant__ memory).
 */
#ifndef BRIEFMATCH_GB300_H
#define BRIEFMATCH_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BM_PATCH_MAX 2048          /* briefmatch_cuda.h:62: 4 floats per sample, N <= 512 */
#define BM_MAX_MEDIAN 47           /* util_cuda.h:56 */
#define BM_CONST_KERNEL_SIZE 100   /* util_cuda.h:58 */

typedef enum bm_status {
    BM_OK = 0,
    BM_ERR_INVALID = 1,  /* null pointer, zero size, unknown id */
    BM_ERR_LIMIT = 2,    /* a parameter beyond a limit (BriefMatchException, briefmatch.cpp:78-96) */
    BM_ERR_CUDA = 3,     /* CUDA runtime error (CudaException, util_cuda.h:85-112) */
    BM_ERR_STATE = 4,    /* call out of order (BriefMatchException, briefmatch.cpp:251) */
    BM_ERR_NOMEM = 5,    /* device or host allocation failed */
    BM_ERR_TIMEOUT = 6,  /* a bounded device-side wait gave up */
    BM_ERR_IO = 7        /* file could not be read or written */
} bm_status;

/* Random stream used by the random search (briefmatch_cuda.cu:237-245). */
enum {
    BM_RNG_XORWOW = 0,   /* the reference stream: curand_init(pixel, 0, 0) + curand_normal */
    BM_RNG_PHILOX = 1    /* counter-based: Philox4x32-10 (subsequence = pixel) seeded by bm_params.seed */
};

/* BMParams, briefmatch.h:65-89 (same fields, same defaults), plus the RNG choice. */
typedef struct bm_params {
    uint32_t sx, sy;          /* up-sampled (matching) resolution */
    uint32_t sx_in, sy_in;    /* input resolution */
    uint32_t N;               /* descriptor length in bits, 2..512 */
    uint32_t iterations;      /* propagation + random-search rounds */
    uint32_t jfMax;           /* largest jump-flood step */
    uint32_t P;               /* Gaussian down-sampling taps (derived from sigma at create) */
    uint32_t fsize;           /* median window */
    float patchArea;          /* BRIEF sampling radius, up-sampled pixels */
    float sigma;              /* Gaussian down-sampling sigma, up-sampled pixels */
    float sEPE, sI, sS;       /* trilateral filter sigmas (flow, intensity, spatial) */
    float maxmot;             /* colour-coding clamp */
    int32_t doubleProp;       /* propagate in both directions per level */
    int32_t filter;           /* run median + trilateral refinement */
    int32_t tInit;            /* temporal initialisation from the previous pair */
    uint32_t rng;             /* BM_RNG_XORWOW or BM_RNG_PHILOX */
    uint64_t seed;            /* seed of the Philox stream */
} bm_params;

typedef struct bm_ctx bm_ctx;

/* Device buffers a context exposes (bm_buffer). */
typedef enum bm_buffer_id {
    BM_BUF_FEAT1 = 0,      /* uint32 descriptors of frame 1 (previous), [sx*sy][stride] */
    BM_BUF_FEAT2 = 1,      /* uint32 descriptors of frame 2 (current) */
    BM_BUF_FLOW = 2,       /* uint32 packed field: low 16 bits nx, high 16 bits ny (int16 each) */
    BM_BUF_COST = 3,       /* uint16 Hamming distance of the current field */
    BM_BUF_UP = 4,         /* float up-sampled current frame, sx*sy */
    BM_BUF_FLOW_IN = 5,    /* float2 planes U then V: down-sampled field, sx_in*sy_in each */
    BM_BUF_FLOW_MED = 6,   /* float planes U then V: median-filtered field */
    BM_BUF_FLOW_OUT = 7,   /* float planes U then V: refined output field */
    BM_BUF_FRAME = 8,      /* float current input frame, sx_in*sy_in */
    BM_BUF_FRAME_PREV = 9  /* float previous input frame, sx_in*sy_in */
} bm_buffer_id;

/* ---- parameters (host only) ------------------------------------------------ */

/* BMParams::BMParams, briefmatch.h:67-84. */
bm_status bm_params_default(bm_params* p);

/* Derivation of OFPipeline::setParams, of_pipeline.cpp:178-190: up-sampled size,
 * patch radius, down-sampling sigma, median size and spatial sigma from the input
 * size and the percentages given on the command line (ux/uy <= 0.1 select the
 * defaults 2.740/3.052 as at :178-179). */
bm_status bm_params_derive(bm_params* p, uint32_t width, uint32_t height, float ux, float uy,
                           float patchRad, float sigmaRad, float fsizeRad, float sSRad);

/* BRIEF sampling pattern, briefmatch.cpp:124-148: 4N values of sign(g)*g^2 with
 * g ~ N(0, 0.2), clamped to [-1,1] and scaled by patchArea.  The reference seeds
 * Boost's mt19937 from time(NULL); here the seed is explicit (std::mt19937_64). */
bm_status bm_make_pattern(const bm_params* p, uint64_t seed, float* h_pattern /* 4*N */);

/* Gaussian taps, briefmatch.cpp:153-172.  *P receives the tap count. */
bm_status bm_gauss_taps(float sigma, float* h_taps /* BM_CONST_KERNEL_SIZE */, uint32_t* P);

/* ---- context ------------------------------------------------------------------ */

/* BriefMatch::setup, briefmatch.cpp:72-214: checks limits, allocates every device
 * buffer, builds the taps and a default pattern (seed 0). */
bm_status bm_create(const bm_params* p, bm_ctx** out);

/* BriefMatch::clean, briefmatch.cpp:217-238. */
bm_status bm_destroy(bm_ctx* ctx);

/* BriefMatch::getParams, briefmatch.h:118 (P is the derived tap count). */
bm_status bm_get_params(const bm_ctx* ctx, bm_params* out);

/* Queue subsequent work on this cudaStream_t (NULL = the context's own stream).
 * Switching to another stream first waits for the work queued on the old one. */
bm_status bm_set_stream(bm_ctx* ctx, void* stream);
bm_status bm_synchronize(bm_ctx* ctx);

/* CUDA_copyPatchToConst, briefmatch_cuda.cu:376-379: install 4*N pattern values. */
bm_status bm_set_pattern(bm_ctx* ctx, const float* h_pattern, uint32_t count);

/* Pointer and byte size of one of the context's device buffers.  Their contents are
 * valid once the work queued on the context's stream is done.  BM_BUF_UP is a dense
 * sx*sy copy of the engine's working up-sampled image (which carries an
 * edge-replicated margin); bm_buffer queues that copy on the context's stream. */
bm_status bm_buffer(bm_ctx* ctx, bm_buffer_id id, void** d_ptr, size_t* bytes);

/* Copy bytes between a context buffer and caller memory (host or device memory
 * per the *_on_device flag).  Host copies complete before the call returns. */
bm_status bm_read_buffer(bm_ctx* ctx, bm_buffer_id id, void* dst, size_t bytes, int dst_on_device);
bm_status bm_write_buffer(bm_ctx* ctx, bm_buffer_id id, const void* src, size_t bytes, int src_on_device);

/* Words per descriptor in the context's layout (ceil(N/32) rounded up to 1,2,4,8,16). */
uint32_t bm_feature_stride(const bm_ctx* ctx);

/* ---- stages (device pointers; mirror the reference kernel layer) --------------- */

/* CUDA_resizeLanczos, util_cuda.cu:250-257: Lanczos-3 from sx_in x sy_in to sx x sy. */
bm_status bm_upsample(bm_ctx* ctx, const float* d_in, float* d_out);
/* The same from 8-bit input (the frame read of of_pipeline.cpp:279-285 fused in). */
bm_status bm_upsample_u8(bm_ctx* ctx, const uint8_t* d_in, float* d_out);

/* CUDA_binaryFeatures, briefmatch_cuda.cu:311-319: descriptors of the up-sampled
 * image d_up into FEAT1 (slot 0) or FEAT2 (slot 1). */
bm_status bm_features(bm_ctx* ctx, const float* d_up, int slot);

/* CUDA_initialize, briefmatch_cuda.cu:321-332. */
bm_status bm_initialize(bm_ctx* ctx, int first);

/* CUDA_propagate, briefmatch_cuda.cu:334-347: one jump-flood pass, direction pd. */
bm_status bm_propagate(bm_ctx* ctx, int pd);

/* CUDA_randomSearch, briefmatch_cuda.cu:349-360: one random candidate per pixel,
 * drawn from the next position of the context's random stream. */
bm_status bm_random_search(bm_ctx* ctx);

/* BriefMatch::match, briefmatch.cpp:248-293: descriptors of d_im2 into FEAT2, then
 * initialise and iterate.  d_im1 is accepted for signature parity and unused, as in
 * the reference (the kernels only read descriptors). */
bm_status bm_match(bm_ctx* ctx, const float* d_im1, const float* d_im2);

/* BriefMatch::downsample, briefmatch.cpp:296-324. */
bm_status bm_downsample(bm_ctx* ctx);

/* BriefMatch::process, briefmatch.cpp:327-352: median + trilateral filter guided by
 * d_prev_in, the previous input-resolution frame (float, 0..255). */
bm_status bm_process(bm_ctx* ctx, const float* d_prev_in);

/* BriefMatch::swap, briefmatch.cpp:240-245. */
bm_status bm_swap(bm_ctx* ctx);

/* BriefMatch::convert, briefmatch.cpp:355-370: copy the output field to the host. */
bm_status bm_convert(bm_ctx* ctx, float* h_u, float* h_v);

/* BriefMatch::computeColors, briefmatch.cpp:373-421, with the colour wheel of
 * util/colorcode.cpp:52-74, on the GPU: the output field (the one bm_convert
 * returns) coloured into rgb, sx_in*sy_in*3 bytes, R G B per pixel, row-major -- the
 * bytes of the reference's colour PNG.  Vectors are divided by params.maxmot when it
 * is > 0, else by the largest known vector length (0 counts as 1); unknown vectors
 * (|u| or |v| > 1e9, NaN; flowIO.cpp:35-39) are black.  rgb is a device pointer when
 * rgb_on_device, else host memory (the call then waits for the copy).  The arithmetic
 * follows the reference's float/double expressions without fused operations; its
 * float atan2 is the correctly rounded one (host math libraries differ from it by one
 * unit in the last place on some inputs, which moves a colour byte by one on rare
 * pixels). */
bm_status bm_colors(bm_ctx* ctx, uint8_t* rgb, int rgb_on_device);

/* No counterpart in the reference (it colours only its own context's field): the same
 * colour coding of any device field (d_u, d_v: width*height floats each) into d_rgb
 * (width*height*3 bytes), normalised by max_motion, which must be a finite positive
 * number; work is queued on `stream` (a cudaStream_t). */
bm_status bm_flow_colors(const float* d_u, const float* d_v, uint32_t width, uint32_t height, float max_motion,
                         uint8_t* d_rgb, void* stream);

/* The field in the reference's layout (sint NX, NY and float D = H/N,
 * briefmatch.h:139-141), written to device arrays of sx*sy elements. */
bm_status bm_export_field(bm_ctx* ctx, int16_t* d_nx, int16_t* d_ny, float* d_dist);

/* Load a field in the reference's layout into the context (recomputes nothing). */
bm_status bm_import_field(bm_ctx* ctx, const int16_t* d_nx, const int16_t* d_ny, const uint16_t* d_cost);

/* The N(0,1) pairs random-search call number `call` uses, as float2 per pixel. */
bm_status bm_normals(bm_ctx* ctx, uint64_t call, float* d_out /* 2*sx*sy */);

/* The source pixel resizeNN picks for every input column (h_x, sx_in values) and row
 * (h_y, sy_in values), util_cuda.cu:165-166.  The reference computes the index with
 * the device's fast division; so does the engine, and these tables expose it. */
bm_status bm_nn_indices(bm_ctx* ctx, uint32_t* h_x, uint32_t* h_y);

/* Position of the random stream: number of random-search calls made so far. */
bm_status bm_rng_position(bm_ctx* ctx, uint64_t* calls);
bm_status bm_set_rng_position(bm_ctx* ctx, uint64_t calls);

/* ---- many pairs at once ------------------------------------------------------------ */

/* A batch of frame pairs of uneven size (no counterpart in the reference, which
 * processes one pair at a time).  Every pair is computed exactly as a fresh context
 * would compute it (bm_create, then bm_frame on its first and second frame); all
 * pairs must share N, iterations, jfMax, doubleProp, filter and the random stream.
 * Each stage runs either as one launch over the union of all pairs' tiles or as
 * one launch per pair (bm_batch_schedule.per_pair); the matching phase can run as one
 * persistent cooperative launch with bounded grid barriers; a whole step can be
 * captured in a CUDA graph.  Frames and flows are packed in pair
 * order: frames = pair0 frame0, pair0 frame1, pair1 frame0, ... (uint8, sx_in*sy_in
 * each); flows = pair0 U, pair0 V, pair1 U, ... (float). */
typedef struct bm_batch bm_batch;

typedef struct bm_batch_schedule {
    uint32_t persistent;     /* matching phase as one persistent launch */
    uint32_t blocks_per_sm;  /* resident blocks per SM of the persistent launch (0 = maximum) */
    uint32_t snake;          /* alternate the tile order between passes */
    uint32_t use_graph;      /* capture the step in a CUDA graph and replay it */
    uint64_t spin_limit;     /* polls before a grid barrier gives up (BM_ERR_TIMEOUT) */
    uint64_t wave_bytes;     /* run pairs in waves whose working sets sum to at most this
                                (smallest pairs first, so a wave stays L2-resident); 0 = one wave */
    uint32_t per_pair;       /* every stage as a launch per pair (the single-pair kernels,
                                parameters in the launch) instead of union-of-tiles launches */
    uint32_t streams;        /* per-pair schedule: pairs dealt to this many concurrent streams
                                forked from and joined back into the batch stream (0, 1 = one);
                                with a proposal, each extra stream gets a copy of the network
                                taken when the schedule or the proposal is set */
} bm_batch_schedule;

bm_status bm_batch_create(const bm_params* pairs, uint32_t count, bm_batch** out);
bm_status bm_batch_destroy(bm_batch* b);
uint32_t bm_batch_count(const bm_batch* b);
bm_status bm_batch_set_stream(bm_batch* b, void* stream);
bm_status bm_batch_set_pattern(bm_batch* b, uint32_t pair, const float* h_pattern, uint32_t count);
size_t bm_batch_frames_bytes(const bm_batch* b);
size_t bm_batch_flows_bytes(const bm_batch* b);
bm_status bm_batch_frame_ptr(bm_batch* b, uint32_t pair, uint32_t which, uint8_t** d_ptr);
bm_status bm_batch_load_frames(bm_batch* b, const uint8_t* packed, size_t bytes, int on_device);
bm_status bm_batch_read_flows(bm_batch* b, float* packed, size_t bytes, int on_device);
bm_status bm_batch_flow_ptr(bm_batch* b, uint32_t pair, float** d_u, float** d_v);
bm_status bm_batch_set_schedule(bm_batch* b, const bm_batch_schedule* s);
bm_status bm_batch_get_schedule(const bm_batch* b, bm_batch_schedule* s);
/* Queue one step (all pairs) on the batch stream. */
bm_status bm_batch_run(bm_batch* b);
/* Wait for the step; BM_ERR_TIMEOUT if a grid barrier of the persistent launch gave up. */
bm_status bm_batch_synchronize(bm_batch* b);
uint64_t bm_batch_launch_count(const bm_batch* b);
/* Time the candidate schedules on this batch and keep the fastest.  cache_path (may be
 * NULL) is a file of JSON lines keyed by GPU and batch shape: a cached choice is reused
 * without timing, a new one is appended.  report receives a one-line summary. */
bm_status bm_batch_autotune(bm_batch* b, const char* cache_path, int reps, char* report, size_t report_len);

/* Seed every pair's matching with a proposal network (NULL detaches), as
 * bm_set_proposal does for a context: per pair, the network on its two frames, the
 * seeded initialisation, then `iterations` rounds with jump-flood maximum jfMax (0
 * keeps the batch's).  Pair i's result equals a fresh context with the same proposal
 * attached.  The batch switches to, and keeps, the per-pair schedule; the network
 * must have been created for the largest pair's (sx_in/4) x (sy_in/4) and must not be
 * used on another stream while the batch runs. */
typedef struct bm_net bm_net;
bm_status bm_batch_set_proposal(bm_batch* b, bm_net* net, float conf_threshold, uint32_t iterations, uint32_t jfMax);
/* The network's input reduction for every pair (bm_set_proposal_reduce); 1 by default. */
bm_status bm_batch_set_proposal_reduce(bm_batch* b, uint32_t reduce);
/* Local refinement steps after each pair's seeded initialisation (bm_set_local_steps). */
bm_status bm_batch_set_local_steps(bm_batch* b, uint32_t count, uint32_t first_radius);

/* Self-test of the bounded grid barrier: `blocks` co-resident blocks wait for `expect`
 * arrivals for at most spin_limit polls each.  With expect > blocks nobody can pass:
 * every block gives up, *timed_out is set and BM_ERR_TIMEOUT returned. */
bm_status bm_selftest_barrier(uint32_t blocks, uint32_t expect, uint64_t spin_limit, int* timed_out);

/* ---- test hooks on the device allocator (no counterpart in the reference) ----------
 * The reference turns any CUDA failure into a CudaException (HANDLE_ERROR,
 * util_cuda.h:102-112); these hooks let tests reach the engine's BM_ERR_NOMEM paths
 * and catch out-of-bounds writes.  All are host-only and off by default. */
/* The k-th device allocation of the library from now on fails as if the device were
 * out of memory (k = 0: none fails). */
void bm_debug_fail_alloc(uint64_t k);
/* Device allocations made so far, and those made and not yet freed. */
uint64_t bm_debug_alloc_count(void);
int64_t bm_debug_live_allocs(void);
/* While on, new allocations carry 256-byte guard bands before and after the buffer
 * (the buffer too starts filled with the guard byte 0xA5). */
void bm_debug_guard_bands(int on);
/* Synchronises the device and checks every live guard band: BM_ERR_STATE (with the
 * buffer and byte in bm_last_error) if a kernel wrote into one; *checked (may be
 * NULL) receives the number of guarded buffers. */
bm_status bm_debug_check_guards(uint64_t* checked);

/* ---- learned flow proposal ---------------------------------------------------------- */

/* No counterpart in the reference.  A 6-layer 3x3 convolutional network (32->32 x5,
 * 32->3; ReLU between; dilations 1, 2, 4, 8, 1, 1) on the two frames at quarter
 * resolution -- each frame's 4x4 pixel block of a cell as 16 input channels -- with
 * BF16 weights and activations and FP32 accumulation on the tensor cores, predicting
 * the flow (quarter-resolution pixels) and a confidence logit per cell.  Parameters
 * are one FP32 vector: for each layer W[cout][9][cin] then b[cout]. */
size_t bm_net_param_count(void);
bm_status bm_net_create(uint32_t max_batch, uint32_t max_h4, uint32_t max_w4, bm_net** out);
bm_status bm_net_destroy(bm_net* n);
bm_status bm_net_set_params(bm_net* n, const float* h_params, size_t count);
bm_status bm_net_get_params(bm_net* n, float* h_params, size_t count);
/* Input image b from two 8-bit W x H device frames (channel 4*j + i of cell (x, y):
 * pixel (4x + i, 4y + j) of frame 0 scaled to [-1, 1]; channels 16..31: frame 1). */
bm_status bm_net_prepare(bm_net* n, uint32_t b, const uint8_t* d_f0, const uint8_t* d_f1, uint32_t W, uint32_t H,
                         void* stream);
/* The same from the frames reduced by `reduce` (1, 2 or 4): reduced pixel (X, Y) is
 * the mean of input pixels (reduce*X + a, reduce*Y + b), a, b < reduce, rounded half
 * to even to an 8-bit value; the image is ((W / reduce) / 4) x ((H / reduce) / 4)
 * cells, each covering 4 * reduce input pixels.  reduce 1 is bm_net_prepare. */
bm_status bm_net_prepare_reduced(bm_net* n, uint32_t b, const uint8_t* d_f0, const uint8_t* d_f1, uint32_t W,
                                 uint32_t H, uint32_t reduce, void* stream);
/* Raw input: B images h x w, bf16 NHWC with 32 channels. */
bm_status bm_net_set_input(bm_net* n, const uint16_t* d_in, uint32_t B, uint32_t h, uint32_t w, void* stream);
/* Forward; d_out (may be NULL) receives [B][h][w][3] floats (u, v, confidence logit). */
bm_status bm_net_forward(bm_net* n, uint32_t B, uint32_t h, uint32_t w, float* d_out, void* stream);
/* Forward + loss against d_target ([B][h][w][3]: u, v, validity) + backward; with
 * lr > 0 also one Adam step.  d_grad_out (may be NULL) receives the FP32 gradient;
 * h_loss (may be NULL) receives (flow loss, confidence loss, confident fraction). */
bm_status bm_net_train_step(bm_net* n, uint32_t B, uint32_t h, uint32_t w, const float* d_target, float lr,
                            float* d_grad_out, float* h_loss, void* stream);
/* No counterpart in the reference.  Training state -- master parameters, both Adam
 * moments and the step count -- copied into snapshot slot 0 or 1 on `stream` (device
 * memory allocated on first use: BM_ERR_NOMEM if that fails), and copied back by
 * bm_net_restore (BM_ERR_STATE for a slot never written).  A training loop rolls back
 * to a snapshot that later steps validated when the loss spikes.  Synchronise
 * `stream` before reading the parameters with bm_net_get_params. */
bm_status bm_net_snapshot(bm_net* n, uint32_t slot, void* stream);
bm_status bm_net_restore(bm_net* n, uint32_t slot, void* stream);
/* Which tensor-core path the convolutions take.  mode 1 (the default where the driver
 * encodes tensor maps): every layer of the forward pass, and the backward-data pass of
 * the 32-channel layers, is a launch of tcgen05 MMAs into tensor memory fed by TMA;
 * mode 2: the six forward layers in one cooperative launch of the same MMAs with a
 * grid barrier between layers (measured slower than mode 1 at 1024x436: the barrier
 * costs more than the launches it saves); mode 0: mma.sync m16n8k16 kernels.  All
 * modes give the same network up to FP32 summation order.  bm_net_umma returns the
 * mode in use. */
bm_status bm_net_set_umma(bm_net* n, int mode);
int bm_net_umma(const bm_net* n);
/* CTAs the mode-2 launch keeps co-resident on this device (it walks each layer's
 * 128-cell tiles with that grid); 0 where cooperative launches are unavailable. */
int bm_net_fused_ctas(const bm_net* n);
/* Synchronises `stream` and reports BM_ERR_TIMEOUT if a tensor-core layer's bounded
 * wait for its copies, its MMAs or (mode 2) the grid barrier gave up since the last
 * check (its outputs are then undefined); clears the record. */
bm_status bm_net_check(bm_net* n, void* stream);

/* Attach a proposal network to a context (NULL detaches).  Every later bm_frame that
 * matches a pair runs the network on the previous and current frames and initialises
 * matching by bm_seed's rule, then runs `iterations` rounds with jump-flood maximum
 * jfMax (0 keeps the context's).  The network must have been created for at least
 * one image of (sx_in/4) x (sy_in/4).  The network's buffers are used on the
 * context's stream: one network may serve several contexts only if their work is
 * serialised (same stream, or the caller orders the streams). */
bm_status bm_set_proposal(bm_ctx* ctx, bm_net* net, float conf_threshold, uint32_t iterations, uint32_t jfMax);
/* No counterpart in the reference.  With side != 0 bm_frame runs the network on a
 * second stream of the context, from the moment the frame is on the device,
 * concurrently with its up-sampling and descriptors; the seed waits for it.  With
 * side == 0 (the default) it runs on the context stream between up-sampling and
 * descriptors.  Results are identical; at 1024x436 the side stream measured about
 * 1.5 % slower per step (its kernels take shared memory from the L1-bound descriptor
 * kernel running beside them). */
bm_status bm_set_proposal_stream(bm_ctx* ctx, int side);
/* No counterpart in the reference.  The network of bm_set_proposal sees the frames
 * reduced by `reduce` (1, the default, 2 or 4; bm_net_prepare_reduced): a cell covers
 * 4 * reduce input pixels and its predicted vector is in those units, which the seed
 * scales accordingly.  The network was trained on 512x384 frames; on larger frames,
 * whose motions exceed what it saw, a reduced input brings them back into its range
 * (on uneven 512-1920 px pairs: proposal 2.0 -> 1.0 px from the truth with reduce 2).
 * BM_ERR_LIMIT if a frame side is below 4 * reduce. */
bm_status bm_set_proposal_reduce(bm_ctx* ctx, uint32_t reduce);

/* Seeded initialisation (the stage entry point): each up-sampled pixel first takes
 * the plain initialisation (CUDA_initialize semantics: zero vector, or the temporal
 * candidate when first == 0), then the prediction's vector of its w4 x h4 cell
 * (d_pred [h4][w4][3]: u, v in cell units, confidence logit) where the confidence
 * reaches conf_threshold -- kept only if its Hamming cost is strictly lower. */
bm_status bm_seed(bm_ctx* ctx, int first, const float* d_pred, uint32_t w4, uint32_t h4, float conf_threshold);

/* Local refinement steps of the seeded schedule (no counterpart in the reference):
 * after the seeded initialisation, `count` steps each try the pixel's own vector moved
 * by r up-sampled pixels left, right, up and down (clamped into the image), keeping a
 * candidate only if its Hamming cost is strictly lower than the best so far; r starts
 * at first_radius and halves down to 1.  Applies to matching seeded by the proposal
 * (bm_set_proposal); 0 steps (the default) leaves the seeded schedule as it was. */
bm_status bm_set_local_steps(bm_ctx* ctx, uint32_t count, uint32_t first_radius);
/* One local refinement step of radius r on the current field (the stage entry point). */
bm_status bm_local_step(bm_ctx* ctx, uint32_t radius);

/* ---- refinement without allocation ------------------------------------------------ */

/* No counterpart in the reference.  The refinement of bm_process (median filter
 * then cross-trilateral filter) on caller-owned device buffers, for callers that
 * cannot allocate device memory while running (pipelines that allocate only at
 * start-up, plugin hosts that own the memory budget, threads that must not take
 * the device synchronisation of cudaMalloc/cudaFree).  It calls no allocator:
 * its intermediate planes live in a fixed 32 MiB array compiled into the library,
 * which every GPU that loads the library holds until the process exits, so it
 * accepts at most bm_refine_noalloc_max_pixels() (2,097,152) input pixels and
 * returns BM_ERR_LIMIT above that.  d_u, d_v: input field, d_guide: previous
 * input frame (0..255), d_uo, d_vo: output field; all width*height floats.  The
 * output planes must not overlap the input planes or each other (BM_ERR_INVALID):
 * the filter reads neighbouring inputs while other threads write outputs.  Sigmas
 * must be finite and positive (BM_ERR_INVALID), and the trilateral half window
 * ceil(2.5*sS) at most the frame's larger side (BM_ERR_LIMIT).
 * stream is a cudaStream_t (NULL = legacy default stream).  The first call on a
 * device looks up the array's device address with that device current; make that
 * first call before any stream capture.  The address belongs to the device's
 * context: after cudaDeviceReset the next call looks it up again in the new
 * context (again before any capture).  All calls share the one array: calls whose
 * work overlaps on the GPU (different streams, or host threads without ordering)
 * race on it; the array needs no clearing between calls, since every element is
 * written before it is read. */
bm_status bm_refine_noalloc(const float* d_u, const float* d_v, const float* d_guide, float* d_uo, float* d_vo,
                            uint32_t width, uint32_t height, uint32_t fsize, float sEPE, float sI, float sS,
                            void* stream);
uint64_t bm_refine_noalloc_max_pixels(void);

/* ---- one frame (OFPipeline::processFrame, of_pipeline.cpp:241-333) --------------- */

/* Feed the next 8-bit frame (sx_in*sy_in bytes, row-major).  frame_on_device says
 * whether `frame` is a device pointer.  The first frame only primes the context
 * (descriptors of that frame) and yields a zero field; every later frame runs
 * up-sampling, matching against the previous frame, down-sampling and refinement
 * and yields the flow from the previous frame to this one on the previous frame's
 * grid.  u and v (sx_in*sy_in floats each, device or host per out_on_device) may be
 * NULL to leave the result in BM_BUF_FLOW_OUT. */
bm_status bm_frame(bm_ctx* ctx, const uint8_t* frame, int frame_on_device,
                   float* u, float* v, int out_on_device);

/* Forget the previous frame: the next bm_frame primes again. */
bm_status bm_reset_sequence(bm_ctx* ctx);

/* Pipelined frames (no counterpart in the reference, which finishes each frame before
 * the next): with on != 0, bm_frame queues a pair's refinement (median and
 * cross-trilateral filter) and its output copies on a second stream of the context,
 * so that they overlap the next frame's up-sampling and matching; results are
 * identical.  bm_frame then returns without waiting even for host outputs (use
 * page-locked host memory for them); the outputs of every frame fed so far are
 * complete after bm_synchronize, or, for work queued behind them on the context
 * stream, after bm_join.  Other calls that read or write the refinement's buffers
 * wait for it themselves. */
bm_status bm_set_pipelined(bm_ctx* ctx, int on);
/* Make the context stream wait (on the device, without blocking the host) for the
 * pipelined refinement queued so far; a no-op for a context that never pipelined. */
bm_status bm_join(bm_ctx* ctx);

/* Count of kernels this context has launched (for launch accounting). */
uint64_t bm_launch_count(const bm_ctx* ctx);

/* Per-kernel device time (the reference's CudaTimer, util_cuda.cu:287-313, per
 * launch instead of per stage).  While enabled, every launch is bracketed by CUDA
 * events on the context's stream; bm_profile_read synchronises the stream and
 * returns one entry per kernel name (name, launches, total milliseconds). */
typedef struct bm_kernel_stat {
    const char* name;
    uint64_t launches;
    double ms;
} bm_kernel_stat;
bm_status bm_profile_enable(bm_ctx* ctx, int on);
bm_status bm_profile_reset(bm_ctx* ctx);
bm_status bm_profile_read(bm_ctx* ctx, bm_kernel_stat* out, uint32_t cap, uint32_t* count);

const char* bm_last_error(void);
const char* bm_version(void);

#ifdef __cplusplus
}
#endif
#endif

/*
 * bm_oracle.h -- CPU restatement of the BriefMatch flow path (TEST INFRASTRUCTURE).
 *
 * The tests compare the GB300 engine with this library; it is never part of the
 * engine: only the tests, the smoke check and bench.py's CPU-baseline leg may
 * load it.  Every
 * function restates one piece of the reference algorithm in plain C (scalar,
 * with OpenMP over rows) and cites the reference file:line it follows.
 *
 * Data layouts follow the reference:
 *   images      float, row-major, width sx (x fastest)
 *   descriptors uint32 [sx*sy][Ns], Ns = ceil(N/32), bit s%32 of word s/32
 *   flow        int16 NX[sx*sy], NY[sx*sy]
 *   cost        uint16 H[sx*sy] = Hamming distance; the reference stores D = H/N
 *
 * Two places where the reference is not deterministic get one fixed meaning here,
 * shared with the engine:
 *   - propagation and temporal init read neighbours from a per-jump-level snapshot
 *     (the reference reads them while other threads write them),
 *   - reads the reference makes outside its buffers (linear neighbour index in
 *     propagation, the unclamped median window) see the guard value 0.
 */
#ifndef BM_ORACLE_H
#define BM_ORACLE_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

int bmo_num_threads(void);
void bmo_set_threads(int n);

/* Lanczos-3 resampling, util_cuda.cu:126-158 (libm sinf, IEEE division). */
void bmo_upsample(const float* in, int sxi, int syi, float* out, int sxo, int syo);
void bmo_u8_to_float(const uint8_t* in, size_t n, float* out);

/* BRIEF descriptors, briefmatch_cuda.cu:82-124. */
void bmo_features(const float* I, int sx, int sy, const float* pattern, int N, uint32_t* F);

/* Zero-flow or temporal initialisation, briefmatch_cuda.cu:149-184. */
void bmo_initialize(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N, int first,
                    int16_t* NX, int16_t* NY, uint16_t* H);

/* One jump-flood level at step p, briefmatch_cuda.cu:206-219 (snapshot semantics). */
void bmo_jump_level(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N,
                    int p, int pd, int doubleProp,
                    const int16_t* NXs, const int16_t* NYs,
                    int16_t* NX, int16_t* NY, uint16_t* H);

/* Full jump-flood pass p = jfMax, jfMax/2, ..., 1, briefmatch_cuda.cu:186-220. */
void bmo_propagate(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N,
                   int pd, int jfMax, int doubleProp,
                   int16_t* NX, int16_t* NY, uint16_t* H);

/* Random search with given N(0,1) pairs normals[p*2+{0,1}], briefmatch_cuda.cu:222-246. */
void bmo_random_search(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N,
                       float dist, const float* normals,
                       int16_t* NX, int16_t* NY, uint16_t* H);

/* BriefMatch::match after the descriptors, briefmatch.cpp:264-290.
 * normals holds iterations blocks of sx*sy*2 values. */
void bmo_match(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N,
               int iterations, int jfMax, int doubleProp, int first, float dist,
               const float* normals, int16_t* NX, int16_t* NY, uint16_t* H);

/* Search radius of the random search, briefmatch.cpp:271. */
float bmo_search_dist(int sx);

/* Gaussian down-sampling taps, briefmatch.cpp:153-172; returns P (<= maxP) or -1. */
int bmo_gauss_taps(float sigma, float* taps, int maxP);

/* BriefMatch::downsample, briefmatch.cpp:296-324 with util_cuda.cu:48-73,113-124,160-183. */
void bmo_downsample(const int16_t* NX, const int16_t* NY, int sx, int sy,
                    int sx_in, int sy_in, const float* taps, int P,
                    const uint32_t* nnx, const uint32_t* nny, float* U, float* V);

/* One pass of the 1-D median, util_cuda.cu:75-111 (linear index, guard 0). */
void bmo_median1d(const float* in, float* out, int dir, int fsize, int sx, int sy);

/* Cross-trilateral filter, briefmatch_cuda.cu:248-297; sigmas are squared. */
void bmo_trilateral(const float* Ui, const float* Vi, const float* Uim, const float* Vim,
                    const float* I, float sigmaEPE2, float sigmaI2, float sigmaS2,
                    int sx, int sy, float* Uo, float* Vo);

/* BriefMatch::process, briefmatch.cpp:327-352: median H,V per component, then trilateral.
 * Umed/Vmed receive the median-filtered flow, Uo/Vo the refined flow. */
void bmo_refine(const float* U, const float* V, const float* Iprev, int sx, int sy,
                int fsize, float sEPE, float sI, float sS,
                float* Umed, float* Vmed, float* Uo, float* Vo);

/* Mean end-point error over known ground truth, briefmatch.cpp:468-514. */
double bmo_epe(const float* U, const float* V, const float* Ugt, const float* Vgt, size_t n);

/* Deterministic N(0,1) pairs for CPU-only runs (splitmix64 + Box-Muller). */
void bmo_normals(uint64_t seed, size_t count, float* out);

/* Colour coding, briefmatch.cpp:373-421 + colorcode.cpp:27-74 (R G B bytes); the float
 * atan2 correctly rounded, or libm's atan2f when libm_atan2f is set. */
void bmo_flow_colors(const float* u, const float* v, size_t n, float maxmot, int libm_atan2f, unsigned char* rgb);

#ifdef __cplusplus
}
#endif
#endif

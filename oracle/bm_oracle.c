/*
 * bm_oracle.c -- CPU restatement of the BriefMatch flow path (TEST INFRASTRUCTURE).
 *
 * The tests compare the GB300 engine with it, and bench.py times it as the CPU
 * baseline; it is never linked into the engine.  Each function cites the reference
 * file:line it restates.  Arithmetic mirrors the reference's types (float with
 * fused multiply-add where the CUDA build contracts a*b+c, int16 flow, integer
 * Hamming distance); transcendental functions come from libm, so results that
 * depend on sin/exp match the GPU within a tolerance, everything else bit-exactly.
 */
#include "bm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* util_cuda.h:61 */
static const double BMO_PI = 3.141592653589793115997963468544;

static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* The reference kernels are built with -use_fast_math, which implies flush-to-zero:
 * single-precision operands and results below the smallest normal float are read
 * and written as (sign-preserving) zero.  The bit-exact pieces apply the same rule. */
static inline float ftzf(float v) { return fabsf(v) < FLT_MIN ? copysignf(0.0f, v) : v; }
static inline float fma_ftz(float a, float b, float c) { return ftzf(fmaf(ftzf(a), ftzf(b), ftzf(c))); }
static inline float mul_ftz(float a, float b) { return ftzf(ftzf(a) * ftzf(b)); }

int bmo_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void bmo_set_threads(int n)
{
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void bmo_u8_to_float(const uint8_t* in, size_t n, float* out)
{
    for (size_t i = 0; i < n; i++) out[i] = (float)in[i];
}

/* Lanczos kernel L(t) for a = 3 as written in util_cuda.cu:144-146 and :149-151. */
static inline float lanczos3(float p, int i)
{
    float xx = (float)(BMO_PI * (double)(p - (float)i));
    float L = 3.0f * sinf(xx) * sinf(xx / 3.0f) / (xx * xx);
    if (L != L) L = 1.0f;
    return L;
}

/* util_cuda.cu:126-158: output (x,y) samples the input at (x*sxi/sxo, y*syi/syo)
 * with taps i = floor(xp)-2 .. floor(xp)+3 (and the same for y), clamp-to-edge,
 * normalised by the sum of the weights. */
void bmo_upsample(const float* in, int sxi, int syi, float* out, int sxo, int syo)
{
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < syo; y++) {
        float yp = (float)y * (float)syi / (float)syo;
        int y1 = (int)floorf(yp);
        float Ly[6];
        int jy[6];
        for (int b = 0; b < 6; b++) {
            Ly[b] = lanczos3(yp, y1 - 2 + b);
            jy[b] = clampi(y1 - 2 + b, 0, syi - 1);
        }
        for (int x = 0; x < sxo; x++) {
            float xp = (float)x * (float)sxi / (float)sxo;
            int x1 = (int)floorf(xp);
            float v = 0.0f, w = 0.0f;
            for (int a = 0; a < 6; a++) {
                int i = x1 - 2 + a;
                float Lx = lanczos3(xp, i);
                int ci = clampi(i, 0, sxi - 1);
                for (int b = 0; b < 6; b++) {
                    w = fmaf(Lx, Ly[b], w);
                    v = fmaf(in[ci + (size_t)jy[b] * sxi] * Lx, Ly[b], v);
                }
            }
            out[x + (size_t)y * sxo] = v / w;
        }
    }
}

/* briefmatch_cuda.cu:82-124: bit s of the descriptor is I[p+o1] > I[p+o2] with
 * o = int(pattern) truncated toward zero and clamped so p+o stays in the image. */
void bmo_features(const float* I, int sx, int sy, const float* pattern, int N, uint32_t* F)
{
    int Ns = (N + 31) / 32;
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < sy; y++) {
        for (int x = 0; x < sx; x++) {
            size_t off = (size_t)x + (size_t)y * sx;
            uint32_t* f = F + off * Ns;
            for (int w = 0; w < Ns; w++) f[w] = 0;
            for (int s = 0; s < N; s++) {
                int ox1 = clampi((int)pattern[4 * s + 0], -x, sx - x - 1);
                int oy1 = clampi((int)pattern[4 * s + 1], -y, sy - y - 1);
                int ox2 = clampi((int)pattern[4 * s + 2], -x, sx - x - 1);
                int oy2 = clampi((int)pattern[4 * s + 3], -y, sy - y - 1);
                float i1 = I[(long)off + ox1 + (long)oy1 * sx];
                float i2 = I[(long)off + ox2 + (long)oy2 * sx];
                if (i1 > i2) f[s >> 5] |= 1u << (s & 31);
            }
        }
    }
}

/* featDist, briefmatch_cuda.cu:60-80, as an integer distance.  The reference
 * stops early once the partial sum exceeds N*D; a candidate stopped that way is
 * never accepted, so the full count gives the same decisions. */
static inline int hamming(const uint32_t* F1, const uint32_t* F2, size_t p, size_t q, int Ns)
{
    const uint32_t* a = F1 + p * Ns;
    const uint32_t* b = F2 + q * Ns;
    int d = 0;
    for (int s = 0; s < Ns; s++) d += __builtin_popcount(a[s] ^ b[s]);
    return d;
}

/* briefmatch_cuda.cu:149-184.  Temporal init reads the previous field from a
 * snapshot taken before any pixel is updated. */
void bmo_initialize(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N, int first,
                    int16_t* NX, int16_t* NY, uint16_t* H)
{
    int Ns = (N + 31) / 32;
    size_t n = (size_t)sx * sy;
    int16_t* SX = NULL;
    int16_t* SY = NULL;
    if (!first) {
        SX = (int16_t*)malloc(n * sizeof(int16_t));
        SY = (int16_t*)malloc(n * sizeof(int16_t));
        memcpy(SX, NX, n * sizeof(int16_t));
        memcpy(SY, NY, n * sizeof(int16_t));
    }
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < sy; y++) {
        for (int x = 0; x < sx; x++) {
            size_t p = (size_t)x + (size_t)y * sx;
            if (first) {
                NX[p] = 0;
                NY[p] = 0;
                H[p] = (uint16_t)hamming(F1, F2, p, p, Ns);
            } else {
                long q = (long)p + SX[p] + (long)SY[p] * sx;
                int vx = (q >= 0 && q < (long)n) ? SX[q] : 0;
                int vy = (q >= 0 && q < (long)n) ? SY[q] : 0;
                int nx = clampi(vx, -x, sx - x - 1);
                int ny = clampi(vy, -y, sy - y - 1);
                NX[p] = (int16_t)nx;
                NY[p] = (int16_t)ny;
                H[p] = (uint16_t)hamming(F1, F2, p, (size_t)((long)p + nx + (long)ny * sx), Ns);
            }
        }
    }
    free(SX);
    free(SY);
}

/* One level of briefmatch_cuda.cu:206-219.  Candidates in reference order
 * d = -1, +1 (only +1 without doubleProp), xy = 0 (vertical) then 1 (horizontal);
 * the neighbour is read at linear index p + doff (rows wrap horizontally), and
 * the guard value 0 is read outside the field.  insert() (:126-147) accepts a
 * candidate iff its cost is strictly lower. */
void bmo_jump_level(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N,
                    int p, int pd, int doubleProp,
                    const int16_t* NXs, const int16_t* NYs,
                    int16_t* NX, int16_t* NY, uint16_t* H)
{
    int Ns = (N + 31) / 32;
    long n = (long)sx * sy;
    int dstart = doubleProp ? -1 : 1;
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < sy; y++) {
        for (int x = 0; x < sx; x++) {
            long pix = (long)x + (long)y * sx;
            int cx = NXs[pix], cy = NYs[pix];
            int h = H[pix];
            for (int d = dstart; d <= 1; d += 2) {
                for (int xy = 0; xy <= 1; xy++) {
                    long doff = (long)pd * p * d * xy + (long)sx * pd * p * d * (1 - xy);
                    long q = pix + doff;
                    int vx = (q >= 0 && q < n) ? NXs[q] : 0;
                    int vy = (q >= 0 && q < n) ? NYs[q] : 0;
                    int nx = clampi(vx, -x, sx - x - 1);
                    int ny = clampi(vy, -y, sy - y - 1);
                    if (nx == cx && ny == cy) continue;
                    int hc = hamming(F1, F2, (size_t)pix, (size_t)(pix + nx + (long)ny * sx), Ns);
                    if (hc < h) {
                        h = hc;
                        cx = nx;
                        cy = ny;
                    }
                }
            }
            NX[pix] = (int16_t)cx;
            NY[pix] = (int16_t)cy;
            H[pix] = (uint16_t)h;
        }
    }
}

void bmo_propagate(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N,
                   int pd, int jfMax, int doubleProp,
                   int16_t* NX, int16_t* NY, uint16_t* H)
{
    size_t n = (size_t)sx * sy;
    int16_t* SX = (int16_t*)malloc(n * sizeof(int16_t));
    int16_t* SY = (int16_t*)malloc(n * sizeof(int16_t));
    for (int p = jfMax; p > 0; p /= 2) {
        memcpy(SX, NX, n * sizeof(int16_t));
        memcpy(SY, NY, n * sizeof(int16_t));
        bmo_jump_level(F1, F2, sx, sy, N, p, pd, doubleProp, SX, SY, NX, NY, H);
    }
    free(SX);
    free(SY);
}

/* briefmatch_cuda.cu:222-246: candidate (round(dist*n1), round(dist*n2)), clamped. */
void bmo_random_search(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N,
                       float dist, const float* normals,
                       int16_t* NX, int16_t* NY, uint16_t* H)
{
    int Ns = (N + 31) / 32;
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < sy; y++) {
        for (int x = 0; x < sx; x++) {
            size_t pix = (size_t)x + (size_t)y * sx;
            int rx = (int)roundf(dist * normals[2 * pix + 0]);
            int ry = (int)roundf(dist * normals[2 * pix + 1]);
            int nx = clampi(rx, -x, sx - x - 1);
            int ny = clampi(ry, -y, sy - y - 1);
            if (nx == NX[pix] && ny == NY[pix]) continue;
            int hc = hamming(F1, F2, pix, (size_t)((long)pix + nx + (long)ny * sx), Ns);
            if (hc < H[pix]) {
                H[pix] = (uint16_t)hc;
                NX[pix] = (int16_t)nx;
                NY[pix] = (int16_t)ny;
            }
        }
    }
}

/* briefmatch.cpp:264-290 */
void bmo_match(const uint32_t* F1, const uint32_t* F2, int sx, int sy, int N,
               int iterations, int jfMax, int doubleProp, int first, float dist,
               const float* normals, int16_t* NX, int16_t* NY, uint16_t* H)
{
    size_t n = (size_t)sx * sy;
    bmo_initialize(F1, F2, sx, sy, N, first, NX, NY, H);
    int pd = -1;
    for (int it = 0; it < iterations; it++) {
        bmo_propagate(F1, F2, sx, sy, N, pd, jfMax, doubleProp, NX, NY, H);
        bmo_random_search(F1, F2, sx, sy, N, dist, normals + (size_t)it * n * 2, NX, NY, H);
        pd = -pd;
    }
}

/* briefmatch.cpp:271 */
float bmo_search_dist(int sx)
{
    return sqrtf(ceilf((float)(unsigned)sx * 0.5f / 3.0f));
}

/* briefmatch.cpp:153-172 */
int bmo_gauss_taps(float sigma, float* taps, int maxP)
{
    float sig = sigma;
    int P = (int)(unsigned)(ceilf(sig * 3) * 2 + 1);
    if (P > maxP) return -1;
    int P2 = P / 2;
    float w = 0;
    for (int i = -P2; i <= P2; i++) {
        taps[i + P2] = expf((float)(-i * i) / (2 * sig * sig));
        w += taps[i + P2];
    }
    for (int i = 0; i < P; i++) taps[i] /= w;
    return P;
}

/* filterConst dir=1 (util_cuda.cu:61-65) evaluated at one up-sampled pixel. */
static inline float gauss_h(const int16_t* L, int sx, int x, int y, const float* taps, int P)
{
    int ks2 = P / 2;
    float s = 0;
    for (int i = 0; i < P; i++) s = fma_ftz(taps[i], (float)L[clampi(x + i - ks2, 0, sx - 1) + (size_t)y * sx], s);
    return s;
}

/* briefmatch.cpp:296-324: int16 -> float (util_cuda.cu:174-183), Gaussian H then V
 * (util_cuda.cu:48-73), nearest-neighbour decimation (util_cuda.cu:160-172) and
 * scaling by sx_in/sx (util_cuda.cu:113-124), with flush-to-zero arithmetic.  Only
 * the decimated pixels are
 * evaluated; each one repeats the reference's per-pass rounding.  The source index
 * round(x*sx/sx_in) is computed on the device with the fast-math division; where
 * that quotient lands exactly on .5 the IEEE quotient used here can round the other
 * way, so callers comparing with a device run pass the device's index tables. */
void bmo_downsample(const int16_t* NX, const int16_t* NY, int sx, int sy,
                    int sx_in, int sy_in, const float* taps, int P,
                    const uint32_t* nnx, const uint32_t* nny, float* U, float* V)
{
    size_t n_in = (size_t)sx_in * sy_in;
    if (sx_in == sx && sy_in == sy) {
        for (size_t i = 0; i < n_in; i++) {
            U[i] = (float)NX[i];
            V[i] = (float)NY[i];
        }
        return;
    }
    float mx = (float)sx_in / (float)(unsigned)sx;
    float my = (float)sy_in / (float)(unsigned)sy;
    int ks2 = P / 2;
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < sy_in; y++) {
        for (int x = 0; x < sx_in; x++) {
            unsigned x1 = nnx ? nnx[x] : (unsigned)roundf((float)x * (float)sx / (float)sx_in);
            unsigned y1 = nny ? nny[y] : (unsigned)roundf((float)y * (float)sy / (float)sy_in);
            size_t o = (size_t)x + (size_t)y * sx_in;
            if (x1 >= (unsigned)sx || y1 >= (unsigned)sy) {
                U[o] = 0;
                V[o] = 0;
                continue;
            }
            float su = 0, sv = 0;
            for (int i = 0; i < P; i++) {
                int yy = clampi((int)y1 + i - ks2, 0, sy - 1);
                su = fma_ftz(taps[i], gauss_h(NX, sx, (int)x1, yy, taps, P), su);
                sv = fma_ftz(taps[i], gauss_h(NY, sx, (int)x1, yy, taps, P), sv);
            }
            U[o] = mul_ftz(su, mx);
            V[o] = mul_ftz(sv, my);
        }
    }
}

/* util_cuda.cu:75-111: fsize samples along x (dir=1) or y (dir=0) around the pixel,
 * read at linear index with no clamp (guard value 0 outside the buffer), partial
 * bubble sort of the first ks+1 positions, result v[ks]. */
void bmo_median1d(const float* in, float* out, int dir, int fsize, int sx, int sy)
{
    long n = (long)sx * sy;
    int ks = fsize / 2;
    #pragma omp parallel for schedule(static)
    for (int y = 0; y < sy; y++) {
        float v[64];
        for (int x = 0; x < sx; x++) {
            int i = 0;
            if (dir) {
                for (int xx = x - ks; xx <= x + ks; xx++) {
                    long idx = (long)xx + (long)y * sx;
                    v[i++] = (idx >= 0 && idx < n) ? in[idx] : 0.0f;
                }
            } else {
                for (int yy = y - ks; yy <= y + ks; yy++) {
                    long idx = (long)x + (long)yy * sx;
                    v[i++] = (idx >= 0 && idx < n) ? in[idx] : 0.0f;
                }
            }
            for (int a = 0; a <= ks; a++)
                for (int b = a + 1; b < fsize; b++)
                    if (v[a] > v[b]) {
                        float t = v[a];
                        v[a] = v[b];
                        v[b] = t;
                    }
            out[(size_t)x + (size_t)y * sx] = v[ks];
        }
    }
}

/* briefmatch_cuda.cu:248-297: window i,j in [-s, s) with s = ceil(2.5*sqrt(sigmaS)),
 * clamp-to-edge, weight exp(-|u-u_med|^2/2sE) exp(-dI^2/2sI) exp(-(i^2+j^2)/2sS)
 * with intensities divided by 255, result uf/max(1e-5, W). */
void bmo_trilateral(const float* Ui, const float* Vi, const float* Uim, const float* Vim,
                    const float* I, float sigmaEPE2, float sigmaI2, float sigmaS2,
                    int sx, int sy, float* Uo, float* Vo)
{
    int s = (int)ceil(2.5 * (double)sqrtf(sigmaS2));
    #pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < sy; y++) {
        for (int x = 0; x < sx; x++) {
            size_t off = (size_t)x + (size_t)y * sx;
            float um0 = Uim[off], vm0 = Vim[off], I0 = I[off] / 255;
            float uf = 0, vf = 0, W = 0;
            for (int i = -s; i < s; i++) {
                for (int j = -s; j < s; j++) {
                    size_t o1 = (size_t)clampi(x + i, 0, sx - 1) + (size_t)clampi(y + j, 0, sy - 1) * sx;
                    float u1 = Ui[o1], v1 = Vi[o1], I1 = I[o1] / 255;
                    float du = u1 - um0, dv = v1 - vm0;
                    float dEPE = du * du + dv * dv;
                    float dI = I1 - I0;
                    float w = expf(-dEPE / (2 * sigmaEPE2)) * expf(-(dI * dI) / (2 * sigmaI2)) *
                              expf(-(float)(i * i + j * j) / (2 * sigmaS2));
                    uf += w * u1;
                    vf += w * v1;
                    W += w;
                }
            }
            double Wd = W > 1e-5 ? (double)W : 1e-5;
            Uo[off] = (float)((double)uf / Wd);
            Vo[off] = (float)((double)vf / Wd);
        }
    }
}

/* briefmatch.cpp:327-352 */
void bmo_refine(const float* U, const float* V, const float* Iprev, int sx, int sy,
                int fsize, float sEPE, float sI, float sS,
                float* Umed, float* Vmed, float* Uo, float* Vo)
{
    size_t n = (size_t)sx * sy;
    float* tmp = (float*)malloc(n * sizeof(float));
    bmo_median1d(U, tmp, 1, fsize, sx, sy);
    bmo_median1d(tmp, Umed, 0, fsize, sx, sy);
    bmo_median1d(V, tmp, 1, fsize, sx, sy);
    bmo_median1d(tmp, Vmed, 0, fsize, sx, sy);
    free(tmp);
    bmo_trilateral(U, V, Umed, Vmed, Iprev, sEPE * sEPE, sI * sI, sS * sS, sx, sy, Uo, Vo);
}

/* briefmatch.cpp:468-514; unknown flow as flowIO.cpp:35-39 (|u| or |v| > 1e9, or NaN). */
double bmo_epe(const float* U, const float* V, const float* Ugt, const float* Vgt, size_t n)
{
    double err = 0;
    size_t cnt = 0;
    for (size_t i = 0; i < n; i++) {
        float fx = Ugt[i], fy = Vgt[i];
        if (fabsf(fx) > 1e9f || fabsf(fy) > 1e9f || fx != fx || fy != fy) continue;
        double dx = (double)fx - U[i], dy = (double)fy - V[i];
        err += sqrt(dx * dx + dy * dy);
        cnt++;
    }
    return cnt ? err / (double)cnt : 0.0;
}

static inline uint64_t splitmix64(uint64_t* s)
{
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

void bmo_normals(uint64_t seed, size_t count, float* out)
{
    uint64_t st = seed;
    for (size_t i = 0; i < count; i += 2) {
        uint64_t r = splitmix64(&st);
        double u1 = ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        r = splitmix64(&st);
        double u2 = ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
        double rad = sqrt(-2.0 * log(u1));
        out[i] = (float)(rad * cos(2.0 * BMO_PI * u2));
        if (i + 1 < count) out[i + 1] = (float)(rad * sin(2.0 * BMO_PI * u2));
    }
}

/* Colour wheel, colorcode.cpp:27-50: integer channel values from integer divisions. */
static int colorwheel[55][3];
static void make_colorwheel(void)
{
    const int RY = 15, YG = 6, GC = 4, CB = 11, BM = 13, MR = 6;
    int k = 0, i;
#define SETCOL(r, g, b) (colorwheel[k][0] = (r), colorwheel[k][1] = (g), colorwheel[k][2] = (b), k++)
    for (i = 0; i < RY; i++) SETCOL(255, 255 * i / RY, 0);
    for (i = 0; i < YG; i++) SETCOL(255 - 255 * i / YG, 255, 0);
    for (i = 0; i < GC; i++) SETCOL(0, 255, 255 * i / GC);
    for (i = 0; i < CB; i++) SETCOL(0, 255 - 255 * i / CB, 255);
    for (i = 0; i < BM; i++) SETCOL(255 * i / BM, 0, 255);
    for (i = 0; i < MR; i++) SETCOL(255, 0, 255 - 255 * i / MR);
#undef SETCOL
}

static int unknown_flow(float u, float v)
{
    return fabsf(u) > 1e9f || fabsf(v) > 1e9f || u != u || v != v; /* flowIO.cpp:35-39 */
}

/* computeColor, colorcode.cpp:52-74, with its declared types (float rad, a, fk, f,
 * col0, col1, col; the double constants 1.0, 2.0, M_PI (BMO_PI), .75, 255.0), writing R G B
 * (the reference writes BGR at pix[2 - b]; its PNG writer swaps to RGB).  The float
 * atan2 is the correctly rounded one (a double atan2 rounded once), or libm's atan2f
 * when libm_atan2f is set (the reference's literal call). */
static void compute_color(float fx, float fy, int libm_atan2f, unsigned char* pix)
{
    const int ncols = 55;
    float rad = sqrtf(fx * fx + fy * fy);
    float at = libm_atan2f ? atan2f(-fy, -fx) : (float)atan2(-(double)fy, -(double)fx);
    float a = (float)((double)at / BMO_PI);
    float fk = (float)(((double)a + 1.0) / 2.0 * (ncols - 1));
    int k0 = (int)fk;
    int k1 = (k0 + 1) % ncols;
    float f = fk - (float)k0;
    for (int b = 0; b < 3; b++) {
        float col0 = (float)(colorwheel[k0][b] / 255.0);
        float col1 = (float)(colorwheel[k1][b] / 255.0);
        float col = (1 - f) * col0 + f * col1;
        if (rad <= 1)
            col = 1 - rad * (1 - col);
        else
            col = (float)((double)col * .75);
        pix[b] = (unsigned char)(int)(255.0 * (double)col);
    }
}

/* BriefMatch::computeColors, briefmatch.cpp:373-421: normalise by maxmot when it is
 * > 0, else by the largest known vector length (0 -> 1); unknown vectors are black. */
void bmo_flow_colors(const float* u, const float* v, size_t n, float maxmot, int libm_atan2f, unsigned char* rgb)
{
    static int built = 0;
    if (!built) {
        make_colorwheel();
        built = 1;
    }
    float maxrad = -1;
    for (size_t i = 0; i < n; i++) {
        if (unknown_flow(u[i], v[i])) continue;
        float rad = sqrtf(u[i] * u[i] + v[i] * v[i]);
        if (rad > maxrad) maxrad = rad;
    }
    if (maxmot > 0) maxrad = maxmot;
    if (maxrad == 0) maxrad = 1;
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; i++) {
        unsigned char* pix = rgb + 3 * i;
        if (unknown_flow(u[i], v[i]))
            pix[0] = pix[1] = pix[2] = 0;
        else
            compute_color(u[i] / maxrad, v[i] / maxrad, libm_atan2f, pix);
    }
}

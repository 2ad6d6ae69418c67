// bm_params.cpp -- host-side parameter logic of the engine: BMParams defaults,
// the command-line derivation, the BRIEF sampling pattern and the Gaussian taps.
#include <algorithm>
#include <cmath>
#include <random>

#include "briefmatch_gb300.h"

extern "C" {

// BMParams::BMParams, briefmatch.h:67-84
bm_status bm_params_default(bm_params* p)
{
    if (!p) return BM_ERR_INVALID;
    *p = bm_params{};
    p->sx = p->sy = p->sx_in = p->sy_in = 64;
    p->iterations = 2;
    p->jfMax = 256;
    p->doubleProp = 1;
    p->filter = 1;
    p->tInit = 1;
    p->sigma = 0.5f;
    p->P = 11;
    p->fsize = 13;
    p->N = 128;
    p->patchArea = 75;
    p->sEPE = 0.4f;
    p->sI = 0.1f;
    p->sS = 6.0f;
    p->maxmot = 5.0f;
    p->rng = BM_RNG_XORWOW;
    p->seed = 0;
    return BM_OK;
}

// OFPipeline::setParams, of_pipeline.cpp:178-190.  The arithmetic keeps the
// reference's types: the up-sampled size is float*unsigned truncated, the
// diagonals are sqrt of unsigned sums in double.
bm_status bm_params_derive(bm_params* p, uint32_t width, uint32_t height, float ux, float uy,
                           float patchRad, float sigmaRad, float fsizeRad, float sSRad)
{
    if (!p || width == 0 || height == 0) return BM_ERR_INVALID;
    if (ux < 0.1f) ux = 2.740f;
    if (uy < 0.1f) uy = 3.052f;
    unsigned int m_sx_in = width, m_sy_in = height;
    unsigned int m_sx = (unsigned int)(ux * (float)m_sx_in);
    unsigned int m_sy = (unsigned int)(uy * (float)m_sy_in);
    p->sx = m_sx;
    p->sy = m_sy;
    p->sx_in = m_sx_in;
    p->sy_in = m_sy_in;
    const double diag_up = std::sqrt((double)(m_sx * m_sx + m_sy * m_sy));
    const double diag_in = std::sqrt((double)(m_sx_in * m_sx_in + m_sy_in * m_sy_in));
    p->patchArea = (float)((double)(0.01f * patchRad) * diag_up);
    p->sigma = (float)((double)(0.01f * sigmaRad) * diag_up);
    p->fsize = (unsigned int)(2 * std::round((double)(0.005f * fsizeRad) * diag_in) + 1);
    p->sS = (float)((double)(0.01f * sSRad) * diag_in);
    return BM_OK;
}

// briefmatch.cpp:124-148 with an explicit seed.
bm_status bm_make_pattern(const bm_params* p, uint64_t seed, float* out)
{
    if (!p || !out) return BM_ERR_INVALID;
    if (p->N < 1 || p->N > BM_PATCH_MAX / 4) return BM_ERR_LIMIT;
    std::mt19937_64 rng(seed);
    std::normal_distribution<double> nd(0.0, 0.2);
    for (uint32_t s = 0; s < 4 * p->N; s++) {
        float val = (float)nd(rng);
        val = (2 * float(val > 0) - 1) * std::pow(std::fabs(val), 2.0f);
        out[s] = p->patchArea * std::max(-1.0f, std::min(1.0f, val));
    }
    return BM_OK;
}

// briefmatch.cpp:153-172
bm_status bm_gauss_taps(float sigma, float* taps, uint32_t* P_out)
{
    if (!taps || !P_out) return BM_ERR_INVALID;
    float sig = sigma;
    unsigned int P = (unsigned int)(std::ceil(sig * 3) * 2 + 1);
    if (P > BM_CONST_KERNEL_SIZE) return BM_ERR_LIMIT;
    int P2 = (int)P / 2;
    float w = 0;
    for (int i = -P2; i <= P2; i++) {
        taps[i + P2] = std::exp((float)(-i * i) / (2 * sig * sig));
        w += taps[i + P2];
    }
    for (unsigned int i = 0; i < P; i++) taps[i] /= w;
    *P_out = P;
    return BM_OK;
}

}  // extern "C"

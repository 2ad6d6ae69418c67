// briefmatch.cpp -- BriefMatch (briefmatch.cpp of the reference) over the engine's C ABI.
#include "briefmatch.h"

#include <cmath>
#include <cstdio>

#include "flow_io.h"

void bm_throw_on_error(bm_status st)
{
    if (st == BM_OK) return;
    const char* msg = bm_last_error();
    if (st == BM_ERR_CUDA || st == BM_ERR_NOMEM || st == BM_ERR_TIMEOUT) throw CudaException(msg);
    throw BriefMatchException(msg);
}

BriefMatch::BriefMatch() : m_ctx(nullptr), m_setup(false), m_verbose(false), m_rng(BM_RNG_XORWOW), m_seed(0) {}

BriefMatch::~BriefMatch() { clean(); }

bm_params BriefMatch::engineParams() const
{
    bm_params p;
    bm_params_default(&p);
    p.sx = m_params.sx;
    p.sy = m_params.sy;
    p.sx_in = m_params.sx_in;
    p.sy_in = m_params.sy_in;
    p.N = m_params.N;
    p.iterations = m_params.iterations;
    p.jfMax = m_params.jfMax;
    p.P = m_params.P;
    p.fsize = m_params.fsize;
    p.patchArea = m_params.patchArea;
    p.sigma = m_params.sigma;
    p.sEPE = m_params.sEPE;
    p.sI = m_params.sI;
    p.sS = m_params.sS;
    p.maxmot = m_params.maxmot;
    p.doubleProp = m_params.doubleProp;
    p.filter = m_params.filter;
    p.tInit = m_params.tInit;
    p.rng = m_rng;
    p.seed = m_seed;
    return p;
}

// briefmatch.cpp:72-214
void BriefMatch::setup()
{
    if (m_setup) return;
    bm_params p = engineParams();
    bm_throw_on_error(bm_create(&p, &m_ctx));
    bm_params got;
    bm_get_params(m_ctx, &got);
    m_params.P = got.P;
    const size_t n = (size_t)m_params.sx_in * m_params.sy_in;
    m_u.assign(n, 0.0f);
    m_v.assign(n, 0.0f);
    m_vis.assign(3 * n, 0);
    if (m_verbose) {
        const float h = std::sqrt((float)(m_params.sx * m_params.sx + m_params.sy * m_params.sy));
        const float h_in = std::sqrt((float)(m_params.sx_in * m_params.sx_in + m_params.sy_in * m_params.sy_in));
        std::fprintf(stderr, "BriefMatch options:\n");
        std::fprintf(stderr, "\tFeature length:            %u\n", m_params.N);
        std::fprintf(stderr, "\tPatch radius:              %0.1f pixels (%0.4f%%)\n", m_params.patchArea,
                     100 * m_params.patchArea / h);
        std::fprintf(stderr, "\tUp-sampling resolution:    %ux%u\n", m_params.sx, m_params.sy);
        std::fprintf(stderr, "\tDown-sampling sigma:       %0.4f pixels\n", m_params.sigma);
        std::fprintf(stderr, "\tIterations / jump max:     %u / %u\n", m_params.iterations, m_params.jfMax);
        std::fprintf(stderr, "\tMedian filter size:        %u pixels (%0.4f%%)\n", m_params.fsize,
                     100 * m_params.fsize / h_in);
        std::fprintf(stderr, "\tSigma EPE / image / spatial: %0.4f / %0.4f / %0.4f\n", m_params.sEPE, m_params.sI,
                     m_params.sS);
    }
    m_setup = true;
}

// briefmatch.cpp:217-238
void BriefMatch::clean()
{
    if (m_ctx) bm_destroy(m_ctx);
    m_ctx = nullptr;
    m_setup = false;
}

void BriefMatch::setPattern(const std::vector<float>& pattern)
{
    if (!m_setup) throw BriefMatchException("BriefMatch is not initialized before use.");
    bm_throw_on_error(bm_set_pattern(m_ctx, pattern.data(), (uint32_t)pattern.size()));
}

void BriefMatch::swap()
{
    if (!m_setup) throw BriefMatchException("BriefMatch is not initialized before use.");
    bm_throw_on_error(bm_swap(m_ctx));
}

// briefmatch.cpp:248-293
void BriefMatch::match(float* im1, float* im2)
{
    if (!m_setup) throw BriefMatchException("BriefMatch is not initialized before use.");
    bm_throw_on_error(bm_match(m_ctx, im1, im2));
}

void BriefMatch::downsample()
{
    if (!m_setup) throw BriefMatchException("BriefMatch is not initialized before use.");
    bm_throw_on_error(bm_downsample(m_ctx));
}

void BriefMatch::process(float* im1)
{
    if (!m_setup) throw BriefMatchException("BriefMatch is not initialized before use.");
    bm_throw_on_error(bm_process(m_ctx, im1));
}

// briefmatch.cpp:355-370
void BriefMatch::convert()
{
    if (!m_setup) throw BriefMatchException("BriefMatch is not initialized before use.");
    bm_throw_on_error(bm_convert(m_ctx, m_u.data(), m_v.data()));
}

// briefmatch.cpp:373-421
void BriefMatch::computeColors(const float* u, const float* v, int width, int height, unsigned char* rgb)
{
    float maxrad = -1;
    const size_t n = (size_t)width * height;
    for (size_t i = 0; i < n; i++) {
        if (bmio::unknown_flow(u[i], v[i])) continue;
        maxrad = std::max(maxrad, std::sqrt(u[i] * u[i] + v[i] * v[i]));
    }
    if (m_params.maxmot > 0) maxrad = m_params.maxmot;
    if (maxrad == 0) maxrad = 1;
    for (size_t i = 0; i < n; i++) {
        if (bmio::unknown_flow(u[i], v[i]))
            rgb[3 * i] = rgb[3 * i + 1] = rgb[3 * i + 2] = 0;
        else
            bmio::flow_color(u[i] / maxrad, v[i] / maxrad, rgb + 3 * i);
    }
}

// The context's own field is coloured on the GPU (bm_colors), the same arithmetic.
void BriefMatch::computeColors()
{
    if (!m_setup) throw BriefMatchException("BriefMatch is not initialized before use.");
    bm_throw_on_error(bm_colors(m_ctx, m_vis.data(), 0));
}

void BriefMatch::printVis(std::string file)
{
    try {
        bmio::write_png_rgb(file, m_vis.data(), (int)m_params.sx_in, (int)m_params.sy_in);
    } catch (std::exception& e) {
        throw BriefMatchException(std::string("Cannot write to image file.\n\t") + e.what());
    }
}

void BriefMatch::printRaw(std::string file)
{
    try {
        bmio::write_raw(file, m_u.data(), m_v.data(), (int)m_params.sx_in, (int)m_params.sy_in);
    } catch (std::exception& e) {
        throw BriefMatchException(e.what());
    }
}

void BriefMatch::print(std::string file)
{
    try {
        bmio::write_flo(file, m_u.data(), m_v.data(), (int)m_params.sx_in, (int)m_params.sy_in);
    } catch (std::exception& e) {
        throw BriefMatchException(std::string("Cannot write .flo file.\n\t") + e.what());
    }
}

// briefmatch.cpp:468-514: mean end-point error over pixels with known ground truth
float BriefMatch::error(std::string file)
{
    std::vector<float> gu, gv;
    int w = 0, h = 0;
    try {
        bmio::read_flo(file, gu, gv, w, h);
    } catch (std::exception& e) {
        throw BriefMatchException(std::string("Failure in flow error computation:\n\t") + e.what());
    }
    if (w != (int)m_params.sx_in || h != (int)m_params.sy_in)
        throw BriefMatchException("Failure in flow error computation:\n\tground truth size differs from the frames");
    double err = 0;
    size_t cnt = 0;
    for (size_t i = 0; i < gu.size(); i++) {
        if (bmio::unknown_flow(gu[i], gv[i])) continue;
        const double dx = gu[i] - m_u[i], dy = gv[i] - m_v[i];
        err += std::sqrt(dx * dx + dy * dy);
        cnt++;
    }
    return cnt ? (float)(err / cnt) : 0.0f;
}

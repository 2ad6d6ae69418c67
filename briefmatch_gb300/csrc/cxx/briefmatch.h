// briefmatch.h -- the reference's host API (briefmatch.h:65-155) over the GB300 engine.
//
// BMParams, BriefMatch and the exception types keep the reference's names, fields,
// defaults and method signatures, so code written against the reference compiles
// against this header.  The device work goes through the engine's C ABI
// (briefmatch_gb300.h); these classes only own a context and host-side outputs.
#ifndef BRIEFMATCH_GB300_CXX_BRIEFMATCH_H
#define BRIEFMATCH_GB300_CXX_BRIEFMATCH_H

#include <cstdint>
#include <exception>
#include <string>
#include <vector>

#include "briefmatch_gb300.h"

typedef short int sint;

// briefmatch.h:65-89
struct BMParams {
    BMParams()
    {
        sx = sy = sx_in = sy_in = 64;
        iterations = 2;
        jfMax = 256;
        doubleProp = true;
        filter = true;
        tInit = true;
        sigma = 0.5f;
        P = 11;
        fsize = 13;
        N = 128;
        patchArea = 75;
        sEPE = 0.4f;
        sI = 0.1f;
        sS = 6.0f;
        maxmot = 5.0f;
    }
    unsigned int sx, sy, sx_in, sy_in, N, iterations, jfMax, P, fsize;
    float patchArea, sigma, sEPE, sI, sS, maxmot;
    bool doubleProp, filter, tInit;
};

class BriefMatchException : public std::exception {
    std::string msg;

public:
    BriefMatchException(const std::string& message) : msg(message) {}
    BriefMatchException(const char* message) : msg(message) {}
    const char* what() const noexcept override { return msg.c_str(); }
};

class CudaException : public std::exception {
    std::string msg;

public:
    CudaException(const std::string& message) : msg(message) {}
    CudaException(const char* message) : msg(message) {}
    const char* what() const noexcept override { return msg.c_str(); }
};

class ParserException : public std::exception {
    std::string msg;

public:
    ParserException(const std::string& message) : msg(message) {}
    ParserException(const char* message) : msg(message) {}
    const char* what() const noexcept override { return msg.c_str(); }
};

// Throws the reference's exception type for a failed engine call.
void bm_throw_on_error(bm_status st);

// briefmatch.h:108-155
class BriefMatch {
public:
    BriefMatch();
    ~BriefMatch();

    void setup();
    void clean();

    void setParams(BMParams params) { m_params = params; }
    BMParams* getParams() { return &m_params; }

    void swap();
    void match(float* im1, float* im2);  // device pointers to up-sampled frames
    void downsample();
    void process(float* im1 = nullptr);  // device pointer to the previous input frame

    void convert();
    void print(std::string file);
    // Middlebury colour coding of (u, v) into rgb (3 bytes per pixel); the
    // reference's overload takes imageLib images (briefmatch.cpp:373-421).
    void computeColors(const float* u, const float* v, int width, int height, unsigned char* rgb);
    void computeColors();
    void printVis(std::string file);
    void printRaw(std::string file);
    float error(std::string filename);

    bool isSetup() { return m_setup; }
    void setVerbose(bool v) { m_verbose = v; }

    // Engine extensions: pattern injection, the random-stream choice and access to
    // the context for the stage-level C ABI.
    void setPattern(const std::vector<float>& pattern);
    void setRng(uint32_t rng, uint64_t seed) { m_rng = rng; m_seed = seed; }
    bm_ctx* context() { return m_ctx; }
    const std::vector<float>& flowU() const { return m_u; }
    const std::vector<float>& flowV() const { return m_v; }

private:
    bm_params engineParams() const;

    BMParams m_params;
    bm_ctx* m_ctx;
    bool m_setup, m_verbose;
    uint32_t m_rng;
    uint64_t m_seed;
    std::vector<float> m_u, m_v;       // converted output field (m_neighX/Y)
    std::vector<unsigned char> m_vis;  // colour-coded field (m_flowVis)
};

#endif

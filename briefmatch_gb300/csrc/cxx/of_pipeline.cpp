// of_pipeline.cpp -- OFPipeline over the engine (reference: of_pipeline.cpp).
#include "of_pipeline.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <sstream>
#include <strings.h>

#include "flow_io.h"

namespace {

// The reference's option registry (util/arg_parser.*): typed options with a long
// and a short name, optional ranges, a required --input, and its error messages.
struct Opt {
    enum Kind { FLAG, UINT, FLOAT, STRING } kind;
    std::string name, shortName, help;
    void* var;
    bool optional, ranged;
    double lo, hi;
};

class Options {
public:
    std::vector<Opt> opts;
    std::string info, post;

    void flag(bool* v, const char* n, const char* s, const char* h) { opts.push_back({Opt::FLAG, n, s, h, v, true, false, 0, 0}); }
    void uint(unsigned int* v, const char* n, const char* s, const char* h, unsigned lo, unsigned hi)
    {
        opts.push_back({Opt::UINT, n, s, h, v, true, true, (double)lo, (double)hi});
    }
    void flt(float* v, const char* n, const char* s, const char* h, float lo, float hi)
    {
        opts.push_back({Opt::FLOAT, n, s, h, v, true, true, lo, hi});
    }
    void str(std::string* v, const char* n, const char* s, const char* h, bool optional = true)
    {
        opts.push_back({Opt::STRING, n, s, h, v, optional, false, 0, 0});
    }

    void help() const
    {
        std::printf("%s\n", info.c_str());
        for (const Opt& o : opts) std::printf("  %-24s %-5s %s\n", o.name.c_str(), o.shortName.c_str(), o.help.c_str());
        std::printf("%s", post.c_str());
    }

    // arg_parser.cpp:205-360
    bool read(int argc, char* argv[])
    {
        for (int i = 1; i < argc; i++) {
            if (!std::strcmp(argv[i], "--help") || !std::strcmp(argv[i], "-help") || !std::strcmp(argv[i], "--h") ||
                !std::strcmp(argv[i], "-h")) {
                help();
                return false;
            }
            bool found = false;
            for (Opt& o : opts) {
                if (std::strcmp(argv[i], o.name.c_str()) && std::strcmp(argv[i], o.shortName.c_str())) continue;
                found = true;
                if (o.kind != Opt::FLAG && argc <= ++i)
                    throw ParserException("No value provided for input option '" + std::string(argv[i - 1]) + "'");
                std::ostringstream ss;
                switch (o.kind) {
                case Opt::FLAG: *(bool*)o.var = true; break;
                case Opt::UINT: {
                    unsigned int a = (unsigned int)std::atoi(argv[i]);
                    if (o.ranged && (a < o.lo || a > o.hi)) {
                        ss << "Argument '" << argv[i - 1] << "' with value '" << a << "' is out of range. Valid range is ["
                           << (unsigned)o.lo << ", " << (unsigned)o.hi << "]";
                        throw ParserException(ss.str());
                    }
                    *(unsigned int*)o.var = a;
                    break;
                }
                case Opt::FLOAT: {
                    float a = (float)std::atof(argv[i]);
                    if (o.ranged && (a < (float)o.lo || a > (float)o.hi)) {
                        ss << "Argument '" << argv[i - 1] << "' with value '" << a << "' is out of range. Valid range is ["
                           << (float)o.lo << ", " << (float)o.hi << "]";
                        throw ParserException(ss.str());
                    }
                    *(float*)o.var = a;
                    break;
                }
                case Opt::STRING: *(std::string*)o.var = argv[i]; break;
                }
                break;
            }
            if (!found) throw ParserException("The argument '" + std::string(argv[i]) + "' is not a valid input option");
        }
        for (const Opt& o : opts) {
            if (o.optional) continue;
            bool seen = false;
            for (int i = 1; i < argc; i++)
                if (!std::strcmp(argv[i], o.name.c_str()) || !std::strcmp(argv[i], o.shortName.c_str())) seen = true;
            if (!seen) throw ParserException("Missing required option '" + o.name + "'");
        }
        return true;
    }
};

std::string format_frame(const std::string& pattern, unsigned int frame)
{
    char buf[1024];
    std::snprintf(buf, sizeof(buf), pattern.c_str(), frame);
    return buf;
}

}  // namespace

OFPipeline::OFPipeline()
    : m_doWriteMOT(false), m_doWriteFLO(false), m_doWriteLDR(false), m_verbose(false), m_doPrintError(false),
      m_endFrame(0), m_frame(0), m_stepFrame(1), m_startFrame(0), m_sx(0), m_sy(0), m_sx_in(0), m_sy_in(0), m_c(0),
      m_rng("xorwow"), m_seed(0), m_propIterations(1), m_propJfMax(128), m_propLocalSteps(2), m_propReduce(1), m_net(nullptr), m_bm(nullptr),
      m_bmP(nullptr), m_first(true)
{
}

OFPipeline::~OFPipeline() { clear(); }

void OFPipeline::clear()
{
    delete m_bm;
    if (m_net) bm_net_destroy(m_net);
    m_net = nullptr;
    delete m_bmP;
    m_bm = nullptr;
    m_bmP = nullptr;
}

std::string OFPipeline::framePath(unsigned int frame) const { return format_frame(m_input, frame); }

// of_pipeline.cpp:90-195.  Every option of both reference build variants is always
// available (the reference compiles the advanced ones only with ADVANCED_OPTIONS).
bool OFPipeline::setParams(int argc, char* argv[])
{
    m_bmP = new BMParams;
    std::string frames;
    float ux = 0, uy = 0;
    float patchRad = 3.0f, sigmaRad = 0.025f, fsizeRad = 1.0f, sSRad = 0.85f;
    Options args;
    args.info = "briefmatch -- Computes the optical flow of a sequence of frames (GB300 engine)\n\n"
                "Usage: briefmatch --input <frames> \\\n"
                "                  --frames <start_frame:step:end_frame> \\\n"
                "                  --output <output>\n";
    args.post = "\nExample: briefmatch -i frames/frame%02d.png -f 7:14 -o output/mot_%02d.flo\n";
    args.str(&m_input, "--input", "-i", "Input sequence of frames", false);
    args.str(&m_output, "--output", "-o", "Output location of the estimated optical flow (.flo, .bin or .png)");
    args.str(&frames, "--frames", "-f", "Input frames, formatted as startframe:step:endframe");
    args.flt(&m_bmP->maxmot, "--vis-max-motion", "-mm", "Max-motion clamping, in conversion of flow field to color encoding", 0.0f, 1e10f);
    args.flag(&m_verbose, "--verbose", "-v", "Verbose mode");
    args.uint(&m_bmP->N, "--feature-length", "-fl", "Length of BRIEF binary feature vectors", 2u, (unsigned)(BM_PATCH_MAX / 4));
    args.flt(&patchRad, "--patch-radius", "-pr", "BRIEF patch radius (in percent of upsampled image diagonal)", 0.0f, 100.0f);
    args.flt(&ux, "--up-sampling-x", "-ux", "Up-sampling factor for image width", 1.0f, 100.0f);
    args.flt(&uy, "--up-sampling-y", "-uy", "Up-sampling factor for image height", 1.0f, 100.0f);
    args.flt(&sigmaRad, "--sigma-downsampling", "-ss", "Down-sampling filter size (in percent of image diagonal)", 0.0f, 100.0f);
    args.uint(&m_bmP->iterations, "--iterations", "-it", "Number of iterations in neighbor search", 0u, 100u);
    args.uint(&m_bmP->jfMax, "--jf-max", "-jm", "Max distance of jump flooding scheme (should be in multiples of 2)", 2u, 10000u);
    args.flt(&fsizeRad, "--median-size", "-ms", "Median filter size in flow refinement filtering (in percent of image diagonal)", 0.0f, 100.0f);
    args.flt(&m_bmP->sEPE, "--range-epe", "-re", "Sigma for correspondence field EPE filtering term", 0.0f, 1e10f);
    args.flt(&m_bmP->sI, "--range-i", "-ri", "Sigma for input image filtering term", 0.0f, 1e10f);
    args.flt(&sSRad, "--range-spatial", "-rs", "Sigma for spatial filering size (in percent of image diagonal)", 0.0f, 100.0f);
    args.str(&m_flowGT, "--flow-gt", "-gt", "Ground truth optical flow");
    args.str(&m_rng, "--random-stream", "-rng", "Random search stream: xorwow (the reference's) or philox");
    unsigned int seed = 0;
    args.uint(&seed, "--pattern-seed", "-ps", "Seed of the BRIEF sampling pattern", 0u, 4294967295u);
    args.str(&m_proposal, "--proposal", "-pn", "Learned proposal weights (float32 file) seeding the matching");
    args.uint(&m_propIterations, "--proposal-iterations", "-pit", "Iterations when seeded by the proposal", 0u, 100u);
    args.uint(&m_propJfMax, "--proposal-jf-max", "-pjm", "Max jump-flooding distance when seeded by the proposal", 1u,
              10000u);
    args.uint(&m_propLocalSteps, "--proposal-local-steps", "-pls",
              "Local refinement steps (radius 2, then 1) after seeding by the proposal", 0u, 16u);
    args.uint(&m_propReduce, "--proposal-reduce", "-prd",
              "Proposal network on the frames reduced 1x, 2x or 4x (2 for frames much larger than 512x384)", 1u, 4u);
    if (!args.read(argc, argv)) return false;
    m_seed = seed;
    if (m_rng != "xorwow" && m_rng != "philox")
        throw ParserException("Input '" + m_rng + "' for argument '--random-stream' is not valid. Valid values are: xorwow philox");

    if (!m_output.empty()) {
        if (hasExtension(m_output.c_str(), ".flo"))
            m_doWriteFLO = true;
        else if (hasExtension(m_output.c_str(), ".bin"))
            m_doWriteMOT = true;
        else if (hasExtension(m_output.c_str(), ".png"))
            m_doWriteLDR = true;
        else
            throw ParserException("Unsupported output format. Supported formats are binary (.bin), Middlebury flow "
                                  "vector format (.flo) and color encoded images (.png).");
    }
    if (!frames.empty() && !getFrameRange(frames, m_frame, m_stepFrame, m_endFrame))
        throw ParserException("Unable to parse frame range from '" + frames + "'. Valid format is startframe:step:endframe");
    if (m_endFrame < m_frame)
        throw ParserException("Invalid frame range '" + frames + "'. End frame should be >= start frame");
    m_startFrame = m_frame;
    m_c = 0;

    std::vector<unsigned char> px;
    int w = 0, h = 0;
    try {
        bmio::read_gray8(framePath(m_frame), px, w, h);
    } catch (std::exception& e) {
        throw BriefMatchException(std::string("Cannot read image file.\n\t") + e.what());
    }
    m_sx_in = (unsigned)w;
    m_sy_in = (unsigned)h;

    // of_pipeline.cpp:178-190
    bm_params p;
    bm_params_default(&p);
    bm_params_derive(&p, m_sx_in, m_sy_in, ux, uy, patchRad, sigmaRad, fsizeRad, sSRad);
    m_sx = p.sx;
    m_sy = p.sy;
    m_bmP->sx = p.sx;
    m_bmP->sy = p.sy;
    m_bmP->sx_in = p.sx_in;
    m_bmP->sy_in = p.sy_in;
    m_bmP->patchArea = p.patchArea;
    m_bmP->sigma = p.sigma;
    m_bmP->fsize = p.fsize;
    m_bmP->sS = p.sS;
    if (m_flowGT.size() > 1) m_doPrintError = true;
    return true;
}

// of_pipeline.cpp:198-238
void OFPipeline::setup()
{
    std::fprintf(stderr, "I/O:\n");
    std::fprintf(stderr, "Input:                   %s\n", m_input.c_str());
    std::fprintf(stderr, "Image resolution:        %ux%u\n", m_sx_in, m_sy_in);
    std::fprintf(stderr, "Frames:                  %u:%u:%u\n", m_frame, m_stepFrame, m_endFrame);
    std::fprintf(stderr, "Output:                  %s\n\n", m_output.empty() ? "--" : m_output.c_str());
    m_bm = new BriefMatch;
    m_bm->setVerbose(m_verbose);
    m_bm->setParams(*m_bmP);
    m_bm->setRng(m_rng == "philox" ? BM_RNG_PHILOX : BM_RNG_XORWOW, m_seed);
    m_bm->setup();
    std::vector<float> pattern(4 * (size_t)m_bmP->N);
    bm_params p;
    bm_get_params(m_bm->context(), &p);
    bm_throw_on_error(bm_make_pattern(&p, m_seed, pattern.data()));
    m_bm->setPattern(pattern);
    if (!m_proposal.empty()) {
        // engine extension: seed every pair's matching with the learned proposal
        std::FILE* f = std::fopen(m_proposal.c_str(), "rb");
        if (!f) throw BriefMatchException("Cannot read proposal weights '" + m_proposal + "'");
        std::vector<float> w(bm_net_param_count());
        const size_t got = std::fread(w.data(), sizeof(float), w.size(), f);
        const bool extra = std::fgetc(f) != EOF;
        std::fclose(f);
        if (got != w.size() || extra)
            throw BriefMatchException("Proposal weights '" + m_proposal + "' do not hold " +
                                      std::to_string(w.size()) + " float32 parameters");
        bm_throw_on_error(bm_net_create(1, m_sy_in / 4, m_sx_in / 4, &m_net));
        bm_throw_on_error(bm_net_set_params(m_net, w.data(), w.size()));
        bm_throw_on_error(bm_set_proposal(m_bm->context(), m_net, 0.5f, m_propIterations, m_propJfMax));
        bm_throw_on_error(bm_set_local_steps(m_bm->context(), m_propLocalSteps, 2));
        bm_throw_on_error(bm_set_proposal_reduce(m_bm->context(), m_propReduce));
        std::fprintf(stderr,
                     "Proposal:                %s (%u iterations, jump-flooding max %u, %u local steps, input reduced %ux)\n\n",
                     m_proposal.c_str(), m_propIterations, m_propJfMax, m_propLocalSteps, m_propReduce);
    }
    m_frameData.resize((size_t)m_sx_in * m_sy_in);
    m_first = true;
}

// of_pipeline.cpp:241-387.  The first frame primes the matcher; every later frame
// writes the flow from the previous frame (the reference writes a flow for the first
// frame too, computed against uninitialised descriptors).
bool OFPipeline::processFrame()
{
    if (m_frame > m_endFrame) return false;
    const std::string path = framePath(m_frame);
    if (m_verbose)
        std::printf("\n\n------------------------------------------------\nProcessing frame '%s'\n", path.c_str());
    else if (m_endFrame > m_startFrame) {
        const unsigned int kv = 100 * (m_frame - m_startFrame) / (m_endFrame - m_startFrame);
        if (kv >= m_c) {
            m_c += 5;
            std::printf("\t%3u%% (frame %3u in range [%u,%u])\n", kv, m_frame, m_startFrame, m_endFrame);
        }
    }
    auto t0 = std::chrono::steady_clock::now();
    int w = 0, h = 0;
    try {
        bmio::read_gray8(path, m_frameData, w, h);
    } catch (std::exception& e) {
        throw BriefMatchException(std::string("Cannot read image file.\n\t") + e.what());
    }
    if ((unsigned)w != m_sx_in || (unsigned)h != m_sy_in)
        throw BriefMatchException("Cannot read image file.\n\tframe size differs from the first frame");
    auto t1 = std::chrono::steady_clock::now();
    bm_throw_on_error(bm_frame(m_bm->context(), m_frameData.data(), 0, nullptr, nullptr, 0));
    bm_throw_on_error(bm_synchronize(m_bm->context()));
    auto t2 = std::chrono::steady_clock::now();
    const bool hadPair = !m_first;
    m_first = false;
    if (m_doWriteMOT || m_doWriteFLO || m_doWriteLDR || m_doPrintError) m_bm->convert();
    if (m_doWriteLDR) m_bm->computeColors();
    if (m_doWriteMOT) m_bm->printRaw(format_frame(m_output, m_frame));
    if (m_doWriteFLO) m_bm->print(format_frame(m_output, m_frame));
    if (m_doWriteLDR) m_bm->printVis(format_frame(m_output, m_frame));
    if (m_doPrintError && hadPair) std::printf("Error (EPE) = %f\n\n", m_bm->error(m_flowGT));
    if (m_verbose) {
        const double rd = std::chrono::duration<double, std::milli>(t1 - t0).count();
        const double pr = std::chrono::duration<double, std::milli>(t2 - t1).count();
        std::printf("Timings:\n\tRead:\t\t\t%0.2fms\n\tProcessing:\t\t%0.2fms / %0.2ffps\n", rd, pr, 1000.0 / pr);
    }
    m_frame += m_stepFrame;
    return true;
}

bool OFPipeline::hasExtension(const char* file_name, const char* extension)
{
    if (!file_name) return false;
    return bmio::has_extension(file_name, extension);
}

// of_pipeline.cpp:408-434: "start:end" or "start:step:end"
bool OFPipeline::getFrameRange(std::string& frames, unsigned int& start, unsigned int& step, unsigned int& end)
{
    int nrDelim = 0;
    for (char ch : frames)
        if (ch == ':') nrDelim++;
    if (nrDelim < 1 || nrDelim > 2) return false;
    unsigned int* range[3] = {&start, &step, &end};
    const char* p = frames.c_str();
    char* e = nullptr;
    for (size_t i = 0; i < 3; i += 3 - nrDelim) {
        *(range[i]) = (unsigned int)std::strtol(p, &e, 10);
        if (p == e) return false;
        p = e + 1;
    }
    return true;
}

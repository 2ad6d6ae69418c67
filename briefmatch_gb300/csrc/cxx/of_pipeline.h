// of_pipeline.h -- OFPipeline (of_pipeline.h:66-97 of the reference): command-line
// options, the frame loop and file output, over the GB300 engine.
#ifndef BRIEFMATCH_GB300_CXX_OF_PIPELINE_H
#define BRIEFMATCH_GB300_CXX_OF_PIPELINE_H

#include <string>
#include <vector>

#include "briefmatch.h"

class OFPipeline {
public:
    OFPipeline();
    ~OFPipeline();
    void clear();
    bool setParams(int argc, char* argv[]);
    void setup();
    bool processFrame();

    // Engine extension: the context, for callers that mix stage-level calls in.
    BriefMatch* matcher() { return m_bm; }

private:
    bool hasExtension(const char* file_name, const char* extension);
    bool getFrameRange(std::string& frames, unsigned int& start, unsigned int& step, unsigned int& end);
    std::string framePath(unsigned int frame) const;

    bool m_doWriteMOT, m_doWriteFLO, m_doWriteLDR, m_verbose, m_doPrintError;
    unsigned int m_endFrame, m_frame, m_stepFrame, m_startFrame, m_sx, m_sy, m_sx_in, m_sy_in, m_c;
    std::string m_input, m_flowGT, m_output, m_rng, m_proposal;
    unsigned long long m_seed;
    unsigned int m_propIterations, m_propJfMax, m_propLocalSteps, m_propReduce;
    bm_net* m_net;
    BriefMatch* m_bm;
    BMParams* m_bmP;
    std::vector<unsigned char> m_frameData;
    bool m_first;
};

#endif

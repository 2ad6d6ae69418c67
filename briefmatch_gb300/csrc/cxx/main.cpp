// main.cpp -- the briefmatch command line over the GB300 engine (reference: main.cpp:44-89).
#include <cstdio>
#include <iostream>

#include "of_pipeline.h"

int main(int argc, char* argv[])
{
    OFPipeline of;
    try {
        if (!of.setParams(argc, argv)) return 1;
        of.setup();
        std::cout << "\n\nRunning optical flow loop...\n";
        while (of.processFrame()) {
        }
        std::cout << "done!\n";
    } catch (ParserException& e) {
        std::fprintf(stderr, "\nbriefmatch input error: %s\n", e.what());
        return 1;
    } catch (BriefMatchException& e) {
        std::fprintf(stderr, "\nbriefmatch error: %s\n", e.what());
        return 1;
    } catch (CudaException& e) {
        std::fprintf(stderr, "\nCuda error: %s\n", e.what());
        return 1;
    } catch (std::exception& e) {
        std::fprintf(stderr, "\nError: %s\n", e.what());
        return 1;
    }
    return 0;
}

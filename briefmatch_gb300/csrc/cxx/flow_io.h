// flow_io.h -- file formats around the flow path: Middlebury .flo, raw planes,
// 8-bit frames (PGM, and PNG when zlib is available) and the Middlebury colour code.
#ifndef BRIEFMATCH_GB300_CXX_FLOW_IO_H
#define BRIEFMATCH_GB300_CXX_FLOW_IO_H

#include <string>
#include <vector>

namespace bmio {

// Middlebury .flo ("PIEH", float 202021.25, int32 width, int32 height, then u,v
// interleaved per pixel, row-major) -- flowIO.cpp:96-133 / :46-93.
void write_flo(const std::string& path, const float* u, const float* v, int width, int height);
void read_flo(const std::string& path, std::vector<float>& u, std::vector<float>& v, int& width, int& height);

// Raw planes: all u, then all v, float32 -- briefmatch.cpp:442-452.
void write_raw(const std::string& path, const float* u, const float* v, int width, int height);

// 8-bit frame as grayscale (colour input is converted with 0.299/0.587/0.114 weights).
// Supports binary PGM/PPM and, when built with zlib, PNG (8-bit, non-interlaced).
void read_gray8(const std::string& path, std::vector<unsigned char>& pixels, int& width, int& height);
void write_pgm(const std::string& path, const unsigned char* pixels, int width, int height);
void write_png_rgb(const std::string& path, const unsigned char* rgb, int width, int height);
bool png_supported();

// Middlebury colour coding of one vector already divided by the normalising radius
// (colorcode.cpp:52-74 algorithm: a 55-entry hue wheel, saturation by magnitude,
// darkened beyond radius 1).  Writes R, G, B.
void flow_color(float fx, float fy, unsigned char* rgb);
bool unknown_flow(float u, float v);

bool has_extension(const std::string& name, const std::string& ext);

}  // namespace bmio

#endif

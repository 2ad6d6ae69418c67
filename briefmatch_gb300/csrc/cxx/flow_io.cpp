// flow_io.cpp -- see flow_io.h.
#include "flow_io.h"

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <strings.h>

#ifdef BM_HAVE_ZLIB
#include <zlib.h>
#endif

namespace bmio {

namespace {

const float kFloTag = 202021.25f;

struct File {
    FILE* f;
    File(const std::string& p, const char* mode) : f(std::fopen(p.c_str(), mode)) {}
    ~File()
    {
        if (f) std::fclose(f);
    }
};

void put_u32be(std::vector<unsigned char>& out, uint32_t v)
{
    out.push_back((unsigned char)(v >> 24));
    out.push_back((unsigned char)(v >> 16));
    out.push_back((unsigned char)(v >> 8));
    out.push_back((unsigned char)v);
}

uint32_t get_u32be(const unsigned char* p) { return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3]; }

unsigned char to_gray(int r, int g, int b)
{
    // Rec.601 luma with rounding, as grayscale loaders commonly do
    return (unsigned char)((r * 4899 + g * 9617 + b * 1868 + 8192) >> 14);
}

}  // namespace

bool has_extension(const std::string& name, const std::string& ext)
{
    if (ext.size() >= name.size()) return false;
    return strcasecmp(name.c_str() + name.size() - ext.size(), ext.c_str()) == 0;
}

void write_flo(const std::string& path, const float* u, const float* v, int width, int height)
{
    File f(path, "wb");
    if (!f.f) throw std::runtime_error("Cannot write .flo file '" + path + "'.");
    std::fwrite(&kFloTag, sizeof(float), 1, f.f);
    int32_t wh[2] = {width, height};
    std::fwrite(wh, sizeof(int32_t), 2, f.f);
    std::vector<float> row(2 * (size_t)width);
    for (int y = 0; y < height; y++) {
        for (int x = 0; x < width; x++) {
            row[2 * x] = u[(size_t)y * width + x];
            row[2 * x + 1] = v[(size_t)y * width + x];
        }
        if (std::fwrite(row.data(), sizeof(float), row.size(), f.f) != row.size())
            throw std::runtime_error("Short write to '" + path + "'.");
    }
}

void read_flo(const std::string& path, std::vector<float>& u, std::vector<float>& v, int& width, int& height)
{
    File f(path, "rb");
    if (!f.f) throw std::runtime_error("Cannot open .flo file '" + path + "'.");
    float tag = 0;
    int32_t wh[2] = {0, 0};
    if (std::fread(&tag, sizeof(float), 1, f.f) != 1 || tag != kFloTag)
        throw std::runtime_error("'" + path + "' is not a .flo file (wrong tag).");
    if (std::fread(wh, sizeof(int32_t), 2, f.f) != 2 || wh[0] < 1 || wh[1] < 1 || wh[0] > 99999 || wh[1] > 99999)
        throw std::runtime_error("'" + path + "': illegal .flo size.");
    width = wh[0];
    height = wh[1];
    const size_t n = (size_t)width * height;
    std::vector<float> buf(2 * n);
    if (std::fread(buf.data(), sizeof(float), buf.size(), f.f) != buf.size())
        throw std::runtime_error("'" + path + "': file is too short.");
    u.resize(n);
    v.resize(n);
    for (size_t i = 0; i < n; i++) {
        u[i] = buf[2 * i];
        v[i] = buf[2 * i + 1];
    }
}

void write_raw(const std::string& path, const float* u, const float* v, int width, int height)
{
    File f(path, "wb");
    if (!f.f) throw std::runtime_error("Invalid output path. Cannot write to file '" + path + "'.");
    const size_t n = (size_t)width * height;
    if (std::fwrite(u, sizeof(float), n, f.f) != n || std::fwrite(v, sizeof(float), n, f.f) != n)
        throw std::runtime_error("Short write to '" + path + "'.");
}

void write_pgm(const std::string& path, const unsigned char* px, int width, int height)
{
    File f(path, "wb");
    if (!f.f) throw std::runtime_error("Cannot write '" + path + "'.");
    std::fprintf(f.f, "P5\n%d %d\n255\n", width, height);
    std::fwrite(px, 1, (size_t)width * height, f.f);
}

static void read_pnm(const std::string& path, std::vector<unsigned char>& out, int& width, int& height)
{
    File f(path, "rb");
    if (!f.f) throw std::runtime_error("Input image '" + path + "' not found.");
    char magic[3] = {0, 0, 0};
    if (std::fread(magic, 1, 2, f.f) != 2 || magic[0] != 'P' || (magic[1] != '5' && magic[1] != '6'))
        throw std::runtime_error("'" + path + "': only binary PGM (P5) and PPM (P6) are supported.");
    int vals[3];
    for (int k = 0; k < 3; k++) {
        int c = std::fgetc(f.f);
        while (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '#') {
            if (c == '#')
                while (c != '\n' && c != EOF) c = std::fgetc(f.f);
            c = std::fgetc(f.f);
        }
        int v = 0;
        if (c < '0' || c > '9') throw std::runtime_error("'" + path + "': bad header.");
        while (c >= '0' && c <= '9') {
            v = v * 10 + (c - '0');
            c = std::fgetc(f.f);
        }
        vals[k] = v;
    }
    width = vals[0];
    height = vals[1];
    if (vals[2] != 255 || width < 1 || height < 1) throw std::runtime_error("'" + path + "': only 8-bit images.");
    const int ch = magic[1] == '5' ? 1 : 3;
    std::vector<unsigned char> raw((size_t)width * height * ch);
    if (std::fread(raw.data(), 1, raw.size(), f.f) != raw.size()) throw std::runtime_error("'" + path + "': truncated.");
    out.resize((size_t)width * height);
    for (size_t i = 0; i < out.size(); i++)
        out[i] = ch == 1 ? raw[i] : to_gray(raw[3 * i], raw[3 * i + 1], raw[3 * i + 2]);
}

#ifdef BM_HAVE_ZLIB
static int paeth(int a, int b, int c)
{
    int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if (pa <= pb && pa <= pc) return a;
    return pb <= pc ? b : c;
}

static void read_png(const std::string& path, std::vector<unsigned char>& out, int& width, int& height)
{
    File f(path, "rb");
    if (!f.f) throw std::runtime_error("Input image '" + path + "' not found.");
    std::vector<unsigned char> data;
    unsigned char buf[65536];
    size_t got;
    while ((got = std::fread(buf, 1, sizeof(buf), f.f)) > 0) data.insert(data.end(), buf, buf + got);
    static const unsigned char sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
    if (data.size() < 8 || std::memcmp(data.data(), sig, 8) != 0) throw std::runtime_error("'" + path + "' is not a PNG.");
    size_t pos = 8;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<unsigned char> idat, palette;
    width = height = 0;
    while (pos + 8 <= data.size()) {
        const uint32_t len = get_u32be(&data[pos]);
        const char* type = (const char*)&data[pos + 4];
        if (pos + 12 + (size_t)len > data.size()) throw std::runtime_error("'" + path + "': truncated chunk.");
        const unsigned char* body = &data[pos + 8];
        if (!std::memcmp(type, "IHDR", 4)) {
            width = (int)get_u32be(body);
            height = (int)get_u32be(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
        } else if (!std::memcmp(type, "PLTE", 4)) {
            palette.assign(body, body + len);
        } else if (!std::memcmp(type, "IDAT", 4)) {
            idat.insert(idat.end(), body, body + len);
        } else if (!std::memcmp(type, "IEND", 4)) {
            break;
        }
        pos += 12 + len;
    }
    if (width < 1 || height < 1 || depth != 8 || interlace != 0)
        throw std::runtime_error("'" + path + "': only 8-bit non-interlaced PNG is supported.");
    int ch;
    switch (ctype) {
    case 0: ch = 1; break;
    case 2: ch = 3; break;
    case 3: ch = 1; break;
    case 4: ch = 2; break;
    case 6: ch = 4; break;
    default: throw std::runtime_error("'" + path + "': unsupported PNG colour type.");
    }
    const size_t stride = (size_t)width * ch;
    std::vector<unsigned char> raw((stride + 1) * height);
    uLongf rawlen = (uLongf)raw.size();
    if (uncompress(raw.data(), &rawlen, idat.data(), (uLong)idat.size()) != Z_OK || rawlen != raw.size())
        throw std::runtime_error("'" + path + "': corrupt PNG data.");
    std::vector<unsigned char> img(stride * height), prev(stride, 0);
    for (int y = 0; y < height; y++) {
        const unsigned char ft = raw[y * (stride + 1)];
        const unsigned char* src = &raw[y * (stride + 1) + 1];
        unsigned char* dst = &img[y * stride];
        for (size_t i = 0; i < stride; i++) {
            const int a = i >= (size_t)ch ? dst[i - ch] : 0, b = prev[i], c = i >= (size_t)ch ? prev[i - ch] : 0;
            int v = src[i];
            switch (ft) {
            case 0: break;
            case 1: v += a; break;
            case 2: v += b; break;
            case 3: v += (a + b) / 2; break;
            case 4: v += paeth(a, b, c); break;
            default: throw std::runtime_error("'" + path + "': bad PNG filter.");
            }
            dst[i] = (unsigned char)v;
        }
        std::memcpy(prev.data(), dst, stride);
    }
    out.resize((size_t)width * height);
    for (size_t i = 0; i < out.size(); i++) {
        const unsigned char* p = &img[i * ch];
        if (ctype == 0 || ctype == 4) {
            out[i] = p[0];
        } else if (ctype == 3) {
            const size_t k = (size_t)p[0] * 3;
            if (k + 2 >= palette.size()) throw std::runtime_error("'" + path + "': bad palette index.");
            out[i] = to_gray(palette[k], palette[k + 1], palette[k + 2]);
        } else {
            out[i] = to_gray(p[0], p[1], p[2]);
        }
    }
}

void write_png_rgb(const std::string& path, const unsigned char* rgb, int width, int height)
{
    const size_t stride = (size_t)width * 3;
    std::vector<unsigned char> raw((stride + 1) * height);
    for (int y = 0; y < height; y++) {
        raw[y * (stride + 1)] = 0;
        std::memcpy(&raw[y * (stride + 1) + 1], rgb + y * stride, stride);
    }
    uLongf zlen = compressBound((uLong)raw.size());
    std::vector<unsigned char> z(zlen);
    if (compress2(z.data(), &zlen, raw.data(), (uLong)raw.size(), 6) != Z_OK)
        throw std::runtime_error("PNG compression failed.");
    z.resize(zlen);
    std::vector<unsigned char> out = {137, 80, 78, 71, 13, 10, 26, 10};
    auto chunk = [&](const char* type, const std::vector<unsigned char>& body) {
        put_u32be(out, (uint32_t)body.size());
        const size_t start = out.size();
        out.insert(out.end(), type, type + 4);
        out.insert(out.end(), body.begin(), body.end());
        put_u32be(out, (uint32_t)crc32(0L, &out[start], (uInt)(out.size() - start)));
    };
    std::vector<unsigned char> ihdr;
    put_u32be(ihdr, (uint32_t)width);
    put_u32be(ihdr, (uint32_t)height);
    ihdr.insert(ihdr.end(), {8, 2, 0, 0, 0});
    chunk("IHDR", ihdr);
    chunk("IDAT", z);
    chunk("IEND", {});
    File f(path, "wb");
    if (!f.f || std::fwrite(out.data(), 1, out.size(), f.f) != out.size())
        throw std::runtime_error("Cannot write to image file '" + path + "'.");
}

bool png_supported() { return true; }
#else
static void read_png(const std::string& path, std::vector<unsigned char>&, int&, int&)
{
    throw std::runtime_error("'" + path + "': PNG support was not built (zlib missing); use PGM input.");
}
void write_png_rgb(const std::string& path, const unsigned char*, int, int)
{
    throw std::runtime_error("'" + path + "': PNG support was not built (zlib missing).");
}
bool png_supported() { return false; }
#endif

void read_gray8(const std::string& path, std::vector<unsigned char>& pixels, int& width, int& height)
{
    if (has_extension(path, ".png"))
        read_png(path, pixels, width, height);
    else
        read_pnm(path, pixels, width, height);
}

bool unknown_flow(float u, float v)
{
    // flowIO.cpp:35-39: |u| or |v| above 1e9, or NaN
    return std::fabs(u) > 1e9f || std::fabs(v) > 1e9f || u != u || v != v;
}

void flow_color(float fx, float fy, unsigned char* rgb)
{
    // The hue wheel, colorcode.cpp:27-50: red->yellow 15 steps, yellow->green 6,
    // green->cyan 4, cyan->blue 11, blue->magenta 13, magenta->red 6; each ramp is an
    // integer division 255*i/steps.
    static int wheel[55][3];
    static bool built = false;
    if (!built) {
        const int seg[6] = {15, 6, 4, 11, 13, 6};
        // start colour of each segment and the channel that ramps (+1 up, -1 down)
        const int start[6][3] = {{255, 0, 0}, {255, 255, 0}, {0, 255, 0}, {0, 255, 255}, {0, 0, 255}, {255, 0, 255}};
        const int ramp_ch[6] = {1, 0, 2, 1, 0, 2};
        const int ramp_dir[6] = {1, -1, 1, -1, 1, -1};
        int k = 0;
        for (int s = 0; s < 6; s++)
            for (int i = 0; i < seg[s]; i++, k++) {
                for (int c = 0; c < 3; c++) wheel[k][c] = start[s][c];
                wheel[k][ramp_ch[s]] = ramp_dir[s] > 0 ? 255 * i / seg[s] : 255 - 255 * i / seg[s];
            }
        built = true;
    }
    // colorcode.cpp:57-72 with its declared types (rad, a, fk, f, col0, col1, col are
    // float; 1.0, 2.0, pi, .75 and 255.0 are double).  The float atan2 is the correctly
    // rounded one, as on the GPU (bm_colors).
    const int ncols = 55;
    const float rad = std::sqrt(fx * fx + fy * fy);
    const float at = (float)std::atan2(-(double)fy, -(double)fx);
    const float a = (float)((double)at / M_PI);
    const float fk = (float)(((double)a + 1.0) / 2.0 * (ncols - 1));
    const int k0 = (int)fk;
    const int k1 = (k0 + 1) % ncols;
    const float f = fk - (float)k0;
    for (int c = 0; c < 3; c++) {
        const float col0 = (float)(wheel[k0][c] / 255.0);
        const float col1 = (float)(wheel[k1][c] / 255.0);
        float col = (1 - f) * col0 + f * col1;
        if (rad <= 1)
            col = 1 - rad * (1 - col);
        else
            col = (float)((double)col * .75);
        rgb[c] = (unsigned char)(int)(255.0 * (double)col);
    }
}

}  // namespace bmio

// Image files written by the `save` post-processor: SaveToImage::process
// (builtin/btrc/builtin/postprocess/save_to_image.cpp:30-61) and Image<T>::save
// (common/btrc/utils/image.h:495-550). The format follows the file extension
// (image.cpp:177-190). Pixel conversion follows the reference: PNG stores 8-bit RGBA with
// byte = min(int(v * 256), 255) (image.h:207-217) and alpha 255; EXR stores float B, G, R
// channels; HDR stores RGBE. The encoders are our own: PNG with stored (uncompressed)
// deflate blocks, EXR uncompressed scanlines, HDR flat RGBE scanlines; the pixel content
// is what the reference writes, the byte streams are not.
#include "image_io.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace bt {

namespace {

std::string upper_ext(const std::string &fn)
{
    const size_t dot = fn.find_last_of('.');
    const size_t slash = fn.find_last_of("/\\");
    if(dot == std::string::npos || (slash != std::string::npos && dot < slash))
        return "";
    std::string e = fn.substr(dot);
    for(char &c : e)
        if(c >= 'a' && c <= 'z')
            c = static_cast<char>(c - 'a' + 'A');
    return e;
}

uint32_t crc32_update(uint32_t crc, const unsigned char *p, size_t n)
{
    static uint32_t table[256];
    static bool init = false;
    if(!init)
    {
        for(uint32_t i = 0; i < 256; ++i)
        {
            uint32_t c = i;
            for(int k = 0; k < 8; ++k)
                c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    crc = ~crc;
    for(size_t i = 0; i < n; ++i)
        crc = table[(crc ^ p[i]) & 0xffu] ^ (crc >> 8);
    return ~crc;
}

void put_be32(std::vector<unsigned char> &v, uint32_t x)
{
    v.push_back(static_cast<unsigned char>(x >> 24));
    v.push_back(static_cast<unsigned char>(x >> 16));
    v.push_back(static_cast<unsigned char>(x >> 8));
    v.push_back(static_cast<unsigned char>(x));
}

void put_le32(std::vector<unsigned char> &v, uint32_t x)
{
    for(int k = 0; k < 4; ++k)
        v.push_back(static_cast<unsigned char>(x >> (8 * k)));
}

void put_le64(std::vector<unsigned char> &v, uint64_t x)
{
    for(int k = 0; k < 8; ++k)
        v.push_back(static_cast<unsigned char>(x >> (8 * k)));
}

void png_chunk(std::vector<unsigned char> &out, const char *type, const std::vector<unsigned char> &data)
{
    put_be32(out, static_cast<uint32_t>(data.size()));
    std::vector<unsigned char> td(type, type + 4);
    td.insert(td.end(), data.begin(), data.end());
    out.insert(out.end(), td.begin(), td.end());
    put_be32(out, crc32_update(0, td.data(), td.size()));
}

void write_file(const std::string &fn, const std::vector<unsigned char> &bytes)
{
    std::ofstream f(fn, std::ios::binary);
    if(!f)
        throw std::runtime_error("failed to open file for writing: " + fn);
    f.write(reinterpret_cast<const char *>(bytes.data()), static_cast<std::streamsize>(bytes.size()));
    if(!f)
        throw std::runtime_error("failed to write file: " + fn);
}

// to_component<uint8_t, float> (common/btrc/utils/image.h:207-217):
// uint8_t(min(int(v * 256), 255)), negative values wrapping modulo 256. A product outside
// the int range or NaN converts to INT_MIN, as the x86-64 conversion instruction does,
// which gives byte 0.
unsigned char to_byte(float v)
{
    const float s = v * 256.0f;
    int i = INT32_MIN;
    if(s > -2147483648.0f && s < 2147483648.0f)
        i = static_cast<int>(s);
    i = std::min(i, 255);
    return static_cast<unsigned char>(static_cast<unsigned int>(i) & 0xffu);
}

void save_png(const std::string &fn, const std::vector<float> &rgba, int w, int h)
{
    // raw scanlines: filter byte 0 + RGBA8
    std::vector<unsigned char> raw;
    raw.reserve(static_cast<size_t>(h) * (1 + 4 * static_cast<size_t>(w)));
    for(int y = 0; y < h; ++y)
    {
        raw.push_back(0);
        for(int x = 0; x < w; ++x)
            for(int c = 0; c < 4; ++c)
                raw.push_back(to_byte(rgba[(static_cast<size_t>(y) * w + x) * 4 + c]));
    }
    // zlib stream of stored deflate blocks (RFC 1950 / 1951)
    std::vector<unsigned char> z = { 0x78, 0x01 };
    size_t pos = 0;
    do
    {
        const size_t len = std::min<size_t>(65535, raw.size() - pos);
        const bool last = pos + len == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(static_cast<unsigned char>(len & 0xff));
        z.push_back(static_cast<unsigned char>(len >> 8));
        z.push_back(static_cast<unsigned char>(~len & 0xff));
        z.push_back(static_cast<unsigned char>((~len >> 8) & 0xff));
        z.insert(z.end(), raw.begin() + static_cast<long>(pos), raw.begin() + static_cast<long>(pos + len));
        pos += len;
    } while(pos < raw.size());
    uint32_t a = 1, b = 0;
    for(unsigned char c : raw)
    {
        a = (a + c) % 65521u;
        b = (b + a) % 65521u;
    }
    put_be32(z, (b << 16) | a);

    std::vector<unsigned char> out = { 0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n' };
    std::vector<unsigned char> ihdr;
    put_be32(ihdr, static_cast<uint32_t>(w));
    put_be32(ihdr, static_cast<uint32_t>(h));
    ihdr.push_back(8);   // bit depth
    ihdr.push_back(6);   // colour type RGBA
    ihdr.push_back(0);
    ihdr.push_back(0);
    ihdr.push_back(0);
    png_chunk(out, "IHDR", ihdr);
    png_chunk(out, "IDAT", z);
    png_chunk(out, "IEND", {});
    write_file(fn, out);
}

void exr_attr(std::vector<unsigned char> &h, const char *name, const char *type, const std::vector<unsigned char> &v)
{
    h.insert(h.end(), name, name + std::strlen(name) + 1);
    h.insert(h.end(), type, type + std::strlen(type) + 1);
    put_le32(h, static_cast<uint32_t>(v.size()));
    h.insert(h.end(), v.begin(), v.end());
}

// OpenEXR 2 single-part scanline file, no compression, FLOAT channels B, G, R
void save_exr(const std::string &fn, const std::vector<float> &rgba, int w, int h)
{
    std::vector<unsigned char> out;
    put_le32(out, 20000630u);  // magic
    put_le32(out, 2u);         // version 2, single-part scanline
    std::vector<unsigned char> v;
    for(const char *ch : { "B", "G", "R" })
    {
        v.insert(v.end(), ch, ch + 2);
        put_le32(v, 2u);           // FLOAT
        v.push_back(0);            // pLinear
        v.push_back(0); v.push_back(0); v.push_back(0);
        put_le32(v, 1u);           // xSampling
        put_le32(v, 1u);           // ySampling
    }
    v.push_back(0);
    exr_attr(out, "channels", "chlist", v);
    exr_attr(out, "compression", "compression", { 0 });
    v.clear();
    put_le32(v, 0); put_le32(v, 0); put_le32(v, static_cast<uint32_t>(w - 1)); put_le32(v, static_cast<uint32_t>(h - 1));
    exr_attr(out, "dataWindow", "box2i", v);
    exr_attr(out, "displayWindow", "box2i", v);
    exr_attr(out, "lineOrder", "lineOrder", { 0 });
    const float one = 1.0f, zero = 0.0f;
    v.assign(reinterpret_cast<const unsigned char *>(&one), reinterpret_cast<const unsigned char *>(&one) + 4);
    exr_attr(out, "pixelAspectRatio", "float", v);
    v.clear();
    v.insert(v.end(), reinterpret_cast<const unsigned char *>(&zero), reinterpret_cast<const unsigned char *>(&zero) + 4);
    v.insert(v.end(), reinterpret_cast<const unsigned char *>(&zero), reinterpret_cast<const unsigned char *>(&zero) + 4);
    exr_attr(out, "screenWindowCenter", "v2f", v);
    v.assign(reinterpret_cast<const unsigned char *>(&one), reinterpret_cast<const unsigned char *>(&one) + 4);
    exr_attr(out, "screenWindowWidth", "float", v);
    out.push_back(0);  // end of header
    const uint64_t line_bytes = 8ull + 3ull * 4ull * static_cast<uint64_t>(w);
    const uint64_t table_end = out.size() + 8ull * static_cast<uint64_t>(h);
    for(int y = 0; y < h; ++y)
        put_le64(out, table_end + static_cast<uint64_t>(y) * line_bytes);
    for(int y = 0; y < h; ++y)
    {
        put_le32(out, static_cast<uint32_t>(y));
        put_le32(out, static_cast<uint32_t>(3 * 4 * w));
        for(int c : { 2, 1, 0 })
            for(int x = 0; x < w; ++x)
            {
                const float f = rgba[(static_cast<size_t>(y) * w + x) * 4 + c];
                uint32_t bits;
                std::memcpy(&bits, &f, 4);
                put_le32(out, bits);
            }
    }
    write_file(fn, out);
}

// Radiance RGBE (Ward), flat scanlines
void save_hdr(const std::string &fn, const std::vector<float> &rgba, int w, int h)
{
    std::string head = "#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y " + std::to_string(h) + " +X " + std::to_string(w) + "\n";
    std::vector<unsigned char> out(head.begin(), head.end());
    for(size_t i = 0; i < static_cast<size_t>(w) * h; ++i)
    {
        const float r = std::max(rgba[i * 4 + 0], 0.0f), g = std::max(rgba[i * 4 + 1], 0.0f),
                    b = std::max(rgba[i * 4 + 2], 0.0f);
        const float m = std::max(r, std::max(g, b));
        if(!(m >= 1e-32f) || !std::isfinite(m))
        {
            out.insert(out.end(), { 0, 0, 0, 0 });
            continue;
        }
        int e;
        const float s = std::frexp(m, &e) * 256.0f / m;
        out.push_back(static_cast<unsigned char>(r * s));
        out.push_back(static_cast<unsigned char>(g * s));
        out.push_back(static_cast<unsigned char>(b * s));
        out.push_back(static_cast<unsigned char>(e + 128));
    }
    write_file(fn, out);
}

} // namespace

void save_image(const std::string &filename, const float *pixels, int width, int height, int channels, float gamma)
{
    if(width <= 0 || height <= 0 || (channels != 3 && channels != 4))
        throw std::invalid_argument("save_image: bad image size or channel count");
    const std::string ext = upper_ext(filename);
    // Image<Vec4f> with alpha 1 for 3-channel input, raised to 1 / gamma (pow_ on all
    // four components, so alpha stays 1)
    std::vector<float> rgba(static_cast<size_t>(width) * height * 4);
    const float inv_gamma = 1.0f / gamma;
    for(size_t i = 0; i < static_cast<size_t>(width) * height; ++i)
    {
        for(int c = 0; c < 4; ++c)
        {
            const float v = c < channels ? pixels[i * channels + c] : 1.0f;
            rgba[i * 4 + c] = gamma == 1.0f ? v : std::pow(v, inv_gamma);
        }
    }
    if(ext == ".PNG")
        save_png(filename, rgba, width, height);
    else if(ext == ".EXR")
        save_exr(filename, rgba, width, height);
    else if(ext == ".HDR")
        save_hdr(filename, rgba, width, height);
    else if(ext == ".JPG" || ext == ".JPEG")
        throw UnsupportedFormat("JPEG output is not supported: " + filename);
    else
        throw std::invalid_argument("unknown image format: " + ext);
}

} // namespace bt

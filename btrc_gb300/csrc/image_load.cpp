// Image files read by 2D `array` textures (builtin/btrc/builtin/texture2d/array2d.cpp:37-45
// through cuda::Texture::initialize(filename) and ImageDynamic::load,
// common/btrc/utils/image.cpp:296-346): PNG (8-bit, 1 / 3 / 4 channels after palette
// expansion, 16-bit samples reduced to their high byte) and Radiance HDR. JPEG is not
// decoded here (BTRC_ERR_UNSUPPORTED); the reference itself cannot load EXR. The decoders
// are our own: inflate per RFC 1951 and the PNG filters per the PNG specification.
#include "image_io.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <vector>

namespace bt {

namespace {

std::vector<unsigned char> read_all(const std::string &fn)
{
    std::ifstream f(fn, std::ios::binary);
    if(!f)
        throw std::runtime_error("failed to open file: " + fn);
    return std::vector<unsigned char>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

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

// ---------------------------------------------------------------- inflate (RFC 1951)

struct BitReader
{
    const unsigned char *p;
    size_t n, pos = 0;
    uint32_t buf = 0;
    int cnt = 0;

    int bit()
    {
        if(cnt == 0)
        {
            if(pos >= n)
                throw std::runtime_error("inflate: unexpected end of data");
            buf = p[pos++];
            cnt = 8;
        }
        const int b = static_cast<int>(buf & 1u);
        buf >>= 1;
        --cnt;
        return b;
    }
    uint32_t bits(int k)
    {
        uint32_t v = 0;
        for(int i = 0; i < k; ++i)
            v |= static_cast<uint32_t>(bit()) << i;
        return v;
    }
    void align() { cnt = 0; }
};

// canonical Huffman code: symbol counts per length and symbols sorted by code
struct Huffman
{
    int count[16] = {};
    std::vector<int> symbol;

    void build(const int *lengths, int n)
    {
        std::fill(count, count + 16, 0);
        for(int i = 0; i < n; ++i)
            ++count[lengths[i]];
        count[0] = 0;
        int offs[16] = {};
        for(int l = 1; l < 16; ++l)
            offs[l] = offs[l - 1] + count[l - 1];
        symbol.assign(n, 0);
        for(int i = 0; i < n; ++i)
            if(lengths[i] != 0)
                symbol[offs[lengths[i]]++] = i;
    }

    int decode(BitReader &br) const
    {
        int code = 0, first = 0, index = 0;
        for(int l = 1; l < 16; ++l)
        {
            code |= br.bit();
            const int c = count[l];
            if(code - first < c)
                return symbol[index + (code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        throw std::runtime_error("inflate: bad Huffman code");
    }
};

const int LEN_BASE[29] = { 3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                           35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258 };
const int LEN_EXTRA[29] = { 0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0 };
const int DIST_BASE[30] = { 1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193, 257, 385, 513, 769,
                            1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577 };
const int DIST_EXTRA[30] = { 0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13 };

void inflate_block(BitReader &br, std::vector<unsigned char> &out, const Huffman &lit, const Huffman &dist)
{
    for(;;)
    {
        const int sym = lit.decode(br);
        if(sym < 256)
            out.push_back(static_cast<unsigned char>(sym));
        else if(sym == 256)
            return;
        else
        {
            const int li = sym - 257;
            if(li >= 29)
                throw std::runtime_error("inflate: bad length symbol");
            const int len = LEN_BASE[li] + static_cast<int>(br.bits(LEN_EXTRA[li]));
            const int di = dist.decode(br);
            if(di >= 30)
                throw std::runtime_error("inflate: bad distance symbol");
            const size_t d = static_cast<size_t>(DIST_BASE[di]) + br.bits(DIST_EXTRA[di]);
            if(d > out.size())
                throw std::runtime_error("inflate: distance too far back");
            const size_t from = out.size() - d;
            for(int k = 0; k < len; ++k)
                out.push_back(out[from + k]);
        }
    }
}

std::vector<unsigned char> zlib_inflate(const unsigned char *p, size_t n)
{
    if(n < 2 || (p[0] & 0x0f) != 8 || ((p[0] << 8) | p[1]) % 31 != 0 || (p[1] & 0x20))
        throw std::runtime_error("inflate: bad zlib header");
    BitReader br{ p + 2, n - 2 };
    std::vector<unsigned char> out;
    int final_block = 0;
    while(!final_block)
    {
        final_block = br.bit();
        const uint32_t type = br.bits(2);
        if(type == 0)
        {
            br.align();
            if(br.pos + 4 > br.n)
                throw std::runtime_error("inflate: truncated stored block");
            const uint32_t len = br.p[br.pos] | (br.p[br.pos + 1] << 8);
            const uint32_t nlen = br.p[br.pos + 2] | (br.p[br.pos + 3] << 8);
            if((len ^ 0xffffu) != nlen)
                throw std::runtime_error("inflate: stored block length mismatch");
            br.pos += 4;
            if(br.pos + len > br.n)
                throw std::runtime_error("inflate: truncated stored block");
            out.insert(out.end(), br.p + br.pos, br.p + br.pos + len);
            br.pos += len;
        }
        else if(type == 1)
        {
            // the fixed codes, built once (thread-safe static initialisation)
            struct Fixed
            {
                Huffman lit, dist;
                Fixed()
                {
                    int l[288];
                    for(int i = 0; i < 288; ++i)
                        l[i] = i < 144 ? 8 : i < 256 ? 9 : i < 280 ? 7 : 8;
                    lit.build(l, 288);
                    int d[30];
                    for(int &v : d)
                        v = 5;
                    dist.build(d, 30);
                }
            };
            static const Fixed fixed;
            inflate_block(br, out, fixed.lit, fixed.dist);
        }
        else if(type == 2)
        {
            const int hlit = static_cast<int>(br.bits(5)) + 257, hdist = static_cast<int>(br.bits(5)) + 1,
                      hclen = static_cast<int>(br.bits(4)) + 4;
            static const int ORDER[19] = { 16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15 };
            int cl[19] = {};
            for(int i = 0; i < hclen; ++i)
                cl[ORDER[i]] = static_cast<int>(br.bits(3));
            Huffman clh;
            clh.build(cl, 19);
            int lens[320] = {};
            int i = 0;
            while(i < hlit + hdist)
            {
                const int sym = clh.decode(br);
                if(sym < 16)
                    lens[i++] = sym;
                else
                {
                    int rep = 0, val = 0;
                    if(sym == 16)
                    {
                        if(i == 0)
                            throw std::runtime_error("inflate: repeat without a previous length");
                        val = lens[i - 1];
                        rep = 3 + static_cast<int>(br.bits(2));
                    }
                    else if(sym == 17)
                        rep = 3 + static_cast<int>(br.bits(3));
                    else
                        rep = 11 + static_cast<int>(br.bits(7));
                    if(i + rep > hlit + hdist)
                        throw std::runtime_error("inflate: too many code lengths");
                    while(rep--)
                        lens[i++] = val;
                }
            }
            Huffman lit, dist;
            lit.build(lens, hlit);
            dist.build(lens + hlit, hdist);
            inflate_block(br, out, lit, dist);
        }
        else
            throw std::runtime_error("inflate: bad block type");
    }
    return out;
}

// ---------------------------------------------------------------- PNG

uint32_t be32(const unsigned char *p)
{
    return (static_cast<uint32_t>(p[0]) << 24) | (static_cast<uint32_t>(p[1]) << 16) |
           (static_cast<uint32_t>(p[2]) << 8) | p[3];
}

int paeth(int a, int b, int c)
{
    const int p = a + b - c, pa = std::abs(p - a), pb = std::abs(p - b), pc = std::abs(p - c);
    if(pa <= pb && pa <= pc)
        return a;
    return pb <= pc ? b : c;
}

LoadedImage load_png(const std::string &fn)
{
    const std::vector<unsigned char> d = read_all(fn);
    static const unsigned char SIG[8] = { 0x89, 'P', 'N', 'G', '\r', '\n', 0x1a, '\n' };
    if(d.size() < 8 || std::memcmp(d.data(), SIG, 8) != 0)
        throw std::runtime_error("not a PNG file: " + fn);
    size_t pos = 8;
    uint32_t w = 0, h = 0;
    int depth = 0, ctype = -1, interlace = 0;
    std::vector<unsigned char> idat, palette, trns;
    while(pos + 12 <= d.size())
    {
        const uint32_t len = be32(&d[pos]);
        if(pos + 12 + static_cast<size_t>(len) > d.size())
            throw std::runtime_error("truncated PNG chunk: " + fn);
        const std::string type(reinterpret_cast<const char *>(&d[pos + 4]), 4);
        const unsigned char *body = &d[pos + 8];
        if(type == "IHDR")
        {
            if(len < 13)
                throw std::runtime_error("bad PNG header: " + fn);
            w = be32(body);
            h = be32(body + 4);
            depth = body[8];
            ctype = body[9];
            interlace = body[12];
        }
        else if(type == "PLTE")
            palette.assign(body, body + len);
        else if(type == "tRNS")
            trns.assign(body, body + len);
        else if(type == "IDAT")
            idat.insert(idat.end(), body, body + len);
        else if(type == "IEND")
            break;
        pos += 12 + static_cast<size_t>(len);
    }
    if(w == 0 || h == 0 || w > (1u << 16) || h > (1u << 16))
        throw std::runtime_error("bad PNG size: " + fn);
    if(interlace != 0)
        throw UnsupportedFormat("interlaced PNG is not supported: " + fn);
    int samples;
    switch(ctype)
    {
    case 0: samples = 1; break;
    case 2: samples = 3; break;
    case 3: samples = 1; break;
    case 4: samples = 2; break;
    case 6: samples = 4; break;
    default: throw std::runtime_error("bad PNG colour type: " + fn);
    }
    if(!(depth == 1 || depth == 2 || depth == 4 || depth == 8 || depth == 16) || (ctype != 0 && ctype != 3 && depth < 8) ||
       (ctype == 3 && depth == 16))
        throw std::runtime_error("bad PNG bit depth: " + fn);
    const std::vector<unsigned char> raw = zlib_inflate(idat.data(), idat.size());
    const size_t bpp = std::max<size_t>(1, static_cast<size_t>(samples) * depth / 8);
    const size_t stride = (static_cast<size_t>(w) * samples * depth + 7) / 8;
    if(raw.size() < static_cast<size_t>(h) * (stride + 1))
        throw std::runtime_error("truncated PNG image data: " + fn);
    std::vector<unsigned char> img(static_cast<size_t>(h) * stride);
    for(uint32_t y = 0; y < h; ++y)
    {
        const unsigned char *src = &raw[static_cast<size_t>(y) * (stride + 1)];
        const int filter = src[0];
        unsigned char *row = &img[static_cast<size_t>(y) * stride];
        const unsigned char *prev = y ? row - stride : nullptr;
        for(size_t x = 0; x < stride; ++x)
        {
            const int a = x >= bpp ? row[x - bpp] : 0;
            const int b = prev ? prev[x] : 0;
            const int c = (prev && x >= bpp) ? prev[x - bpp] : 0;
            int v = src[1 + x];
            switch(filter)
            {
            case 0: break;
            case 1: v += a; break;
            case 2: v += b; break;
            case 3: v += (a + b) / 2; break;
            case 4: v += paeth(a, b, c); break;
            default: throw std::runtime_error("bad PNG filter: " + fn);
            }
            row[x] = static_cast<unsigned char>(v & 0xff);
        }
    }
    // expand to 8-bit samples (16-bit: high byte; low depths scaled to 0..255)
    auto sample = [&](uint32_t x, uint32_t y, int s) -> int {
        const unsigned char *row = &img[static_cast<size_t>(y) * stride];
        const size_t i = static_cast<size_t>(x) * samples + s;
        if(depth == 8)
            return row[i];
        if(depth == 16)
            return row[i * 2];
        const size_t bit = i * depth;
        const int v = (row[bit / 8] >> (8 - depth - static_cast<int>(bit % 8))) & ((1 << depth) - 1);
        return ctype == 3 ? v : v * 255 / ((1 << depth) - 1);
    };
    LoadedImage out;
    out.width = static_cast<int>(w);
    out.height = static_cast<int>(h);
    out.is_float = false;
    if(ctype == 3)
        out.channels = trns.empty() ? 3 : 4;
    else
        out.channels = samples;
    if(out.channels == 2)
        throw std::runtime_error("ImageDynamic::load: unsupported channels: 2");
    out.texels.resize(static_cast<size_t>(w) * h * 4);
    for(uint32_t y = 0; y < h; ++y)
        for(uint32_t x = 0; x < w; ++x)
        {
            float *t = &out.texels[(static_cast<size_t>(y) * w + x) * 4];
            int rgba[4] = { 0, 0, 0, 255 };
            if(ctype == 3)
            {
                const int idx = sample(x, y, 0);
                if(static_cast<size_t>(idx) * 3 + 2 >= palette.size())
                    throw std::runtime_error("PNG palette index out of range: " + fn);
                rgba[0] = palette[idx * 3];
                rgba[1] = palette[idx * 3 + 1];
                rgba[2] = palette[idx * 3 + 2];
                rgba[3] = static_cast<size_t>(idx) < trns.size() ? trns[idx] : 255;
            }
            else
            {
                for(int s = 0; s < samples; ++s)
                    rgba[s] = sample(x, y, s);
                if(samples == 1)
                    rgba[1] = rgba[2] = 0;  // a one-channel texture reads (v, 0, 0, 1)
            }
            for(int c = 0; c < 4; ++c)
                t[c] = static_cast<float>(rgba[c]) / 255.0f;
        }
    return out;
}

// ---------------------------------------------------------------- Radiance HDR

LoadedImage load_hdr(const std::string &fn)
{
    const std::vector<unsigned char> d = read_all(fn);
    size_t pos = 0;
    auto line = [&]() {
        std::string s;
        while(pos < d.size() && d[pos] != '\n')
            s.push_back(static_cast<char>(d[pos++]));
        if(pos < d.size())
            ++pos;
        return s;
    };
    const std::string magic = line();
    if(magic != "#?RADIANCE" && magic != "#?RGBE")
        throw std::runtime_error("not a Radiance HDR file: " + fn);
    for(;;)
    {
        if(pos >= d.size())
            throw std::runtime_error("truncated HDR header: " + fn);
        const std::string l = line();
        if(l.empty())
            break;
        if(l.rfind("FORMAT=", 0) == 0 && l != "FORMAT=32-bit_rle_rgbe")
            throw UnsupportedFormat("unsupported HDR format: " + l);
    }
    char ya[3] = {}, xa[3] = {};
    int h = 0, w = 0;
    const std::string res = line();
    if(std::sscanf(res.c_str(), "%2s %d %2s %d", ya, &h, xa, &w) != 4 || std::string(ya) != "-Y" ||
       std::string(xa) != "+X" || w <= 0 || h <= 0 || w > (1 << 16) || h > (1 << 16))
        throw UnsupportedFormat("unsupported HDR orientation or size: " + res);
    LoadedImage out;
    out.width = w;
    out.height = h;
    out.channels = 3;
    out.is_float = true;
    out.texels.resize(static_cast<size_t>(w) * h * 4);
    std::vector<unsigned char> scan(static_cast<size_t>(w) * 4);
    for(int y = 0; y < h; ++y)
    {
        if(pos + 4 <= d.size() && w >= 8 && w < 32768 && d[pos] == 2 && d[pos + 1] == 2 && !(d[pos + 2] & 0x80) &&
           ((d[pos + 2] << 8) | d[pos + 3]) == w)
        {
            // adaptive run-length encoding, one component plane at a time
            pos += 4;
            for(int c = 0; c < 4; ++c)
            {
                int x = 0;
                while(x < w)
                {
                    if(pos >= d.size())
                        throw std::runtime_error("truncated HDR data: " + fn);
                    int count = d[pos++];
                    if(count > 128)
                    {
                        count -= 128;
                        if(pos >= d.size() || x + count > w)
                            throw std::runtime_error("bad HDR run: " + fn);
                        const unsigned char v = d[pos++];
                        for(int k = 0; k < count; ++k)
                            scan[static_cast<size_t>(x++) * 4 + c] = v;
                    }
                    else
                    {
                        if(count == 0 || pos + count > d.size() || x + count > w)
                            throw std::runtime_error("bad HDR dump: " + fn);
                        for(int k = 0; k < count; ++k)
                            scan[static_cast<size_t>(x++) * 4 + c] = d[pos++];
                    }
                }
            }
        }
        else
        {
            if(pos + scan.size() > d.size())
                throw std::runtime_error("truncated HDR data: " + fn);
            std::memcpy(scan.data(), &d[pos], scan.size());
            pos += scan.size();
        }
        for(int x = 0; x < w; ++x)
        {
            const unsigned char *e = &scan[static_cast<size_t>(x) * 4];
            float *t = &out.texels[(static_cast<size_t>(y) * w + x) * 4];
            if(e[3] == 0)
                t[0] = t[1] = t[2] = 0.0f;
            else
            {
                const float f = std::ldexp(1.0f, static_cast<int>(e[3]) - (128 + 8));
                t[0] = e[0] * f;
                t[1] = e[1] * f;
                t[2] = e[2] * f;
            }
            t[3] = 1.0f;
        }
    }
    return out;
}

} // namespace

LoadedImage load_image(const std::string &filename)
{
    const std::string ext = upper_ext(filename);
    if(ext == ".PNG")
        return load_png(filename);
    if(ext == ".HDR")
        return load_hdr(filename);
    if(ext == ".JPG" || ext == ".JPEG")
        throw UnsupportedFormat("JPEG textures are not supported: " + filename);
    if(ext == ".EXR")
        throw UnsupportedFormat("ImageDynamic::load: EXR is not supported");
    throw std::invalid_argument("unknown image format: " + ext);
}

} // namespace bt

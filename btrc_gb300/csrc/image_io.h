// Image file output of the `save` post-processor (PNG / EXR / HDR by extension).
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

namespace bt {

struct UnsupportedFormat : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

// pixels: width * height * channels floats (3 or 4), top row first. Values are raised to
// 1 / gamma before encoding. Throws std::invalid_argument on a bad size or unknown
// extension, UnsupportedFormat for JPEG, std::runtime_error on I/O failure.
void save_image(const std::string &filename, const float *pixels, int width, int height, int channels, float gamma);

// An image as a 2D texture reads it: RGBA floats, top row first. 8-bit files hold v / 255
// (sRGB decoding is the texture's business); a one-channel file reads (v, 0, 0, 1) and a
// three-channel one (r, g, b, 1).
struct LoadedImage
{
    int width = 0, height = 0;
    int channels = 0;       // channels in the file after palette expansion: 1, 3 or 4
    bool is_float = false;  // HDR: float texels; PNG: 8-bit normalised
    std::vector<float> texels;
};

// Load a .png or .hdr file (common/btrc/utils/image.cpp:296-346). Throws
// UnsupportedFormat for JPEG, EXR and interlaced PNG, std::invalid_argument for an unknown
// extension, std::runtime_error for unreadable or malformed files.
LoadedImage load_image(const std::string &filename);

} // namespace bt

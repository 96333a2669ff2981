// Image file output of the `save` post-processor (PNG / EXR / HDR by extension).
#pragma once

#include <stdexcept>
#include <string>

namespace bt {

struct UnsupportedFormat : std::runtime_error
{
    using std::runtime_error::runtime_error;
};

// pixels: width * height * channels floats (3 or 4), top row first. Values are raised to
// 1 / gamma before encoding. Throws std::invalid_argument on a bad size or unknown
// extension, UnsupportedFormat for JPEG, std::runtime_error on I/O failure.
void save_image(const std::string &filename, const float *pixels, int width, int height, int channels, float gamma);

} // namespace bt

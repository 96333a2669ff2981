// Host side of 2D textures: compiling Texture2D JSON nodes into texture programs over an
// image table, and the environment-light importance table of the ibl light.
#pragma once

#include <map>
#include <string>
#include <vector>

#include "json.h"
#include "layout.h"

namespace bt {

struct TexStore
{
    std::string scene_dir;
    std::vector<TexImage> images;
    std::vector<float> texels;          // 4 floats per texel
    std::vector<TexInstr> instr;
    std::map<std::string, int> image_cache;  // file + sampling description -> image
};

// A Texture2D node (core/btrc/core/texture2d.h; builtin/btrc/builtin/texture2d/*): a value
// or {"type": "constant"} gives a constant (returns -1, value in `constant`); "array",
// "add", "sub", "mul", "div" and "transform" compile to a program (returns its first
// instruction). Throws std::runtime_error on unsupported or malformed nodes.
int compile_texture2d(TexStore &T, const json::NodeP &n, V3 &constant);

// EnvirLightSampler::preprocess (builtin/btrc/builtin/light/env_sampler.cpp:83-135): tile
// luminance from 256 Hammersley samples over a 1.2x enlarged tile, weights
// max(0, area * (lum - mean lum)), normalised when their sum exceeds 1e-3.
void build_env_sampler(const TexStore &T, int prog, int lut_w, int lut_h, std::vector<float> &probs,
                       std::vector<AliasEntry8> &alias);

} // namespace bt

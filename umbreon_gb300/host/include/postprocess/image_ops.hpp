// Image helpers of the umbreon API: supersample resolve, assumed gamma and
// sRGB encoding of a FrameResult (host-side; the frame pipeline runs the
// resolve and gamma on the GPU).
#pragma once

#include <cstdint>
#include <vector>

#include "render/render_types.hpp"

namespace umbreon {

std::vector<float> boxDownsample(const std::vector<float>& src, int w, int h, int channels, int ss);
void applyAssumedGamma(FrameResult& frame, float g);
std::vector<std::uint8_t> srgbEncode8(const FrameResult& frame, int channels);
float srgbEncodeF(float v);
float srgbDecodeF(float s);

}  // namespace umbreon

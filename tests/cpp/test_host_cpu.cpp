// Host-side parts of the umbreon API that need no GPU: the image helpers
// (the reference's tests/test_image_ops.cpp expectations), RenderProgress and
// the log sink.
#include <limits>
#include <string>
#include <vector>

#include "check.hpp"
#include "log.hpp"
#include "postprocess/image_ops.hpp"
#include "umbreon.hpp"

int main() {
  Checks c;
  {
    std::vector<float> src(16);
    for (int i = 0; i < 16; ++i) src[i] = float(i);
    const std::vector<float> out = umbreon::boxDownsample(src, 4, 4, 1, 2);
    c("downsample size 4", out.size() == 4);
    c("downsample block means", near(out[0], 2.5f, 1e-6f) && near(out[1], 4.5f, 1e-6f) &&
                                    near(out[2], 10.5f, 1e-6f) && near(out[3], 12.5f, 1e-6f));
    const float nan = std::numeric_limits<float>::quiet_NaN(), inf = std::numeric_limits<float>::infinity();
    const std::vector<float> g = umbreon::boxDownsample({nan, 2.0f, 4.0f, inf}, 2, 2, 1, 2);
    c("downsample non-finite guard = 1.5", near(g[0], 1.5f, 1e-6f));
  }
  {
    umbreon::FrameResult f;
    f.width = f.height = 1;
    f.color = {0.5f, 0.4f, 0.2f, 0.7f};
    umbreon::applyAssumedGamma(f, 1.0f);
    c("gamma 1 no-op", near(f.color[0], 0.5f, 1e-6f));
    umbreon::applyAssumedGamma(f, 2.0f);
    c("gamma 2 squares rgb, keeps alpha", near(f.color[0], 0.25f, 1e-6f) && near(f.color[1], 0.16f, 1e-6f) &&
                                              near(f.color[3], 0.7f, 1e-6f));
    umbreon::FrameResult g;
    g.width = g.height = 1;
    g.color = {-0.5f, 0, 0, 1};
    umbreon::applyAssumedGamma(g, 2.0f);
    c("gamma clamps negative to 0", g.color[0] == 0.0f);
  }
  {
    umbreon::FrameResult f;
    f.width = f.height = 1;
    f.color = {0.0f, 0.5f, 1.0f, 0.5f};
    const auto px = umbreon::srgbEncode8(f, 4);
    c("srgb 0 / 0.5 / 1 -> 0 / 188 / 255", px[0] == 0 && px[1] == 188 && px[2] == 255);
    c("srgb alpha linear 0.5 -> 128", px[3] == 128);
    c("srgb decode(encode(x)) == x", near(umbreon::srgbDecodeF(umbreon::srgbEncodeF(0.3f)), 0.3f, 1e-5f));
  }
  {
    umbreon::RenderProgress p;
    c("progress idle at 0", p.fraction() == 0.0f);
    p.beginPhase(umbreon::RenderPhase::Primary, 10);
    const float a = p.fraction();
    p.advance(5);
    const float b = p.fraction();
    p.markDone();
    c("progress monotone and done at 1", a < b && b < 1.0f && p.fraction() == 1.0f);
    p.requestCancel();
    c("cancel flag", p.cancelRequested());
    c("phase names", std::string(umbreon::toString(umbreon::RenderPhase::Primary)) == "Primary");
  }
  {
    std::string got;
    umbreon::setLogSink([&](umbreon::LogLevel, const char* t) { got = t; });
    umbreon::logMessage(umbreon::LogLevel::Info, "value %d", 42);
    umbreon::setLogSink(nullptr);
    c("log sink receives formatted text", got == "value 42");
  }
  return c.report("host_cpu");
}

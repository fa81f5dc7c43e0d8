// FrameResult of the umbreon API (same fields as the reference).  This
// library fills color (final size), depth and viewZ (supersampled grid, as
// the reference leaves them), renderSeconds, pt1Timing.bvhBuild/primary,
// effectiveTriangles and cancelled.
#pragma once

#include <cstddef>
#include <cstdint>
#include <vector>

namespace umbreon {

struct Pt1Timing {
  double bvhBuild = 0.0;
  double primary = 0.0;
  double direct = 0.0;
  double gather = 0.0;
  double denoise = 0.0;
  double upsample = 0.0;
  double total = 0.0;
};

struct Pt1RayCounts {
  std::uint64_t gatherRays = 0;
  std::uint64_t gatherHits = 0;
  std::uint64_t neeRays = 0;
  std::uint64_t neeOccluded = 0;
  std::uint64_t gbufferRays = 0;
};

struct FrameResult {
  int width = 0;
  int height = 0;
  std::vector<float> color;
  std::vector<float> albedo;
  std::vector<float> normal;
  std::vector<float> depth;
  std::vector<float> viewZ;
  std::vector<std::uint32_t> objectId;
  std::vector<std::uint32_t> materialId;
  std::vector<float> surfAlpha;
  std::vector<std::uint8_t> clipCut;
  std::vector<float> clipNearVz;
  std::vector<float> clipFarVz;
  std::vector<float> contactAo;
  std::vector<float> shapeAo;
  std::vector<float> bentNormal;
  std::vector<float> avgHitDist;
  std::vector<float> position;
  std::vector<float> indirect;
  std::vector<float> giRecordViz;
  std::vector<float> giOcclusion;
  std::vector<float> aaMask;
  std::vector<float> aoPatchMask;
  double renderSeconds = 0.0;
  double aoCoarseSeconds = 0.0;
  std::size_t effectiveTriangles = 0;
  bool cancelled = false;
  Pt1Timing pt1Timing;
  Pt1RayCounts pt1Rays;
  int denoiserUsed = 0;
  int pt1DenoiserUsed = 0;
};

}  // namespace umbreon

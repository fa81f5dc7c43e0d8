// RenderOptions of the umbreon API (same fields and defaults as the
// reference).  This library honours the ray-cast + shade fields: output size,
// supersample, adaptive AA, AO (legacy and enhanced estimators, AOVs,
// coarse grid), shadows, environment dome, specular scale, transparency and
// the a-trous denoiser (OIDN requests run it, as the reference does without
// OIDN).  GI and the edge passes are not part of it (see umbreon.hpp for how
// render() treats them).
#pragma once

#include "render/edge_types.hpp"

namespace umbreon {

struct RenderOptions {
  int width = 1024;
  int height = 768;
  int supersample = 1;

  int aaMode = 0;
  float aaThreshold = 0.1f;
  int aaDepth = 0;
  bool aaDebug = false;

  int aoSamples = 0;
  float aoDistance = 1.0e20f;
  float aoIntensity = 1.0f;
  float aoFalloffPower = 0.0f;
  bool aoMultiScale = false;
  bool aoBentNormal = false;
  float aoSkyColor[3] = {1.0f, 1.0f, 1.0f};
  float aoGroundColor[3] = {1.0f, 1.0f, 1.0f};
  bool aoUseCameraUp = true;
  float aoUp[3] = {0.0f, 1.0f, 0.0f};
  bool aoMultibounce = false;
  bool aoLowDiscrepancy = false;
  float aoDiffuseFactor = 0.0f;
  bool aoWriteAov = false;
  int aoResDiv = 0;
  bool aoResDebug = false;
  bool aoEnhanced() const {
    return aoFalloffPower > 0.0f || aoMultiScale || aoBentNormal || aoMultibounce || aoLowDiscrepancy ||
           aoDiffuseFactor > 0.0f;
  }

  bool gi = false;
  int giSamples = 64;
  int giBounces = 1;
  float giMaxDistance = 0.0f;
  float giIntensity = 1.0f;
  float giEnvIntensity = 1.0f;
  float giAccuracy = 0.15f;
  float giRecordSpacing = 0.0f;
  bool giGradients = false;
  bool giOutlierReject = true;
  bool giAdaptive = false;
  float giNormalReject = 0.85f;
  bool giComponentReject = true;
  bool giSeedPerVertex = false;
  int giIntegrator = 2;
  int pt1Spp = 8;
  bool pt1HalfRes = true;
  bool pt1Denoise = true;
  unsigned pt1Seed = 0;
  int pt1SkyMode = 0;
  float pt1SkyRadiance[3] = {1.0f, 1.0f, 1.0f};
  float pt1UpsampleNormalPow = 32.0f;
  float pt1UpsampleDepthScale = 0.02f;
  bool pt1Ld = true;
  float pt1Clamp = 0.0f;
  int pt1GatherDiv = -1;
  bool pt1EdgePatch = true;
  int pt1EdgePatchSppMul = 4;
  float pt1EdgePatchThresh = 0.3f;
  bool pt1Stats = false;
  int pt2Pattern = 1;
  bool pt2Emissive = true;
  int pt2Rounds = 0;
  float pt2Radius = 16.0f;
  bool pt2Unbiased = false;
  float pt2MCap = 100.0f;
  float pt2WClamp = 0.0f;
  bool pt2Adaptive = false;
  float pt2AdaptiveThresh = 0.15f;
  int pt2AdaptiveMul = 4;
  bool pt2EmissiveNee = true;
  bool pt2Reflect = true;
  bool pt2Glossy = true;
  int pt2GlossySpp = 8;
  bool pt2GlossyDenoise = true;

  int denoiser = 0;
  int denoiseIters = 5;
  float denoiseSigmaZ = 1.0f;
  float denoiseSigmaN = 128.0f;
  float denoiseSigmaL = 4.0f;
  bool denoiseDemodulateAlbedo = true;
  bool oidnCleanAux = true;
  int oidnMaxMemoryMB = 1024;

  bool shadows = false;
  int shadowSamples = 1;
  float lightRadius = 0.0f;

  int envLights = 0;
  float envIntensity = 1.0f;
  float envKeyScale = 0.0f;
  float envAngle = 90.0f;

  float specularScale = 1.0f;

  bool transparency = true;
  bool transparentBackground = false;
  int maxTransparentLayers = 256;

  StrokeEdgeOptions strokeEdges;
  ObjectSpaceEdgeOptions objectSpaceEdges;
};

}  // namespace umbreon

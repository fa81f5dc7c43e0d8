// gi.cuh -- the path-traced GI pass (pt1 and its pt2 extensions): the types
// the frame's host code fills and the launchers of gi.cu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "ubr_internal.h"

namespace ubr {

// Emissive primitives sampled as lights at gather origins (pt2 emissive NEE,
// integrator/pt2/pt2_emissive.hpp): mesh triangles first, then real spheres
// and the lateral surfaces / disk caps of real capped cylinders, with a
// power-weighted CDF over all records.  Record r is kEmitF4 float4s:
//   triangle: (p0, area) (p1, 0) (p2, 0) (e0, 0) (e1, 0) (e2, 0) (unit ng, 0)
//   CSG:      (p0, area) (unit axis, kind) (Le, radius) (len, 0, 0, 0)
// with kind 1 sphere, 2 cylinder side, 3 cylinder cap (a float holding the
// integer).  Index tables map a hit's primID to its record (0xFFFFFFFF: not
// an emitter): triangles by mesh primID (base triangles), spheres by sphere
// primID, capped cylinders by primID to (side, cap0, cap1).
constexpr int kEmitF4 = 7;
struct EmitD {
  uint32_t n = 0, triCount = 0;
  uint32_t nTriIndex = 0, nSphereIndex = 0, nCylIndex = 0;
  const float* cdf = nullptr;
  const float* pdfChoose = nullptr;
  const float4* rec = nullptr;
  const uint32_t* triIndex = nullptr;
  const uint32_t* sphereIndex = nullptr;
  const uint4* cylIndex = nullptr;
};

// The gather's constants (embree_renderer.cpp:581-660) and its counters.
struct GiP {
  int spp, bounces, ld;
  float maxDist, clampLum;
  uint32_t seedMix;   // hashU32(pt1Seed)
  float envI;         // giEnvIntensity
  f3 amb, sky, ground, envUp;
  // [0] gather rays (all bounces), [1] NEE shadow rays, [2] G-buffer rays
  unsigned long long* stats;
  unsigned long long* overflow;  // the frame's traversal-overflow counter
  // pt2 extensions (Pt2GatherCfg, embree_renderer.cpp:620-660)
  int pt2;             // 1: Sobol first bounce, area-light NEE jitter, emission
  int pattern;         // 0 Owen-scrambled Sobol per point, 1 blue noise
  uint32_t sppPow2;    // blue-noise section length (power of two >= the sample budget)
  int sampleOffset;    // first sample index (adaptive refinement continues the sequence)
  int emissive;        // emission at gather vertices
  float* halfE;        // per grid point: sum of the first spp/2 samples (adaptive), or null
  EmitD em;            // emissive NEE (em.n == 0: none)
  // ReSTIR candidate reservoirs (pt2Rounds > 0), kRsvF4 float4s per grid
  // point, or null; a gather that fills them runs one thread per point
  float4* rsv;
};

// A ReSTIR reservoir (Pt2Reservoir, integrator/pt2/pt2_reservoir.hpp:36-42)
// as three float4s: (sample position, M) (sample normal, W) (radiance, 0).
constexpr int kRsvF4 = 3;

// The spatial rounds' settings (Pt2SpatialParams, pt2_spatial.hpp:51-59).
struct GiSpatial {
  int rounds;
  float radius, mCap, wClamp;
  int unbiased;
  uint32_t seedMix;
};

// A grid the gather runs on, per pixel: the first hit's position and ray
// distance (pd), its shading normal with the gather eligibility in w (ne),
// and its geometric normal (ng; null: the shading normal stands in, as the
// render grid carries none).
struct GiGrid {
  int W, H;
  const float4* pd;
  const float4* ne;
  const float4* ng;
};

// First-hit traced-reflection record per render-grid pixel (pt2):
// (Material::reflection or 1 for principled, GGX alpha (0 = mirror),
// anisotropy aspect, 0), Fresnel F0 (1,1,1 for POV), the rotation-baked
// tangent of an anisotropic lobe (zero: isotropic).
struct ReflD {
  float4* amt;  // x reflectivity, y alpha, z aspect
  float4* f0;
  float4* tan;
};

// The camera as the primary loop built it (perspective rays from camPos).
struct GiCam {
  f3 pos, dir;
  int ortho;
};

// --- launchers (gi.cu); km is the kind mask of the scene's variant ---
void giGBuffer(int km, cudaStream_t s, const Params& p, const DScene& sc, int w, int h, float4* pd, float4* ne,
               float4* ng, unsigned long long* stats, unsigned long long* overflow);
void giGather(int km, cudaStream_t s, const GiP& g, const DScene& sc, const LightD* lights, int nLights,
              const GiGrid& grid, const uint32_t* list, const uint32_t* listCount, uint32_t n, int spp, float4* E);
void giDenoiseInit(cudaStream_t s, uint32_t n, float4* E, const float4* ne, uint8_t* valid, float4* irr);
void giDenoiseAux(cudaStream_t s, int W, int H, const uint8_t* valid, const float4* irr, const float4* pd,
                  float* var, float* pgrad);
void giDenoiseIter(cudaStream_t s, int W, int H, int step, const uint8_t* valid, const float4* ne,
                   const float4* pd, const float4* irr, const float* var, const float* pgrad, float sigmaN,
                   float sigmaZ, float sigmaL, float4* next);
void giDenoiseWrite(cudaStream_t s, uint32_t n, const uint8_t* valid, const float4* irr, float4* E);
// joint-bilateral upsample of E to the render grid; the pixels that need the
// edge patch are flagged and listed in pixel order (count on the device)
size_t giPatchListBytes(uint32_t n);
cudaError_t giUpsample(cudaStream_t s, int W, int H, const float4* fpd, const float4* fne, const GiGrid& lo,
                       const float4* Elo, float normalPow, float depthScale, int fallbackR, int patchOn,
                       float patchThresh, float4* E, uint8_t* patchFlag, void* listTemp, size_t listTempBytes,
                       uint32_t* patchList, uint32_t* patchCount, unsigned long long* holes);
void giSmooth(cudaStream_t s, int W, int H, const uint32_t* list, const uint32_t* count, uint32_t n,
              const float4* fpd, const float4* fne, float normalPow, float depthScale, int radius,
              const float4* Esrc, float4* E);
void giComposite(cudaStream_t s, uint32_t n, const float4* ne, const float4* refl, const float4* E, float gI,
                 float4* color);
// pt2 adaptive spp: refinement mask of the eligible points, 3x3 dilation,
// and the merge of the refinement means into the base
void giAdaptiveMask(cudaStream_t s, int W, int H, const float4* E, const float* halfE, const float4* ne, int spp,
                    float threshold, uint8_t* mask);
void giDilate(cudaStream_t s, int W, int H, const uint8_t* in, const float4* ne, uint8_t* out);
void giMaskList(cudaStream_t s, uint32_t n, const uint8_t* mask, uint32_t* list, uint32_t* count);
void giMerge(cudaStream_t s, const uint32_t* list, const uint32_t* count, uint32_t n, int spp, int extra,
             const float4* Er, float4* E);
// pt2 ReSTIR spatial round `round` over a grid's reservoirs (in -> out); the
// last round (E non-null) writes E.xyz of the eligible points
void giSpatialRound(int km, cudaStream_t s, const GiSpatial& sp, const DScene& sc, const GiGrid& grid,
                    const float4* in, float4* out, int round, float4* E, unsigned long long* overflow);
// pt2 traced mirror reflection and the glossy GGX gather at the render grid
void giReflect(int km, cudaStream_t s, const GiP& g, const DScene& sc, const LightD* lights, int nLights,
               const GiGrid& full, const ReflD& r, const GiCam& cam, uint32_t n, float4* color);
void giGlossy(int km, cudaStream_t s, const GiP& g, const DScene& sc, const LightD* lights, int nLights,
              const GiGrid& full, const ReflD& r, const GiCam& cam, uint32_t n, int spp, uint32_t frameSeed,
              float4* Espec);
// glossy E_spec to the output grid over glossy samples (mean of them, guides
// averaged, normal renormalised) and the composite color += reflection * E
void giGlossyDown(cudaStream_t s, int W, int H, int ss, const ReflD& r, const float4* Espec, const float4* fpd,
                  const float4* fne, float4* Eo, float4* pdo, float4* neo);
void giGlossyComposite(cudaStream_t s, uint32_t n, const ReflD& r, const float4* Espec, float4* color);
// a guide grid whose eligibility is "glossy pixel": ne.w = 1 where the
// pixel's reflection record is glossy (copy of fne otherwise zero)
void giGlossyElig(cudaStream_t s, uint32_t n, const ReflD& r, const float4* fne, float4* out);

}  // namespace ubr

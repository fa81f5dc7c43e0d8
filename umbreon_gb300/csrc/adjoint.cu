// adjoint.cu -- ubr_adjoint: reverse-mode derivative of a single-layer sphere
// frame (the forward path of render.cu restricted to one opaque layer of
// spheres, POV shading, hard shadows, legacy or enhanced AO, fog, box
// downsample and gamma) with respect to the scene and render parameters.
//
// Nothing from a forward render is stored or reused.  The adjoint re-traces:
//   k_adj_primary   closest hit of every hi-res primary ray (the hit record
//                   and the 3x3 interior test read it)
//   k_adj_shade     (only when the assumed gamma is not 1) the forward
//                   colour of every hi-res sample, re-tracing its shadow and
//                   AO rays, then k_adj_down averages it per output pixel:
//                   the gamma derivative needs the downsampled value
//   k_adj_shade     per hi-res sample: re-trace the shadow rays (any hit) and
//                   the AO rays (nearest hit and its sphere), recompute the
//                   shaded colour and push dL/d(colour) back through gamma,
//                   downsample, fog, shadeLocal (shading.hpp:76-192), the AO
//                   estimators (ambient_occlusion.hpp:33-57, 171-267) and the
//                   sphere hit (t, P, N, self-intersection epsilon)
// Visibility (which sphere a ray hits, each shadow bit, each AO sample's
// grazing test and occluder, the frame-from-normal branch) is a constant of
// the derivative; per-sphere gradients are scattered with float atomics,
// global ones reduced per warp and block and added in double.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "trace.cuh"

namespace ubr {
namespace {

constexpr int kAdjLights = UBR_ADJOINT_MAX_LIGHTS;

// global gradient slots
enum : int {
  gAmbient = 0,
  gDiffuse,
  gSpecular,
  gRoughness,
  gBrilliance,
  gPhong,
  gPhongSize,
  gReflection,
  gEmission,
  gAmbColor = 9,      // 3
  gBg = 12,           // 3
  gFogStart = 15,
  gFogEnd = 16,
  gFogColor = 17,     // 3
  gAoDistance = 20,
  gAoIntensity = 21,
  gSpecScale = 22,
  gLightL = 23,       // 3 per light: d/d (unit) light vector
  gLightC = 23 + 3 * kAdjLights,  // 3 per light: d/d light colour x intensity
  kGlobals = 23 + 6 * kAdjLights
};

struct AdjBufs {
  const float2* hit;        // per hi-res sample: t, ref bits
  const float4* dOut;       // dL/d(output colour), outW x outH
  const float4* outFwd;     // forward output colour (gamma derivative), or null
  float4* colorHi;          // forward mode: fogged hi-res colour
  const LightD* lights;
  float* gColor;            // per input sphere x 3
  float* gCenter;           // per input sphere x 3
  float* gRadius;           // per input sphere
  double* gGlobal;          // kGlobals
  unsigned long long* stats;  // 0 samples, 1 rays, 2 overflow
  uint32_t flags;
};

UBR_D void atomicAdd3(float* a, uint32_t k, f3 v) {
  if (!a) return;
  atomicAdd(a + 3 * k, v.x);
  atomicAdd(a + 3 * k + 1, v.y);
  atomicAdd(a + 3 * k + 2, v.z);
}

UBR_D f3 mul3(f3 a, f3 b) { return f3{a.x * b.x, a.y * b.y, a.z * b.z}; }

// d(a / |a|) transposed applied to g: (g - n (n.g)) / |a| with n = a / |a|
UBR_D f3 normalizeBack(f3 n, float len, f3 g) {
  const float ng = dot(n, g);
  const float inv = 1.0f / len;
  return f3{(g.x - n.x * ng) * inv, (g.y - n.y * ng) * inv, (g.z - n.z * ng) * inv};
}

__global__ void __launch_bounds__(128) k_adj_primary(Params p, TravScene ts, float2* hit, uint32_t npix,
                                                     unsigned long long* stats) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t ovf = 0, traced = 0;
  if (i < npix) {
    const int px = int(i % uint32_t(p.W)), py = int(i / uint32_t(p.W));
    f3 org, rd;
    primaryRay(p, px, py, org, rd);
    float tn, tf;
    clipRange(p, rd, tn, tf);
    Hit h;
    h.t = 0.0f;
    const bool any = traverse<false, kMaskSphere, false>(ts, Ray{org, rd, tn, tf}, h, ovf, nullptr, false);
    hit[i] = make_float2(any ? h.t : 0.0f, __uint_as_float(any ? h.ref : kInvalid));
    traced = 1;
  }
  warpCount(&stats[1], traced);
  warpCount(&stats[2], ovf);
}

// Fog factor of view-z z (fog.cpp:17-36) and its partial derivatives (zero
// where the factor is clamped or the fog is a step).
struct FogD {
  float f, dz, dStart, dEnd;
  bool on;
};
UBR_D FogD fogAt(const Params& p, float z) {
  FogD r{1.0f, 0.0f, 0.0f, 0.0f, false};
  if (!p.fogOn || !(z > 0.0f)) return r;
  r.on = true;
  const float denom = p.fogEnd - p.fogStart;
  if (denom <= 0.0f) {
    r.f = z < p.fogEnd ? 1.0f : 0.0f;
    return r;
  }
  const float f = (p.fogEnd - z) / denom;
  if (f < 0.0f) {
    r.f = 0.0f;
  } else if (f > 1.0f) {
    r.f = 1.0f;
  } else {
    r.f = f;
    r.dz = -1.0f / denom;
    r.dStart = (p.fogEnd - z) / (denom * denom);
    r.dEnd = (z - p.fogStart) / (denom * denom);
  }
  return r;
}

// One hi-res sample.  GRAD = false: forward colour after fog into colorHi.
// GRAD = true: the sample's share of every gradient.
template <bool GRAD>
__global__ void __launch_bounds__(128) k_adj_shade(Params p, DScene s, AdjBufs b, uint32_t npix) {
  __shared__ float sAcc[kGlobals];
  for (int k = threadIdx.x; k < kGlobals; k += blockDim.x) sAcc[k] = 0.0f;
  if (GRAD) __syncthreads();
  float G[kGlobals];
#pragma unroll
  for (int k = 0; k < kGlobals; ++k) G[k] = 0.0f;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t used = 0, traced = 0, ovf = 0;
  const TravScene ts = travOf(s);
  if (i < npix) {
    const int px = int(i % uint32_t(p.W)), py = int(i / uint32_t(p.W));
    const float2 hr = b.hit[i];
    const uint32_t ref = __float_as_uint(hr.y);
    // dL/d(this sample's fogged colour)
    float4 g = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    bool active = !GRAD;
    if (GRAD) {
      const int ox = px / p.ss, oy = py / p.ss;
      const uint32_t o = uint32_t(oy) * uint32_t(p.outW) + uint32_t(ox);
      g = b.dOut[o];
      if (!(fabsf(p.gamma - 1.0f) <= 1.0e-4f)) {
        // applyAssumedGamma: v > 0 ? v^gamma : 0 (image_ops.cpp:37-46)
        const float4 v = b.outFwd[o];
        g.x = v.x > 0.0f ? g.x * p.gamma * powf(v.x, p.gamma - 1.0f) : 0.0f;
        g.y = v.y > 0.0f ? g.y * p.gamma * powf(v.y, p.gamma - 1.0f) : 0.0f;
        g.z = v.z > 0.0f ? g.z * p.gamma * powf(v.z, p.gamma - 1.0f) : 0.0f;
      }
      if (p.ss > 1) {
        const float inv = 1.0f / float(p.ss * p.ss);
        g = make_float4(g.x * inv, g.y * inv, g.z * inv, g.w * inv);
      }
      active = g.x != 0.0f || g.y != 0.0f || g.z != 0.0f || g.w != 0.0f;
      if (active && (b.flags & UBR_ADJOINT_INTERIOR_ONLY)) {
        for (int dy = -1; dy <= 1 && active; ++dy)
          for (int dx = -1; dx <= 1; ++dx) {
            const int qx = px + dx, qy = py + dy;
            if (qx < 0 || qy < 0 || qx >= p.W || qy >= p.H) continue;
            if (__float_as_uint(b.hit[uint32_t(qy) * uint32_t(p.W) + uint32_t(qx)].y) != ref) {
              active = false;
              break;
            }
          }
      }
    }
    if (active && ref == kInvalid) {
      // background: colour = bg * coverage, alpha = coverage, no fog (view-z 0)
      const float cov = p.transparentBg ? 0.0f : 1.0f;
      if (GRAD) {
        G[gBg] += g.x * cov;
        G[gBg + 1] += g.y * cov;
        G[gBg + 2] += g.z * cov;
        used = 1;
      } else {
        b.colorHi[i] = make_float4(p.bg.x * cov, p.bg.y * cov, p.bg.z * cov, cov);
      }
    } else if (active) {
      const uint32_t prim = refPrim(ref);
      const uint32_t sk = s.baseSph ? prim % s.baseSph : prim;
      const float4 sc = __ldg(&s.sph[prim]);
      const f3 cc{sc.x, sc.y, sc.z};
      const float rad = sc.w;
      f3 org, rd;
      primaryRay(p, px, py, org, rd);
      const float t = hr.x;
      const f3 P{org.x + rd.x * t, org.y + rd.y * t, org.z + rd.z * t};
      const f3 Ng = rd * t - (cc - org);  // isectSphere's geometric normal
      const float ngLen = length(Ng);
      const f3 nHat = normalize(Ng);
      const float sgn = dot(nHat, rd) > 0.0f ? -1.0f : 1.0f;  // faceForward
      const f3 N = nHat * sgn;
      const f3 V = normalize(f3{-rd.x, -rd.y, -rd.z});
      const float eps = selfIntersectEps(P, rd, t);
      const float4 fc = __ldg(&s.primColor[kSphere][prim]);
      const f3 C{fc.x, fc.y, fc.z};
      const ubr_material m = s.mats[__ldg(&s.primMat[kSphere][prim])];
      const bool fromEdge = __ldg(&s.primFromEdge[kSphere][prim]) != 0;
      const bool aoOn = !fromEdge && p.aoSamples > 0;
      const bool shOn = !fromEdge && p.shadowsActive != 0;
      // secondary-ray origin (k_surface): P + safeNormalize(Ng toward N) * eps
      f3 ng = dot(Ng, N) < 0.0f ? neg(Ng) : Ng;
      ng = safeNormalize(ng, N);
      const f3 O = P + ng * eps;
      // fog of this sample
      const float z = t * dot(rd, p.camDir);
      const FogD fog = fogAt(p, z);
      const f3 gc = (fog.on && !p.transparentBg) ? f3{g.x * fog.f, g.y * fog.f, g.z * fog.f} : f3{g.x, g.y, g.z};
      const LightD* lights = b.lights;
      const int nL = p.nLights;
      // shadow bits (re-traced any hit) and N.L per light
      uint32_t lit = 0, shadowed = 0;
#pragma unroll
      for (int l = 0; l < kAdjLights; ++l) {
        if (l >= nL) break;
        const LightD L = lights[l];
        if (dot(N, L.L) > 0.0f) {
          lit |= 1u << l;
          if (shOn) {
            Hit h;
            if (traverse<false, kMaskSphere, true>(ts, Ray{O, L.L, eps, kInfF}, h, ovf, nullptr, true))
              shadowed |= 1u << l;
            ++traced;
          }
        }
      }
      const float ambTerm = dot(mul3(gc, C), p.ambLight);  // sum_c g_c C_c amb_c
      // dL/d(openness), which does not depend on the openness itself
      float gOpen = 0.0f;
      if (GRAD && aoOn) {
        gOpen = m.ambient * ambTerm * p.aoIntensity;
        if (p.aoDiffuseFactor > 0.0f) {
          float sdiff = 0.0f;
#pragma unroll
          for (int l = 0; l < kAdjLights; ++l) {
            if (l >= nL) break;
            if (!(lit & (1u << l))) continue;
            const LightD L = lights[l];
            const float ndl = dot(N, L.L);
            float d;
            if (m.brilliance == 1.0f) d = ndl;
            else if (m.brilliance == 0.0f) d = 1.0f;
            else d = powf(ndl, m.brilliance);
            const float sf = (shadowed & (1u << l)) ? 0.0f : 1.0f;
            sdiff += m.diffuse * d * dot(mul3(gc, C), L.color) * sf;
          }
          gOpen += sdiff * p.aoDiffuseFactor;
        }
      }
      // --- AO: re-trace every sample; accumulate openness and, for the
      // enhanced estimator, push dL/d(obs) into the occluder, the origin,
      // the sample direction (through the frame of N) and the AO distance
      float openness = 1.0f;
      f3 gO{0.0f, 0.0f, 0.0f}, gN{0.0f, 0.0f, 0.0f};
      if (aoOn) {
        const Frame3 fr = frameFromNormal(N);
        const float R = p.aoDistance;
        float radius[3], weight[3], scaleOf[3];
        int K;
        if (p.aoMultiScale) {
          K = 3;
          scaleOf[0] = 0.08f; scaleOf[1] = 0.30f; scaleOf[2] = 1.00f;
          radius[0] = 0.08f * R; radius[1] = 0.30f * R; radius[2] = 1.00f * R;
          weight[0] = 0.55f; weight[1] = 0.35f; weight[2] = 0.10f;
        } else {
          K = 1;
          scaleOf[0] = scaleOf[1] = scaleOf[2] = 1.0f;
          radius[0] = radius[1] = radius[2] = R;
          weight[0] = 1.0f; weight[1] = weight[2] = 0.0f;
        }
        const float gObs = -gOpen / float(p.aoSamples);
        f3 blo, bhi;
        aoBox(O, R, blo, bhi);
        const int start = boxStartNode(ts, blo, bhi);
        float obsSum = 0.0f;
        f3 gT{0.0f, 0.0f, 0.0f}, gB{0.0f, 0.0f, 0.0f};
        float gR = 0.0f;
        for (int k = 0; k < p.aoSamples; ++k) {
          float u1, u2;
          aoUV(p, px, py, k, u1, u2);
          // cosineSampleHemisphere (secondary_rays.hpp:66-73) with its coefficients kept
          const float phi = 6.2831853072f * u1;
          const float rr = sqrtf(u2);
          const float cz = sqrtf(fmaxf(0.0f, 1.0f - u2));
          const float cx = cosf(phi) * rr;
          const float cy = sinf(phi) * rr;
          const f3 dir = fr.t * cx + fr.b * cy + fr.n * cz;
          if (dot(dir, N) < 0.01f) {
            obsSum += 1.0f;
            continue;
          }
          ++traced;
          if (!p.aoEnhanced) {
            Hit h;
            if (traverse<false, kMaskSphere, true>(ts, Ray{O, dir, eps, R}, h, ovf, nullptr, true, start))
              obsSum += 1.0f;
            continue;
          }
          Hit h;
          if (!traverse<false, kMaskSphere, false>(ts, Ray{O, dir, eps, R}, h, ovf, nullptr, false, start)) continue;
          const float th = h.t;
          float per = 0.0f, dPerDt = 0.0f, dPerDR = 0.0f;
          for (int q = 0; q < K; ++q) {
            if (th < radius[q]) {
              float fk = 1.0f;
              if (p.aoFalloffPower > 0.0f) {
                float a = 1.0f - th / radius[q];
                if (a < 0.0f) a = 0.0f;
                fk = powf(a, p.aoFalloffPower);
                if (GRAD && a > 0.0f) {
                  const float da = p.aoFalloffPower * powf(a, p.aoFalloffPower - 1.0f);
                  dPerDt += weight[q] * da * (-1.0f / radius[q]);
                  dPerDR += weight[q] * da * th / (radius[q] * radius[q]) * scaleOf[q];
                }
              }
              per += weight[q] * fk;
            }
          }
          obsSum += per;
          if (GRAD && gObs != 0.0f) {
            gR += gObs * dPerDR;
            const float gth = gObs * dPerDt;
            if (gth != 0.0f) {
              // th solves |O + th dir - c_j|^2 = r_j^2
              const uint32_t pj = refPrim(h.ref);
              const float4 sj = __ldg(&s.sph[pj]);
              const f3 Q = O + dir * th - f3{sj.x, sj.y, sj.z};
              const float den = dot(Q, dir);
              if (den != 0.0f) {
                const float w = gth / den;
                const uint32_t kj = s.baseSph ? pj % s.baseSph : pj;
                atomicAdd3(b.gCenter, kj, Q * w);
                if (b.gRadius) atomicAdd(b.gRadius + kj, w * sj.w);
                gO = gO - Q * w;
                const f3 gDir = Q * (-w * th);
                gT = gT + gDir * cx;
                gB = gB + gDir * cy;
                gN = gN + gDir * cz;
              }
            }
          }
        }
        openness = 1.0f - obsSum / float(p.aoSamples);
        if (GRAD) {
          G[gAoDistance] += gR;
          // frame of N (scene.hpp:69-76): t = seed / |seed|, b = N x t
          // b = N x t:  dN += t x gB,  dt += gB x N
          gN = gN + cross(fr.t, gB);
          gT = gT + cross(gB, N);
          const bool useSeed0 = fabsf(N.x) < fabsf(N.y);
          const f3 seed = useSeed0 ? f3{0.0f, N.z, -N.y} : f3{-N.z, 0.0f, N.x};
          const float sl2 = dot(seed, seed);
          if (!(sl2 < 1.0e-18f)) {
            const f3 gSeed = normalizeBack(fr.t, sqrtf(sl2), gT);
            if (useSeed0) {
              gN.z += gSeed.y;
              gN.y -= gSeed.z;
            } else {
              gN.z -= gSeed.x;
              gN.x += gSeed.z;
            }
          }
        }
      }
      // --- shadeLocal, POV branch, forward and backward ---
      float aoF = 1.0f, diffuseAo = 1.0f;
      if (aoOn) {
        aoF = 1.0f - p.aoIntensity * (1.0f - openness);
        if (p.aoDiffuseFactor > 0.0f) diffuseAo = 1.0f - p.aoDiffuseFactor * (1.0f - openness);
      }
      f3 out{m.emission * C.x + aoF * m.ambient * C.x * p.ambLight.x,
             m.emission * C.y + aoF * m.ambient * C.y * p.ambLight.y,
             m.emission * C.z + aoF * m.ambient * C.z * p.ambLight.z};
      f3 gC{gc.x * (m.emission + aoF * m.ambient * p.ambLight.x),
            gc.y * (m.emission + aoF * m.ambient * p.ambLight.y),
            gc.z * (m.emission + aoF * m.ambient * p.ambLight.z)};
      if (GRAD) {
        G[gEmission] += dot(gc, C);
        G[gAmbient] += aoF * ambTerm;
        G[gAmbColor] += gc.x * aoF * m.ambient * C.x;
        G[gAmbColor + 1] += gc.y * aoF * m.ambient * C.y;
        G[gAmbColor + 2] += gc.z * aoF * m.ambient * C.z;
        if (aoOn) G[gAoIntensity] += m.ambient * ambTerm * (openness - 1.0f);
      }
      const float ex = blinnExp(m.roughness);
      float gEx = 0.0f;
#pragma unroll
      for (int l = 0; l < kAdjLights; ++l) {
        if (l >= nL) break;
        if (!(lit & (1u << l))) continue;
        const LightD L = lights[l];
        const float ndl = dot(N, L.L);
        const float sf = (shOn && (shadowed & (1u << l))) ? 0.0f : 1.0f;
        const f3 Lc = L.color * sf;
        float d, dDdn, dDdb;
        if (m.brilliance == 1.0f) {
          d = ndl;
          dDdn = 1.0f;
        } else if (m.brilliance == 0.0f) {
          d = 1.0f;
          dDdn = 0.0f;
        } else {
          d = powf(ndl, m.brilliance);
          dDdn = m.brilliance * powf(ndl, m.brilliance - 1.0f);
        }
        dDdb = d * logf(ndl);
        const float dk = m.diffuse * d * diffuseAo;
        out.x += dk * C.x * Lc.x;
        out.y += dk * C.y * Lc.y;
        out.z += dk * C.z * Lc.z;
        f3 gLc = mul3(gc, C) * dk;
        gC = gC + mul3(gc, Lc) * dk;
        const float gDk = dot(mul3(gc, C), Lc);
        float gNdl = 0.0f;
        f3 gL{0.0f, 0.0f, 0.0f};
        if (GRAD) {
          G[gDiffuse] += gDk * d * diffuseAo;
          const float gD = gDk * m.diffuse * diffuseAo;
          gNdl += gD * dDdn;
          G[gBrilliance] += gD * dDdb;
        }
        if (L.highlight) {
          f3 hl;
          float fr = 0.0f, dFr = 0.0f;
          if (m.metallic) {
            float c = ndl;
            if (c > 1.0f) c = 1.0f;
            const float x = acosf(c) * 0.63661977f;
            fr = 0.014567225f / ((x - 1.12f) * (x - 1.12f)) - 0.011612903f;
            const float dx = c < 1.0f ? -0.63661977f / sqrtf(1.0f - c * c) : 0.0f;
            dFr = -2.0f * 0.014567225f / ((x - 1.12f) * (x - 1.12f) * (x - 1.12f)) * dx;
            if (fr < 0.0f) {
              fr = 0.0f;
              dFr = 0.0f;
            }
            if (fr > 1.0f) {
              fr = 1.0f;
              dFr = 0.0f;
            }
            hl = f3{Lc.x * (fr + (1.0f - fr) * C.x), Lc.y * (fr + (1.0f - fr) * C.y),
                    Lc.z * (fr + (1.0f - fr) * C.z)};
          } else {
            hl = Lc;
          }
          float s1 = 0.0f, s2 = 0.0f, nh = 0.0f, rv = 0.0f;
          f3 H{0.0f, 0.0f, 0.0f}, LV{0.0f, 0.0f, 0.0f};
          if (m.specular > 0.0f) {
            LV = f3{L.L.x + V.x, L.L.y + V.y, L.L.z + V.z};
            H = normalize(LV);
            nh = dot(N, H);
            if (nh > 0.0f) s1 = m.specular * powf(nh, ex);
          }
          f3 Rr{0.0f, 0.0f, 0.0f};
          if (m.phong > 0.0f) {
            Rr = 2.0f * ndl * N - L.L;
            rv = dot(Rr, V);
            if (rv > 0.0f && (m.phong_size < 60.0f || rv > 0.0008f)) s2 = m.phong * powf(rv, m.phong_size);
          }
          const float specW = s1 + s2;
          if (specW > 0.0f) {
            const float scl = specW * p.specularScale;
            out.x += scl * hl.x;
            out.y += scl * hl.y;
            out.z += scl * hl.z;
            if (GRAD) {
              const f3 gHl = gc * scl;
              const float gSpecW = p.specularScale * dot(gc, hl);
              G[gSpecScale] += specW * dot(gc, hl);
              if (m.metallic) {
                const f3 mix{fr + (1.0f - fr) * C.x, fr + (1.0f - fr) * C.y, fr + (1.0f - fr) * C.z};
                gLc = gLc + mul3(gHl, mix);
                gC = gC + mul3(gHl, Lc) * (1.0f - fr);
                const float gFr = gHl.x * Lc.x * (1.0f - C.x) + gHl.y * Lc.y * (1.0f - C.y) +
                                  gHl.z * Lc.z * (1.0f - C.z);
                gNdl += gFr * dFr;
              } else {
                gLc = gLc + gHl;
              }
              if (s1 > 0.0f) {
                G[gSpecular] += gSpecW * powf(nh, ex);
                const float gNh = gSpecW * m.specular * ex * powf(nh, ex - 1.0f);
                gEx += gSpecW * s1 * logf(nh);
                gN = gN + H * gNh;
                gL = gL + normalizeBack(H, length(LV), N * gNh);
              }
              if (s2 > 0.0f) {
                G[gPhong] += gSpecW * powf(rv, m.phong_size);
                const float gRv = gSpecW * m.phong * m.phong_size * powf(rv, m.phong_size - 1.0f);
                G[gPhongSize] += gSpecW * s2 * logf(rv);
                const f3 gR = V * gRv;
                gNdl += 2.0f * dot(gR, N);
                gN = gN + gR * (2.0f * ndl);
                gL = gL - gR;
              }
            }
          }
        }
        if (GRAD) {
          gN = gN + L.L * gNdl;
          gL = gL + N * gNdl;
          G[gLightL + 3 * l] += gL.x;
          G[gLightL + 3 * l + 1] += gL.y;
          G[gLightL + 3 * l + 2] += gL.z;
          G[gLightC + 3 * l] += gLc.x * sf;
          G[gLightC + 3 * l + 1] += gLc.y * sf;
          G[gLightC + 3 * l + 2] += gLc.z * sf;
        }
      }
      if (m.reflection > 0.0f) {
        out.x += m.reflection * p.bg.x;
        out.y += m.reflection * p.bg.y;
        out.z += m.reflection * p.bg.z;
        if (GRAD) {
          G[gReflection] += dot(gc, p.bg);
          G[gBg] += m.reflection * gc.x;
          G[gBg + 1] += m.reflection * gc.y;
          G[gBg + 2] += m.reflection * gc.z;
        }
      } else if (GRAD) {
        G[gReflection] += dot(gc, p.bg);
      }
      if (!GRAD) {
        float4 c4 = make_float4(out.x, out.y, out.z, 1.0f);
        if (fog.on) {
          if (p.transparentBg) {
            c4.w *= fog.f;
          } else {
            c4.x = p.fogColor.x * (1.0f - fog.f) + c4.x * fog.f;
            c4.y = p.fogColor.y * (1.0f - fog.f) + c4.y * fog.f;
            c4.z = p.fogColor.z * (1.0f - fog.f) + c4.z * fog.f;
          }
        }
        b.colorHi[i] = c4;
      } else {
        // roughness -> Blinn exponent (shading.hpp:34-41), zero where clamped
        if (gEx != 0.0f && m.roughness >= 1e-6f) {
          const float e = 1.0f / m.roughness;
          if (e > 1.0f && e < 1.0e6f) G[gRoughness] += gEx * (-e * e);
        }
        // fog backward
        float gT = 0.0f;
        if (fog.on) {
          float gF;
          if (p.transparentBg) {
            gF = g.w;
          } else {
            G[gFogColor] += g.x * (1.0f - fog.f);
            G[gFogColor + 1] += g.y * (1.0f - fog.f);
            G[gFogColor + 2] += g.z * (1.0f - fog.f);
            gF = g.x * (out.x - p.fogColor.x) + g.y * (out.y - p.fogColor.y) + g.z * (out.z - p.fogColor.z);
          }
          G[gFogStart] += gF * fog.dStart;
          G[gFogEnd] += gF * fog.dEnd;
          gT += gF * fog.dz * dot(rd, p.camDir);
        }
        // secondary-ray origin O = P + ng eps (ng = N for a sphere)
        f3 gP = gO;
        gN = gN + gO * eps;
        const float gEps = dot(ng, gO);
        {
          // eps = K max(|Px|, |Py|, |Pz|, dirMax t)  (secondary_rays.hpp:38-46)
          const float K = 0x1.0fp-21f;
          const float dirMax = fmaxf(fabsf(rd.x), fmaxf(fabsf(rd.y), fabsf(rd.z)));
          const float ax = fabsf(P.x), ay = fabsf(P.y), az = fabsf(P.z), at = dirMax * t;
          const float mx = fmaxf(fmaxf(ax, ay), fmaxf(az, at));
          if (mx == ax) gP.x += gEps * K * copysignf(1.0f, P.x);
          else if (mx == ay) gP.y += gEps * K * copysignf(1.0f, P.y);
          else if (mx == az) gP.z += gEps * K * copysignf(1.0f, P.z);
          else gT += gEps * K * dirMax;
        }
        // N = sgn Ng / |Ng|, Ng = P - c, P = org + rd t(c, r)
        const f3 gNg = normalizeBack(nHat, ngLen, gN * sgn);
        gP = gP + gNg;
        f3 gCenter = neg(gNg);
        const float den = dot(Ng, rd);
        float gRad = 0.0f;
        if (den != 0.0f) {
          const float gtt = gT + dot(rd, gP);
          gCenter = gCenter + Ng * (gtt / den);
          gRad = gtt * rad / den;
        }
        atomicAdd3(b.gColor, sk, gC);
        atomicAdd3(b.gCenter, sk, gCenter);
        if (b.gRadius) atomicAdd(b.gRadius + sk, gRad);
        used = 1;
      }
    }
  }
  if (GRAD) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < kGlobals; ++k) {
      float v = G[k];
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 16);
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 8);
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 4);
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 2);
      v += __shfl_xor_sync(0xFFFFFFFFu, v, 1);
      if (lane == 0 && v != 0.0f) atomicAdd(&sAcc[k], v);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kGlobals; k += blockDim.x)
      if (sAcc[k] != 0.0f) atomicAdd(&b.gGlobal[k], double(sAcc[k]));
    warpCount(&b.stats[0], used);
  }
  warpCount(&b.stats[1], traced);
  warpCount(&b.stats[2], ovf);
}

// Box average of the fogged hi-res colour with the non-finite guard
// (image_ops.cpp:9-35): the value the gamma derivative is taken at.
__global__ void k_adj_down(Params p, const float4* colorHi, float4* out, uint32_t nOut) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nOut) return;
  const int ox = int(o % uint32_t(p.outW)), oy = int(o / uint32_t(p.outW));
  float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  for (int dy = 0; dy < p.ss; ++dy)
    for (int dx = 0; dx < p.ss; ++dx) {
      const float4 c = colorHi[size_t(oy * p.ss + dy) * p.W + size_t(ox * p.ss + dx)];
      a[0] += isfinite(c.x) ? c.x : 0.0f;
      a[1] += isfinite(c.y) ? c.y : 0.0f;
      a[2] += isfinite(c.z) ? c.z : 0.0f;
      a[3] += isfinite(c.w) ? c.w : 0.0f;
    }
  const float inv = 1.0f / float(p.ss * p.ss);
  out[o] = make_float4(a[0] * inv, a[1] * inv, a[2] * inv, a[3] * inv);
}

ubr_status adjointCheck(Context* c, const Scene& sc, const ubr_render_desc& d, const Params& p) {
  if (sc.primCount[kMesh] || sc.primCount[kRound] || sc.primCount[kCone])
    return setError(c, UBR_INVALID_ARGUMENT, "adjoint: only sphere scenes are differentiable");
  if (sc.primCount[kSphere] == 0) return setError(c, UBR_INVALID_ARGUMENT, "adjoint: scene has no spheres");
  if (p.maxIters > 1 && !sc.opaque)
    return setError(c, UBR_INVALID_ARGUMENT, "adjoint: needs one opaque layer (opaque spheres or transparency off)");
  if (d.env_lights > 0) return setError(c, UBR_INVALID_ARGUMENT, "adjoint: env dome lights are not differentiable");
  if (p.nLights > kAdjLights) return setError(c, UBR_INVALID_ARGUMENT, "adjoint: at most 4 lights");
  if (p.shadowsActive && p.shadowRays != p.nLights)
    return setError(c, UBR_INVALID_ARGUMENT, "adjoint: soft shadows are not differentiable");
  if (p.aoSamples > 0 && p.aoEnhanced && (p.aoBentNormal || p.aoMultibounce))
    return setError(c, UBR_INVALID_ARGUMENT, "adjoint: AO bent normal / multibounce are not differentiable");
  if (sc.principled) return setError(c, UBR_INVALID_ARGUMENT, "adjoint: principled materials are not differentiable");
  if (p.aaMode == 1 && (p.ss > 1 || d.aa_depth > 1))
    return setError(c, UBR_INVALID_ARGUMENT, "adjoint: adaptive AA is not differentiable (use the grid)");
  if ((d.ao_res_div < 0 ? p.ss : d.ao_res_div) > 1 && p.aoSamples > 0)
    return setError(c, UBR_INVALID_ARGUMENT, "adjoint: coarse-grid AO is not differentiable");
  return UBR_OK;
}

}  // namespace

ubr_status adjoint(Context* c, const Scene* sc, const ubr_render_desc& d, const float* dColor, ubr_grads& g) {
  Params p;
  std::vector<LightD> lights;
  ubr_status st = makeParams(c, d, p, lights);
  if (st != UBR_OK) return st;
  if ((st = adjointCheck(c, *sc, d, p)) != UBR_OK) return st;
  if (!dColor) return setError(c, UBR_INVALID_ARGUMENT, "adjoint: d_color is NULL");
  const bool dev = g.memory == UBR_MEMORY_DEVICE;
  const uint32_t npix = uint32_t(p.W) * uint32_t(p.H), nout = uint32_t(p.outW) * uint32_t(p.outH);
  const uint64_t nSph = sc->view.baseSph;
  const bool needFwd = !(std::fabs(p.gamma - 1.0f) <= 1.0e-4f);
  cudaStream_t s = c->stream;
  AdjBufs b{};
  float2* hit = scratchT<float2>(c, 60, npix, st);
  float4* colorHi = needFwd ? scratchT<float4>(c, 61, npix, st) : nullptr;
  float4* outFwd = needFwd ? scratchT<float4>(c, 62, nout, st) : nullptr;
  LightD* dl = scratchT<LightD>(c, 63, lights.size() + 1, st);
  double* gg = scratchT<double>(c, 64, kGlobals, st);
  unsigned long long* stats = scratchT<unsigned long long>(c, 65, 4, st);
  const float4* dOut = reinterpret_cast<const float4*>(dColor);
  float4* dOutDev = nullptr;
  if (!dev) dOutDev = scratchT<float4>(c, 66, nout, st);
  // per-sphere accumulators: the caller's device arrays, or scratch copied back
  float* gCol = g.sphere_color;
  float* gCen = g.sphere_center;
  float* gRad = g.sphere_radius;
  if (!dev) {
    gCol = g.sphere_color ? scratchT<float>(c, 67, 3 * nSph, st) : nullptr;
    gCen = g.sphere_center ? scratchT<float>(c, 68, 3 * nSph, st) : nullptr;
    gRad = g.sphere_radius ? scratchT<float>(c, 69, nSph, st) : nullptr;
  }
  if (st != UBR_OK) return st;
  cudaEventRecord(c->ev[0], s);
  if (!dev) {
    UBR_CUDA(c, cudaMemcpyAsync(dOutDev, dColor, size_t(nout) * 16, cudaMemcpyHostToDevice, s));
    dOut = dOutDev;
  }
  if (!lights.empty())
    UBR_CUDA(c, cudaMemcpyAsync(dl, lights.data(), lights.size() * sizeof(LightD), cudaMemcpyHostToDevice, s));
  UBR_CUDA(c, cudaMemsetAsync(gg, 0, kGlobals * sizeof(double), s));
  UBR_CUDA(c, cudaMemsetAsync(stats, 0, 4 * sizeof(unsigned long long), s));
  if (gCol) UBR_CUDA(c, cudaMemsetAsync(gCol, 0, 3 * nSph * sizeof(float), s));
  if (gCen) UBR_CUDA(c, cudaMemsetAsync(gCen, 0, 3 * nSph * sizeof(float), s));
  if (gRad) UBR_CUDA(c, cudaMemsetAsync(gRad, 0, nSph * sizeof(float), s));
  b.hit = hit;
  b.dOut = dOut;
  b.outFwd = outFwd;
  b.colorHi = colorHi;
  b.lights = dl;
  b.gColor = gCol;
  b.gCenter = gCen;
  b.gRadius = gRad;
  b.gGlobal = gg;
  b.stats = stats;
  b.flags = g.flags;
  const int TB = 128;
  const uint32_t grid = (npix + TB - 1) / TB;
  cudaEventRecord(c->ev[2], s);
  k_adj_primary<<<grid, TB, 0, s>>>(p, travOf(sc->view), hit, npix, stats);
  if (needFwd) {
    k_adj_shade<false><<<grid, TB, 0, s>>>(p, sc->view, b, npix);
    k_adj_down<<<(nout + 255) / 256, 256, 0, s>>>(p, colorHi, outFwd, nout);
  }
  k_adj_shade<true><<<grid, TB, 0, s>>>(p, sc->view, b, npix);
  UBR_CUDA(c, cudaGetLastError());
  cudaEventRecord(c->ev[3], s);
  const cudaMemcpyKind back = cudaMemcpyDeviceToHost;
  if (!dev) {
    if (gCol) UBR_CUDA(c, cudaMemcpyAsync(g.sphere_color, gCol, 3 * nSph * sizeof(float), back, s));
    if (gCen) UBR_CUDA(c, cudaMemcpyAsync(g.sphere_center, gCen, 3 * nSph * sizeof(float), back, s));
    if (gRad) UBR_CUDA(c, cudaMemcpyAsync(g.sphere_radius, gRad, nSph * sizeof(float), back, s));
  }
  double hg[kGlobals];
  unsigned long long hs[4];
  UBR_CUDA(c, cudaMemcpyAsync(hg, gg, sizeof(hg), back, s));
  UBR_CUDA(c, cudaMemcpyAsync(hs, stats, sizeof(hs), back, s));
  UBR_CUDA(c, cudaStreamSynchronize(s));
  float ms = 0.0f;
  cudaEventElapsedTime(&ms, c->ev[2], c->ev[3]);
  // fill the host struct; light vectors: L = normalize(-direction),
  // colour x intensity (buildSceneLights, embree_renderer.cpp:436-458)
  for (int k = 0; k < 9; ++k) g.material[k] = float(hg[k]);
  for (int k = 0; k < 3; ++k) {
    g.ambient_color[k] = float(hg[gAmbColor + k]);
    g.background[k] = float(hg[gBg + k]);
    g.fog_color[k] = float(hg[gFogColor + k]);
  }
  g.fog_start = float(hg[gFogStart]);
  g.fog_end = float(hg[gFogEnd]);
  g.ao_distance = float(hg[gAoDistance]);
  g.ao_intensity = float(hg[gAoIntensity]);
  g.specular_scale = float(hg[gSpecScale]);
  for (int l = 0; l < kAdjLights; ++l) {
    for (int k = 0; k < 3; ++k) g.light_direction[l][k] = g.light_color[l][k] = 0.0f;
    g.light_intensity[l] = 0.0f;
    if (l >= int(d.light_count)) continue;
    const ubr_light& ul = d.lights[l];
    const double dir[3] = {ul.direction[0], ul.direction[1], ul.direction[2]};
    const double len = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
    const double gL[3] = {hg[gLightL + 3 * l], hg[gLightL + 3 * l + 1], hg[gLightL + 3 * l + 2]};
    if (len > 0.0) {
      const double Lv[3] = {-dir[0] / len, -dir[1] / len, -dir[2] / len};
      const double lg = Lv[0] * gL[0] + Lv[1] * gL[1] + Lv[2] * gL[2];
      for (int k = 0; k < 3; ++k) g.light_direction[l][k] = float(-(gL[k] - Lv[k] * lg) / len);
    }
    double gi = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double gc = hg[gLightC + 3 * l + k];
      g.light_color[l][k] = float(gc * ul.intensity);
      gi += gc * ul.color[k];
    }
    g.light_intensity[l] = float(gi);
  }
  g.samples = hs[0];
  g.rays = hs[1];
  g.adjoint_ms = ms;
  return UBR_OK;
}

}  // namespace ubr

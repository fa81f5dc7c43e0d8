// gi.cu -- the path-traced GI pass on the GPU: the pt1 gather
// (integrator/pt1/pt1_gather.hpp) on the render grid or on a reduced grid
// with its own primary rays (pt1_gbuffer.hpp), the a-trous denoise of E
// (pt1_denoise.cpp), the joint-bilateral upsample and the edge patch
// (pt1_upsample.hpp), the [E] composite (render/embree_renderer.cpp:908-927),
// and the pt2 extensions layered onto the same gather (integrator/pt2/):
// the Owen-scrambled Sobol / blue-noise first bounce, area-light NEE jitter,
// emission at gather vertices, emissive-primitive NEE with MIS, traced mirror
// and glossy reflection, variance-adaptive spp, ReSTIR spatial rounds
// (integrator/pt2/pt2_reservoir.hpp, pt2_spatial.hpp).
//
// Up to eight lanes share a gather point, each taking every eighth sample (a
// ReSTIR gather, whose reservoir streams the samples in order, runs one
// thread per point); every stream is a pure function of (grid index, sample
// index, pt1Seed), as in the reference, so the oracle draws the same samples
// and the frames agree up to traversal float order.
#include <algorithm>

#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>
#include <thrust/iterator/permutation_iterator.h>
#include <thrust/iterator/transform_iterator.h>

#include "gi.cuh"
#include "trace.cuh"

namespace ubr {
namespace {

// ---- pt2 sampler (integrator/pt2/pt2_sampler.hpp): shuffled, hash-based
// Owen-scrambled Sobol after Burley, "Practical Hash-based Owen Scrambling"
// (JCGT 9(4), 2020), the Laine-Karras style nested hash on reversed bits,
// and the blue-noise pixel arrangement (pixels own contiguous sections of
// one global sequence, ordered along a scrambled Morton curve). ----
UBR_D uint32_t owenHash(uint32_t n, uint32_t seed) {
  n ^= n * 0x3d20adeau;
  n += seed;
  n *= (seed >> 16) | 1u;
  n ^= n * 0x05526c56u;
  n ^= n * 0x53a22864u;
  return n;
}
// the base-4 variant keeps each 2x2 quad of the Morton curve together
UBR_D uint32_t owenHashBase4(uint32_t n, uint32_t seed) {
  n ^= n * 0x3d20adeau;
  n ^= (n >> 1) & (n << 1) & 0x55555555u;
  n += seed;
  n *= (seed >> 16) | 1u;
  n ^= (n >> 1) & (n << 1) & 0x55555555u;
  n ^= n * 0x05526c56u;
  n ^= n * 0x53a22864u;
  return n;
}
UBR_D uint32_t expandBits16(uint32_t x) {
  x &= 0x0000ffffu;
  x = (x ^ (x << 8)) & 0x00ff00ffu;
  x = (x ^ (x << 4)) & 0x0f0f0f0fu;
  x = (x ^ (x << 2)) & 0x33333333u;
  x = (x ^ (x << 1)) & 0x55555555u;
  return x;
}
UBR_D float uintToFloatExcl(uint32_t n) { return float(n) * (1.0f / 4294967808.0f); }
// One dimension of the scrambled Sobol point whose (shuffled) index has
// reversed bit order.  Dimension 0 is the Van der Corput sequence; the
// direction numbers of dimension 1 in reversed-bit order are the rows of
// Pascal's triangle mod 2 (v0 = 1, v(i) = v(i-1) ^ (v(i-1) << 1)).
UBR_D float sobolDim(uint32_t revIndex, int dim, uint32_t scramble) {
  uint32_t result = 0;
  if (dim == 0) {
    result = __brev(revIndex);
  } else {
    uint32_t i = 0, v = 1u, vi = 0;  // v = direction number vi
    while (revIndex != 0u) {
      const uint32_t j = __clz(revIndex);
      const uint32_t target = i + j;
      while (vi < target) {
        v ^= v << 1;
        ++vi;
      }
      result ^= v;
      i += j + 1;
      revIndex <<= j;
      revIndex <<= 1;
    }
  }
  return uintToFloatExcl(__brev(owenHash(result, scramble)));
}
// pt2SobolBurley2D: the dimension-set-0 scramble constants of the scheme
UBR_D void sobol2D(uint32_t index, uint32_t seed, float& u1, float& u2) {
  index = owenHash(__brev(index), seed ^ 0xf8ade99au);
  u1 = sobolDim(index, 0, seed ^ 0xe0aaaf76u);
  u2 = sobolDim(index, 1, seed ^ 0x94964d4eu);
}
// environmentRadiance (irradiance_cache.hpp:188-196): the gather's miss term.
UBR_D f3 giEnvironment(const GiP& g, f3 wi) {
  const float w = 0.5f * (dot(wi, g.envUp) + 1.0f);
  const float e = g.envI;
  return f3{e * g.amb.x * (g.ground.x + (g.sky.x - g.ground.x) * w),
            e * g.amb.y * (g.ground.y + (g.sky.y - g.ground.y) * w),
            e * g.amb.z * (g.ground.z + (g.sky.z - g.ground.z) * w)};
}

// A gather-ray hit as a path vertex.
struct Vertex {
  f3 rad, emitted, alb, P, N;
};

// pt1EvalVertex (pt1_gather.hpp:117-227): its reflected, shadow-tested direct
// light, its reflectance kd * C, position and shading normal faced toward the
// ray origin; with `emit` its emission * pigment; with a stream (pt2) an
// area light (radius > 0) gets one cone-jittered shadow ray drawn from it,
// otherwise the light's centre ray.  Outline primitives end the path.
template <int KM>
UBR_D bool evalVertex(const DScene& s, const LightD* lights, int nLights, const Hit& h, f3 O, f3 wi, bool emit,
                      uint32_t* r0, uint32_t* r1, Vertex& v, uint32_t& nee, uint32_t& ovf) {
  const int kind = refKind(h.ref);
  const uint32_t prim = refPrim(h.ref);
  f3 C, NgSh, Ny;
  uint32_t mi;
  if (kind == kMesh) {
    const uint32_t i0 = __ldg(&s.meshIdx[3 * prim]), i1 = __ldg(&s.meshIdx[3 * prim + 1]),
                   i2 = __ldg(&s.meshIdx[3 * prim + 2]);
    const float w0 = 1.0f - h.u - h.v;
    float nb[3];
    for (int k = 0; k < 3; ++k)
      nb[k] = w0 * __ldg(&s.meshNrm[3 * i0 + k]) + h.u * __ldg(&s.meshNrm[3 * i1 + k]) +
              h.v * __ldg(&s.meshNrm[3 * i2 + k]);
    const float4 c0 = __ldg(&s.meshCol[i0]), c1 = __ldg(&s.meshCol[i1]), c2 = __ldg(&s.meshCol[i2]);
    C = f3{w0 * c0.x + h.u * c1.x + h.v * c2.x, w0 * c0.y + h.u * c1.y + h.v * c2.y,
           w0 * c0.z + h.u * c1.z + h.v * c2.z};
    Ny = normalize(f3{nb[0], nb[1], nb[2]});
    mi = s.meshTriMat ? __ldg(&s.meshTriMat[s.baseTri ? prim % s.baseTri : 0]) : s.meshMat;
    NgSh = h.Ng;
  } else {
    if (__ldg(&s.primFromEdge[kind][prim])) return false;
    const float4 fc = __ldg(&s.primColor[kind][prim]);
    mi = __ldg(&s.primMat[kind][prim]);
    C = f3{fc.x, fc.y, fc.z};
    Ny = safeNormalize(h.Ng);
    NgSh = Ny;
  }
  const ubr_material& m = s.mats[mi];
  const float kd = diffuseWeight(m);
  if (dot(Ny, wi) > 0.0f) Ny = neg(Ny);
  const f3 Py{O.x + wi.x * h.t, O.y + wi.y * h.t, O.z + wi.z * h.t};
  const float eps = selfIntersectEps(Py, wi, h.t);
  f3 ng = dot(NgSh, Ny) < 0.0f ? neg(NgSh) : NgSh;
  ng = safeNormalize(ng, Ny);
  const f3 So{Py.x + ng.x * eps, Py.y + ng.y * eps, Py.z + ng.z * eps};
  const TravScene ts = travOf(s);
  f3 E{0.0f, 0.0f, 0.0f};
  for (int l = 0; l < nLights; ++l) {
    const LightD L = lights[l];
    const float ndl = dot(Ny, L.L);
    if (ndl <= 0.0f) continue;
    f3 dir = L.L;
    if (r0 && L.radius > 0.0f) {
      tea2(*r0, *r1);
      dir = sampleLightDir(L, u32ToUnorm(*r0), u32ToUnorm(*r1));
    }
    Ray r{So, dir, eps, kInfF};
    Hit hh;
    Count cnt;
    const float sh = traverse<false, KM, true>(ts, r, hh, ovf, &cnt, true) ? 0.0f : 1.0f;
    ++nee;
    E.x += ndl * L.color.x * sh;
    E.y += ndl * L.color.y * sh;
    E.z += ndl * L.color.z * sh;
  }
  v.rad = f3{kd * C.x * E.x, kd * C.y * E.y, kd * C.z * E.z};
  v.emitted = f3{0.0f, 0.0f, 0.0f};
  if (emit && m.emission > 0.0f) v.emitted = f3{m.emission * C.x, m.emission * C.y, m.emission * C.z};
  v.alb = f3{kd * C.x, kd * C.y, kd * C.z};
  v.P = Py;
  v.N = Ny;
  return true;
}

// ---- emissive NEE (pt2_emissive.hpp:279-520) ----
constexpr float kPiF = 3.14159265358979323846f;

UBR_D float emitPdfTri(const EmitD& el, uint32_t ti, float dist2, float cosL) {
  if (cosL <= 1.0e-6f) return 0.0f;
  const float area = el.rec[size_t(ti) * kEmitF4].w;
  return el.pdfChoose[ti] * dist2 / (cosL * area);
}

// One power-sampled emitter draw from receiver (P, N): exactly two tea2
// draws (pick, point), visibility, balance-heuristic weight against the
// cosine gather; returns the E_stored term.
template <int KM>
UBR_D f3 emissiveNee(const EmitD& el, const DScene& s, f3 P, f3 N, f3 Ng, float epsT, uint32_t& s0, uint32_t& s1,
                     uint32_t& ovf) {
  const f3 zero{0.0f, 0.0f, 0.0f};
  tea2(s0, s1);
  const float u = u32ToUnorm(s0);
  uint32_t lo = 0, hi = el.n - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) / 2;
    if (el.cdf[mid] < u) lo = mid + 1;
    else hi = mid;
  }
  const float4* r = el.rec + size_t(lo) * kEmitF4;
  f3 dir, Le;
  float target, pdfSA;
  if (lo < el.triCount) {
    tea2(s0, s1);
    const float b0 = u32ToUnorm(s0), b1 = u32ToUnorm(s1);
    const float sq = sqrtf(b0);
    const float w1 = 1.0f - sq, w2 = b1 * sq, w0 = 1.0f - w1 - w2;
    const float4 p0 = r[0], p1 = r[1], p2 = r[2], e0 = r[3], e1 = r[4], e2 = r[5], nn = r[6];
    const f3 S{p0.x * w0 + p1.x * w1 + p2.x * w2, p0.y * w0 + p1.y * w1 + p2.y * w2,
               p0.z * w0 + p1.z * w1 + p2.z * w2};
    Le = f3{e0.x * w0 + e1.x * w1 + e2.x * w2, e0.y * w0 + e1.y * w1 + e2.y * w2,
            e0.z * w0 + e1.z * w1 + e2.z * w2};
    const f3 d{S.x - P.x, S.y - P.y, S.z - P.z};
    const float dist2 = dot(d, d);
    if (dist2 <= 1.0e-12f) return zero;
    const float dist = sqrtf(dist2);
    dir = f3{d.x / dist, d.y / dist, d.z / dist};
    const float cosP = dot(N, dir);
    if (cosP <= 0.0f) return zero;
    const float cosL = fabsf(nn.x * dir.x + nn.y * dir.y + nn.z * dir.z);
    pdfSA = emitPdfTri(el, lo, dist2, cosL);
    if (pdfSA <= 0.0f) return zero;
    target = dist;
  } else {
    tea2(s0, s1);
    const float u1 = u32ToUnorm(s0), u2 = u32ToUnorm(s1);
    const float phi = 2.0f * kPiF * u2;
    const float4 q0 = r[0], q1 = r[1], q2 = r[2], q3 = r[3];
    const int kindE = int(q1.w);
    const f3 g0{q0.x, q0.y, q0.z}, axis{q1.x, q1.y, q1.z};
    const float area = q0.w, radius = q2.w, len = q3.x;
    Le = f3{q2.x, q2.y, q2.z};
    if (kindE == 1) {
      // uniform solid-angle cone toward the sphere
      const f3 d{g0.x - P.x, g0.y - P.y, g0.z - P.z};
      const float dc2 = dot(d, d);
      const float r2 = radius * radius;
      if (dc2 <= r2 * 1.0002f) return zero;
      const float dc = sqrtf(dc2);
      const float sin2Max = r2 / dc2;
      const float cosMax = sqrtf(fmaxf(0.0f, 1.0f - sin2Max));
      const float oneMinusCos = sin2Max / (1.0f + cosMax);
      const float cosT = 1.0f - u1 * oneMinusCos;
      const float sinT = sqrtf(fmaxf(0.0f, 1.0f - cosT * cosT));
      const Frame3 fr = frameFromNormal(f3{d.x / dc, d.y / dc, d.z / dc});
      const float sx = sinT * cosf(phi), sy = sinT * sinf(phi);
      dir = f3{fr.t.x * sx + fr.b.x * sy + fr.n.x * cosT, fr.t.y * sx + fr.b.y * sy + fr.n.y * cosT,
               fr.t.z * sx + fr.b.z * sy + fr.n.z * cosT};
      pdfSA = el.pdfChoose[lo] / (2.0f * kPiF * oneMinusCos);
      const float b = dot(d, dir);
      const float disc = fmaxf(0.0f, b * b - (dc2 - r2));
      target = b - sqrtf(disc);
    } else {
      const Frame3 fr = frameFromNormal(axis);
      f3 S, nS;
      if (kindE == 2) {
        const float cp = cosf(phi), sp = sinf(phi);
        nS = f3{fr.t.x * cp + fr.b.x * sp, fr.t.y * cp + fr.b.y * sp, fr.t.z * cp + fr.b.z * sp};
        const float hgt = u1 * len;
        S = f3{g0.x + axis.x * hgt + nS.x * radius, g0.y + axis.y * hgt + nS.y * radius,
               g0.z + axis.z * hgt + nS.z * radius};
      } else {
        const float rr = radius * sqrtf(u1);
        const float cp = cosf(phi), sp = sinf(phi);
        S = f3{g0.x + (fr.t.x * cp + fr.b.x * sp) * rr, g0.y + (fr.t.y * cp + fr.b.y * sp) * rr,
               g0.z + (fr.t.z * cp + fr.b.z * sp) * rr};
        nS = axis;
      }
      const f3 d{S.x - P.x, S.y - P.y, S.z - P.z};
      const float dist2 = dot(d, d);
      if (dist2 <= 1.0e-12f) return zero;
      const float dist = sqrtf(dist2);
      dir = f3{d.x / dist, d.y / dist, d.z / dist};
      const float cosL = fabsf(dot(nS, dir));
      if (cosL <= 1.0e-6f) return zero;
      pdfSA = el.pdfChoose[lo] * dist2 / (cosL * area);
      target = dist;
    }
    const float cosP0 = dot(N, dir);
    if (cosP0 <= 0.0f) return zero;
    if (pdfSA <= 0.0f) return zero;
  }
  const float cosP = dot(N, dir);
  const float eps = selfIntersectEps(P, dir, epsT);
  f3 ng = dot(Ng, N) < 0.0f ? neg(Ng) : Ng;
  ng = safeNormalize(ng, N);
  const f3 O{P.x + ng.x * eps, P.y + ng.y * eps, P.z + ng.z * eps};
  Ray ry{O, dir, eps, target - 2.0f * eps};
  Hit hh;
  Count cnt;
  if (ry.tnear < ry.tfar && traverse<false, KM, true>(travOf(s), ry, hh, ovf, &cnt, true)) return zero;
  const float pdfCos = cosP * (1.0f / kPiF);
  const float w = pdfSA / (pdfSA + pdfCos);
  const float k = w * cosP / (kPiF * pdfSA);
  return f3{Le.x * k, Le.y * k, Le.z * k};
}

// pt2EmissiveHitWeight (pt2_emissive.hpp:446-520): the cosine side's balance
// weight for a first-bounce hit on an NEE-covered emitter; 1 otherwise.
UBR_D float emissiveHitWeight(const EmitD& el, int kind, uint32_t prim, f3 O, f3 wi, float tfar, float cosP,
                              f3 ngHit) {
  if (el.n == 0) return 1.0f;
  const float pdfCos = (cosP > 0.0f ? cosP : 0.0f) * (1.0f / kPiF);
  if (pdfCos <= 0.0f) return 1.0f;
  if (kind == kMesh) {
    if (prim >= el.nTriIndex) return 1.0f;
    const uint32_t ti = el.triIndex[prim];
    if (ti == 0xFFFFFFFFu) return 1.0f;
    const float4 nn = el.rec[size_t(ti) * kEmitF4 + 6];
    const float cosL = fabsf(nn.x * wi.x + nn.y * wi.y + nn.z * wi.z);
    const float pdfSA = emitPdfTri(el, ti, tfar * tfar, cosL);
    if (pdfSA <= 0.0f) return 1.0f;
    return pdfCos / (pdfCos + pdfSA);
  }
  if (kind == kSphere) {
    if (prim >= el.nSphereIndex) return 1.0f;
    const uint32_t ci = el.sphereIndex[prim];
    if (ci == 0xFFFFFFFFu) return 1.0f;
    const float4* r = el.rec + size_t(el.triCount + ci) * kEmitF4;
    const f3 d{r[0].x - O.x, r[0].y - O.y, r[0].z - O.z};
    const float dc2 = dot(d, d);
    const float r2 = r[2].w * r[2].w;
    if (dc2 <= r2 * 1.0002f) return 1.0f;
    const float sin2Max = r2 / dc2;
    const float cosMax = sqrtf(fmaxf(0.0f, 1.0f - sin2Max));
    const float oneMinusCos = sin2Max / (1.0f + cosMax);
    if (oneMinusCos <= 0.0f) return 1.0f;
    const float pdfSA = el.pdfChoose[el.triCount + ci] / (2.0f * kPiF * oneMinusCos);
    if (pdfSA <= 0.0f) return 1.0f;
    return pdfCos / (pdfCos + pdfSA);
  }
  if (kind == kCone) {
    if (prim >= el.nCylIndex) return 1.0f;
    const uint4 ref = el.cylIndex[prim];
    uint32_t part = ref.x;
    const uint32_t probe = ref.x != 0xFFFFFFFFu ? ref.x : ref.y != 0xFFFFFFFFu ? ref.y : ref.z;
    if (probe == 0xFFFFFFFFu) return 1.0f;
    const float4 ax4 = el.rec[size_t(el.triCount + probe) * kEmitF4 + 1];
    const f3 axis{ax4.x, ax4.y, ax4.z};
    const f3 ng = safeNormalize(ngHit, axis);
    const float nu = dot(ng, axis);
    if (nu >= 0.99f) part = ref.z;
    else if (nu <= -0.99f) part = ref.y;
    if (part == 0xFFFFFFFFu) return 1.0f;
    const float area = el.rec[size_t(el.triCount + part) * kEmitF4].w;
    const float cosL = fabsf(dot(ng, wi));
    if (cosL <= 1.0e-6f) return 1.0f;
    const float pdfSA = el.pdfChoose[el.triCount + part] * tfar * tfar / (cosL * area);
    if (pdfSA <= 0.0f) return 1.0f;
    return pdfCos / (pdfCos + pdfSA);
  }
  return 1.0f;
}

// pt1GatherPoint (pt1_gather.hpp:268-523) at one grid point (px, py) of a
// grid: E_stored = (1/spp) sum over cosine-hemisphere paths of the NEE
// radiance (and, pt2, the MIS-weighted emission) at every vertex and the sky
// where the path escapes, plus (pt2 with emitters) one emissive NEE draw per
// sample at the origin; Russian roulette from the second vertex on; a first
// bounce below the geometric horizon adds nothing.  First bounce: pt2 the
// scrambled Sobol point (blue-noise section or per-point sequence), pt1
// Hammersley + Cranley-Patterson when ld, else the tea2 stream.  Returns
// (sum of E, number of first bounces that hit or fall below the horizon)
// over the samples sFirst, sFirst + sStep, ... < spp; `half` gets the sum of
// those among the first spp/2.
// ReSTIR (rsv non-null, sFirst 0, sStep 1): every sample is also one
// candidate streamed, in sample order, into the point's reservoir
// (pt1_gather.hpp:287-297, 451-470, 486-499).
template <int KM>
UBR_D float4 gatherPoint(const GiP& g, const DScene& s, const LightD* lights, int nLights, f3 P, f3 N, f3 Ng,
                         float tEps, uint32_t seed, uint32_t px, uint32_t py, int spp, int sFirst, int sStep,
                         f3& half, uint32_t& rays, uint32_t& nee, uint32_t& ovf, float4* rsv = nullptr) {
  const Frame3 f = frameFromNormal(N);
  const float eps = selfIntersectEps(P, N, tEps);
  const f3 O{P.x + N.x * eps, P.y + N.y * eps, P.z + N.z * eps};
  const int maxB = g.bounces < 1 ? 1 : g.bounces;
  float cpx = 0.0f, cpy = 0.0f;
  if (g.ld) {
    uint32_t c0 = seed, c1 = 0x9E3779B9u;
    tea2(c0, c1);
    cpx = u32ToUnorm(c0);
    cpy = u32ToUnorm(c1);
  }
  // pt2MakePixelSampler: a section of the global sequence (blue noise) or
  // an independent sequence per point
  uint32_t idxBase = 0, sSeed = seed;
  if (g.pt2 && g.pattern == 1) {
    const uint32_t morton = (expandBits16(px) << 1) | expandBits16(py);
    idxBase = __brev(owenHashBase4(__brev(morton), g.seedMix)) * g.sppPow2;
    sSeed = g.seedMix;
  }
  const bool emitNee = g.pt2 && g.em.n > 0;
  const TravScene ts = travOf(s);
  f3 Esum{0.0f, 0.0f, 0.0f};
  half = f3{0.0f, 0.0f, 0.0f};
  int nOcc = 0;
  uint32_t rs0 = seed ^ 0x52455354u, rs1 = 0x47490001u;
  double rWSum = 0.0;
  f3 rPos{0.0f, 0.0f, 0.0f}, rNrm{0.0f, 0.0f, 0.0f}, rRad{0.0f, 0.0f, 0.0f};
  float rPHat = 0.0f;
  for (int sI = sFirst; sI < spp; sI += sStep) {
    uint32_t s0 = seed, s1 = uint32_t(sI + g.sampleOffset);
    tea2(s0, s1);
    float u1, u2;
    if (g.pt2) {
      sobol2D(idxBase + uint32_t(sI + g.sampleOffset), sSeed, u1, u2);
    } else if (g.ld) {
      u1 = float(sI) / float(spp) + cpx;
      u2 = radicalInverse2(uint32_t(sI)) + cpy;
      if (u1 >= 1.0f) u1 -= 1.0f;
      if (u2 >= 1.0f) u2 -= 1.0f;
    } else {
      u1 = u32ToUnorm(s0);
      u2 = u32ToUnorm(s1);
    }
    f3 wi = cosineSampleHemisphere(u1, u2, f);
    const bool horizonOk = dot(wi, Ng) > 0.0f;
    if (!horizonOk) ++nOcc;
    const float cand0Cos = dot(wi, N);
    f3 org = O;
    float tnear = eps;
    f3 thr{1.0f, 1.0f, 1.0f}, L{0.0f, 0.0f, 0.0f};
    f3 candPos{0.0f, 0.0f, 0.0f}, candN{0.0f, 0.0f, 0.0f};
    bool candValid = false;
    for (int bnc = 1; horizonOk && bnc <= maxB; ++bnc) {
      Ray r{org, wi, tnear, g.maxDist};
      Hit h;
      Count cnt;
      traverse<false, KM>(ts, r, h, ovf, &cnt, false);
      ++rays;
      if (h.ref == kInvalid) {
        const f3 env = giEnvironment(g, wi);
        L.x += thr.x * env.x;
        L.y += thr.y * env.y;
        L.z += thr.z * env.z;
        if (rsv && bnc == 1) {  // escaped: the candidate sits 1e7 along the segment
          candPos = f3{O.x + wi.x * 1.0e7f, O.y + wi.y * 1.0e7f, O.z + wi.z * 1.0e7f};
          candN = neg(wi);
          candValid = true;
        }
        break;
      }
      if (bnc == 1) ++nOcc;
      Vertex v;
      if (!evalVertex<KM>(s, lights, nLights, h, org, wi, g.pt2 && g.emissive, g.pt2 ? &s0 : nullptr,
                          g.pt2 ? &s1 : nullptr, v, nee, ovf)) {
        if (rsv && bnc == 1) {  // absorbed by an outline: a zero-radiance candidate at the hit
          candPos = f3{org.x + wi.x * h.t, org.y + wi.y * h.t, org.z + wi.z * h.t};
          candN = neg(wi);
          candValid = true;
        }
        break;
      }
      if (rsv && bnc == 1) {
        candPos = v.P;
        candN = v.N;
        candValid = true;
      }
      float emW = 1.0f;
      if (emitNee && bnc == 1)
        emW = emissiveHitWeight(g.em, refKind(h.ref), refPrim(h.ref), org, wi, h.t, cand0Cos, h.Ng);
      L.x += thr.x * (v.rad.x + emW * v.emitted.x);
      L.y += thr.y * (v.rad.y + emW * v.emitted.y);
      L.z += thr.z * (v.rad.z + emW * v.emitted.z);
      if (bnc == maxB) break;
      thr.x *= v.alb.x;
      thr.y *= v.alb.y;
      thr.z *= v.alb.z;
      if (bnc >= 2) {
        tea2(s0, s1);
        float pc = fmaxf(thr.x, fmaxf(thr.y, thr.z));
        pc = fminf(0.95f, fmaxf(0.05f, pc));
        if (u32ToUnorm(s0) >= pc) break;
        const float inv = 1.0f / pc;
        thr.x *= inv;
        thr.y *= inv;
        thr.z *= inv;
      }
      tea2(s0, s1);
      const Frame3 fv = frameFromNormal(v.N);
      wi = cosineSampleHemisphere(u32ToUnorm(s0), u32ToUnorm(s1), fv);
      const float epsV = selfIntersectEps(v.P, wi, h.t);
      org = f3{v.P.x + v.N.x * epsV, v.P.y + v.N.y * epsV, v.P.z + v.N.z * epsV};
      tnear = epsV;
    }
    if (emitNee) {
      const f3 e = emissiveNee<KM>(g.em, s, P, N, Ng, tEps, s0, s1, ovf);
      ++nee;
      L.x += e.x;
      L.y += e.y;
      L.z += e.z;
    }
    if (g.clampLum > 0.0f) {
      const float lum = 0.2126f * L.x + 0.7152f * L.y + 0.0722f * L.z;
      if (lum > g.clampLum) {
        const float k = g.clampLum / lum;
        L.x *= k;
        L.y *= k;
        L.z *= k;
      }
    }
    if (rsv) {  // RIS weight pi * lum(L): p_hat = lum(L) cos over the cosine pdf
      float w = 0.0f, pHat = 0.0f;
      if (candValid && cand0Cos > 0.0f) {
        pHat = lumOf(L.x, L.y, L.z) * cand0Cos;
        w = lumOf(L.x, L.y, L.z) * kPiF;
      }
      tea2(rs0, rs1);
      rWSum += double(w);
      if (w > 0.0f && double(u32ToUnorm(rs0)) * rWSum <= double(w)) {
        rPos = candPos;
        rNrm = candN;
        rRad = L;
        rPHat = pHat;
      }
    }
    Esum.x += L.x;
    Esum.y += L.y;
    Esum.z += L.z;
    if (sI < spp / 2) {
      half.x += L.x;
      half.y += L.y;
      half.z += L.z;
    }
  }
  if (rsv) {  // W = wSum / (M p_hat(selected)), M = every candidate
    const float M = float(spp > 0 ? spp : 1);
    const float W = (rPHat > 0.0f && rWSum > 0.0) ? float(rWSum / (double(M) * double(rPHat))) : 0.0f;
    rsv[0] = make_float4(rPos.x, rPos.y, rPos.z, M);
    rsv[1] = make_float4(rNrm.x, rNrm.y, rNrm.z, W);
    rsv[2] = make_float4(rRad.x, rRad.y, rRad.z, 0.0f);
  }
  return make_float4(Esum.x, Esum.y, Esum.z, float(nOcc));
}

// gatherPt1Grid (pt1_gather.hpp:525-614): E and the hit fraction of every
// eligible point of a grid (or of the points a list names), seeded
// hashU32(pix ^ hashU32(pt1Seed)); the primary hit distance scales the
// origin epsilon.  Points not eligible get zero (grid form; a list names
// eligible points).  `listCount` (device) bounds the list when non-null.
// LANES neighbouring threads share one point, lane k taking its samples
// k, k + LANES, ...: a warp traces 32 / LANES points' sample fans from a few
// origins (coherent node fetches, as the AO rays of one hit), and a short
// list (the edge patch) still fills the GPU.  The lanes' sums meet in a
// shuffle tree, so E is the same mean summed in another order.
// point i of a grid in 2 x 2 quads (a warp's four points form one quad), the
// odd column and row in row order: a bijection on [0, W H)
UBR_D uint32_t quadPixel(uint32_t i, uint32_t W, uint32_t H) {
  const uint32_t fw = W & ~1u, fh = H & ~1u, nt = fw * fh;
  if (i < nt) {
    const uint32_t t = i >> 2, k = i & 3u, qx = fw >> 1;
    return ((t / qx) * 2u + (k >> 1)) * W + (t % qx) * 2u + (k & 1u);
  }
  uint32_t j = i - nt;
  const uint32_t rw = W - fw;
  if (j < rw * fh) return (j / rw) * W + fw + j % rw;
  j -= rw * fh;
  return fh * W + j;
}

// point i of a grid in 4 x 4 tiles of 2 x 2 quads (32 points, a warp of one
// thread per point, cover two adjacent tiles: an 8 x 4 block), the columns
// and rows past the last whole tile in row order: a bijection on [0, W H)
UBR_D uint32_t tilePixel4(uint32_t i, uint32_t W, uint32_t H) {
  const uint32_t fw = W & ~3u, fh = H & ~3u, nt = fw * fh;
  if (i < nt) {
    const uint32_t t = i >> 4, k = i & 15u, tx = fw >> 2;
    const uint32_t x = (t % tx) * 4u + ((k >> 1) & 2u) + (k & 1u);
    const uint32_t y = (t / tx) * 4u + ((k >> 2) & 2u) + ((k >> 1) & 1u);
    return y * W + x;
  }
  uint32_t j = i - nt;
  const uint32_t rw = W - fw;
  if (j < rw * fh) return (j / rw) * W + fw + j % rw;
  j -= rw * fh;
  return fh * W + j;
}

template <int KM, int LANES>
__global__ void __launch_bounds__(128, 8) k_gather(GiP g, DScene s, const LightD* lights, int nLights, GiGrid grid,
                                                const uint32_t* list, const uint32_t* listCount, uint32_t n, int spp,
                                                float4* E) {
  uint32_t rays = 0, nee = 0, ovf = 0;
  const uint32_t cnt = listCount ? min(n, *listCount) : n;
  const uint64_t total = uint64_t(cnt) * LANES, stride = uint64_t(gridDim.x) * blockDim.x;
  // grid-stride over (point, lane) pairs; a warp's lanes run the same
  // iterations, as the shuffles below need
  for (uint64_t t0 = uint64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31u); t0 < total; t0 += stride) {
    const uint64_t t = t0 + (threadIdx.x & 31u);
    const uint32_t i = uint32_t(t / LANES);
    const int lane = int(t % LANES);
    float4 e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    f3 half{0.0f, 0.0f, 0.0f};
    uint32_t pix = 0;
    if (i < cnt) {
      // several lanes per point: a warp's points form a quad; one thread per
      // point (the reservoir gather): its 32 points form an 8 x 4 block
      // (-15 % against quads along a row)
      pix = list                ? list[i]
            : LANES == 1        ? tilePixel4(i, uint32_t(grid.W), uint32_t(grid.H))
                                : quadPixel(i, uint32_t(grid.W), uint32_t(grid.H));
      const float4 ne = grid.ne[pix];
      if (ne.w != 0.0f) {
        const float4 pd = grid.pd[pix];
        const f3 N{ne.x, ne.y, ne.z};
        f3 Ng = N;
        if (grid.ng) {
          const float4 q = grid.ng[pix];
          Ng = f3{q.x, q.y, q.z};
        }
        const uint32_t seed = hashU32(pix ^ g.seedMix);
        const float tEps = pd.w > 0.0f ? pd.w : 1.0f;
        e = gatherPoint<KM>(g, s, lights, nLights, f3{pd.x, pd.y, pd.z}, N, Ng, tEps, seed, pix % uint32_t(grid.W),
                            pix / uint32_t(grid.W), spp, lane, LANES, half, rays, nee, ovf,
                            LANES == 1 && g.rsv ? g.rsv + size_t(kRsvF4) * pix : nullptr);
      }
    }
#pragma unroll
    for (int o = LANES / 2; o > 0; o >>= 1) {
      e.x += __shfl_xor_sync(0xFFFFFFFFu, e.x, o);
      e.y += __shfl_xor_sync(0xFFFFFFFFu, e.y, o);
      e.z += __shfl_xor_sync(0xFFFFFFFFu, e.z, o);
      e.w += __shfl_xor_sync(0xFFFFFFFFu, e.w, o);
      half.x += __shfl_xor_sync(0xFFFFFFFFu, half.x, o);
      half.y += __shfl_xor_sync(0xFFFFFFFFu, half.y, o);
      half.z += __shfl_xor_sync(0xFFFFFFFFu, half.z, o);
    }
    if (i < cnt && lane == 0) {
      const float invN = 1.0f / float(spp > 0 ? spp : 1);
      E[pix] = make_float4(e.x * invN, e.y * invN, e.z * invN, e.w * invN);
      if (g.halfE) {
        g.halfE[3 * size_t(pix)] = half.x;
        g.halfE[3 * size_t(pix) + 1] = half.y;
        g.halfE[3 * size_t(pix) + 2] = half.z;
      }
    }
  }
  warpCount(&g.stats[0], rays);
  warpCount(&g.stats[1], nee);
  warpCount(g.overflow, ovf);
}

// tracePt1GBuffer (pt1_gbuffer.hpp:83-196): one primary ray per point of a
// w x h grid over the same image plane as the render grid, closest hit in
// [0, inf) (no clip planes): position and ray distance, the face-forwarded
// shading normal (mesh: interpolated vertex normal; primitive: its geometric
// normal) with hit = 1, the face-forwarded geometric normal.  Outline
// primitives and misses are not gather points (zeros).
template <int KM>
__global__ void __launch_bounds__(128) k_gbuffer(Params p, DScene s, int w, int h, float4* pd, float4* ne,
                                                 float4* ng, unsigned long long* stats,
                                                 unsigned long long* overflow) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t traced = 0, ovf = 0;
  if (i < uint32_t(w) * uint32_t(h)) {
    const int px = int(i % uint32_t(w)), py = int(i / uint32_t(w));
    const float v = 1.0f - 2.0f * (float(py) + 0.5f) / float(h);
    const float u = 2.0f * (float(px) + 0.5f) / float(w) - 1.0f;
    f3 org, rd;
    if (p.ortho) {
      org = p.camPos + p.right * (u * p.halfW) + p.up * (v * p.halfH);
      rd = p.camDir;
    } else {
      org = p.camPos;
      rd = normalize(p.camDir + p.right * (u * p.persHalfW) + p.up * (v * p.persHalfH));
    }
    Ray r{org, rd, 0.0f, kInfF};
    Hit hh;
    Count cnt;
    traverse<false, KM>(travOf(s), r, hh, ovf, &cnt, false);
    traced = 1;
    float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), b = a, c = a;
    if (hh.ref != kInvalid) {
      const int kind = refKind(hh.ref);
      const uint32_t prim = refPrim(hh.ref);
      bool ok = true;
      f3 N, Ng;
      if (kind == kMesh) {
        const uint32_t i0 = __ldg(&s.meshIdx[3 * prim]), i1 = __ldg(&s.meshIdx[3 * prim + 1]),
                       i2 = __ldg(&s.meshIdx[3 * prim + 2]);
        const float w0 = 1.0f - hh.u - hh.v;
        float nb[3];
        for (int k = 0; k < 3; ++k)
          nb[k] = w0 * __ldg(&s.meshNrm[3 * i0 + k]) + hh.u * __ldg(&s.meshNrm[3 * i1 + k]) +
                  hh.v * __ldg(&s.meshNrm[3 * i2 + k]);
        N = safeNormalize(f3{nb[0], nb[1], nb[2]});
        Ng = safeNormalize(hh.Ng);
      } else {
        ok = __ldg(&s.primFromEdge[kind][prim]) == 0;
        N = safeNormalize(hh.Ng);
        Ng = N;
      }
      if (ok) {
        if (dot(N, rd) > 0.0f) N = neg(N);
        if (dot(Ng, rd) > 0.0f) Ng = neg(Ng);
        a = make_float4(org.x + rd.x * hh.t, org.y + rd.y * hh.t, org.z + rd.z * hh.t, hh.t);
        b = make_float4(N.x, N.y, N.z, 1.0f);
        c = make_float4(Ng.x, Ng.y, Ng.z, 0.0f);
      }
    }
    pd[i] = a;
    ne[i] = b;
    ng[i] = c;
  }
  warpCount(&stats[2], traced);
  warpCount(overflow, ovf);
}

// ---- denoisePt1E (pt1_denoise.cpp:20-80): the a-trous filter of
// denoise_atrous.cpp:27-220 on E at gather resolution, normal and position
// guides, no albedo demodulation (E is irradiance) ----
constexpr float kDnEps = 1.0e-3f;

// non-finite E scrubbed to 0; a point is valid when its normal is unit-length
__global__ void k_gdn_init(uint32_t n, float4* E, const float4* ne, uint8_t* valid, float4* irr) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  float4 e = E[p];
  if (!isfinite(e.x)) e.x = 0.0f;
  if (!isfinite(e.y)) e.y = 0.0f;
  if (!isfinite(e.z)) e.z = 0.0f;
  E[p] = e;
  irr[p] = e;
  const float4 q = ne[p];
  valid[p] = (q.x * q.x + q.y * q.y + q.z * q.z) > 0.25f ? 1 : 0;
}

// per valid point: the largest distance to a valid 4-neighbour's position
// (floor kDnEps) and the luminance variance over the valid 3x3 neighbourhood
__global__ void k_gdn_aux(int W, int H, const uint8_t* valid, const float4* irr, const float4* pd, float* var,
                          float* pgrad) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= uint32_t(W) * uint32_t(H)) return;
  float v = 0.0f, gr = kDnEps;
  if (valid[p]) {
    const int x = int(p % uint32_t(W)), y = int(p / uint32_t(W));
    const float4 pp = pd[p];
    const int nb[4][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}};
    for (int k = 0; k < 4; ++k) {
      const int qx = x + nb[k][0], qy = y + nb[k][1];
      if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
      const size_t q = size_t(qy) * W + qx;
      if (!valid[q]) continue;
      const float4 pq = pd[q];
      const float dx = pp.x - pq.x, dy = pp.y - pq.y, dz = pp.z - pq.z;
      gr = fmaxf(gr, sqrtf(dx * dx + dy * dy + dz * dz));
    }
    float sm = 0.0f, s2 = 0.0f;
    int n = 0;
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int qx = x + dx, qy = y + dy;
        if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
        const size_t q = size_t(qy) * W + qx;
        if (!valid[q]) continue;
        const float4 c = irr[q];
        const float l = lumOf(c.x, c.y, c.z);
        sm += l;
        s2 += l * l;
        ++n;
      }
    if (n > 0) {
      const float mean = sm / float(n);
      v = fmaxf(0.0f, s2 / float(n) - mean * mean);
    }
  }
  var[p] = v;
  pgrad[p] = gr;
}

// one iteration: 5x5 B3 taps at 2^it spacing with the normal^sigmaN,
// exp(-|dP| / (sigmaZ grad step + eps)) and exp(-|dl| / (sigmaL sqrt(var) +
// eps)) edge-stops, in the reference's weight order
__global__ void k_gdn_iter(int W, int H, int step, const uint8_t* valid, const float4* ne, const float4* pd,
                           const float4* irr, const float* var, const float* pgrad, float sigmaN, float sigmaZ,
                           float sigmaL, float4* next) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= uint32_t(W) * uint32_t(H)) return;
  const float4 ip = irr[p];
  if (!valid[p]) {
    next[p] = ip;
    return;
  }
  const float h5[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
  const int x = int(p % uint32_t(W)), y = int(p / uint32_t(W));
  const float4 n4 = ne[p], p4 = pd[p];
  const f3 np{n4.x, n4.y, n4.z}, pp{p4.x, p4.y, p4.z};
  const float lp = lumOf(ip.x, ip.y, ip.z);
  const float lDenom = sigmaL * sqrtf(var[p]) + kDnEps;
  const float zDenom = sigmaZ * pgrad[p] * float(step) + kDnEps;
  float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f, wsum = 0.0f;
  for (int dy = -2; dy <= 2; ++dy) {
    const int qy = y + dy * step;
    if (qy < 0 || qy >= H) continue;
    for (int dx = -2; dx <= 2; ++dx) {
      const int qx = x + dx * step;
      if (qx < 0 || qx >= W) continue;
      const size_t q = size_t(qy) * W + qx;
      if (!valid[q]) continue;
      float w = h5[dx + 2] * h5[dy + 2];
      const float4 nq = ne[q], pq = pd[q], iq = irr[q];
      const float nd = fmaxf(0.0f, np.x * nq.x + np.y * nq.y + np.z * nq.z);
      w *= powf(nd, sigmaN);
      const float ddx = pp.x - pq.x, ddy = pp.y - pq.y, ddz = pp.z - pq.z;
      w *= expf(-sqrtf(ddx * ddx + ddy * ddy + ddz * ddz) / zDenom);
      w *= expf(-fabsf(lp - lumOf(iq.x, iq.y, iq.z)) / lDenom);
      s0 += w * iq.x;
      s1 += w * iq.y;
      s2 += w * iq.z;
      wsum += w;
    }
  }
  next[p] = wsum > 0.0f ? make_float4(s0 / wsum, s1 / wsum, s2 / wsum, ip.w) : ip;
}

__global__ void k_gdn_write(uint32_t n, const uint8_t* valid, const float4* irr, float4* E) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n || !valid[p]) return;
  const float4 v = irr[p];
  E[p] = make_float4(fmaxf(0.0f, v.x), fmaxf(0.0f, v.y), fmaxf(0.0f, v.z), E[p].w);
}

// upsampleJointBilateral (pt1_upsample.hpp:40-199): E (and the hit fraction)
// of every eligible render-grid pixel from the 2x2 gather-grid points around
// its centre, weighted bilinear x max(0, N.Nh)^normalPow x
// exp(-|z - zh| / (depthScale z + 1e-6)); when every weight dies, the
// nearest valid point of the quad, then (coarse grids, fallbackR > 0) the
// nearest valid point of the (2r)^2 window.  With the edge patch on, pixels
// whose weights died or summed below patchThresh are appended to the patch
// list.  Pixels not eligible get zero.
__global__ void k_upsample(int W, int H, const float4* fpd, const float4* fne, GiGrid lo, const float4* Elo,
                           float normalPow, float depthScale, int fallbackR, int patchOn, float patchThresh,
                           float4* E, uint8_t* patchFlag, unsigned long long* holes) {
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  bool patch = false, hole = false;
  if (pix < uint32_t(W) * uint32_t(H)) {
    const float4 nf4 = fne[pix];
    float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (nf4.w != 0.0f) {
      const int px = int(pix % uint32_t(W)), py = int(pix / uint32_t(W));
      const int hw = lo.W, hh = lo.H;
      const float sy = (float(py) + 0.5f) * float(hh) / float(H) - 0.5f;
      const int by = int(floorf(sy));
      const float fy = sy - float(by);
      const float sx = (float(px) + 0.5f) * float(hw) / float(W) - 0.5f;
      const int bx = int(floorf(sx));
      const float fx = sx - float(bx);
      const f3 Nf{nf4.x, nf4.y, nf4.z};
      const float zf = fpd[pix].w;
      float wSum = 0.0f, e0 = 0.0f, e1 = 0.0f, e2 = 0.0f, oS = 0.0f, bestBilin = -1.0f;
      int bestPix = -1;
      for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
          const int hx = min(max(bx + dx, 0), hw - 1), hy = min(max(by + dy, 0), hh - 1);
          const int hp = hy * hw + hx;
          const float4 nh = lo.ne[hp];
          if (nh.w == 0.0f) continue;
          const float wb = (dx ? fx : 1.0f - fx) * (dy ? fy : 1.0f - fy);
          if (wb > bestBilin) {
            bestBilin = wb;
            bestPix = hp;
          }
          const float wn = powf(fmaxf(0.0f, Nf.x * nh.x + Nf.y * nh.y + Nf.z * nh.z), normalPow);
          const float zh = lo.pd[hp].w;
          const float wz = expf(-fabsf(zf - zh) / (depthScale * zf + 1e-6f));
          const float w = wb * wn * wz;
          const float4 eh = Elo[hp];
          wSum += w;
          e0 += w * eh.x;
          e1 += w * eh.y;
          e2 += w * eh.z;
          oS += w * eh.w;
        }
      if (wSum >= 1e-6f) {
        patch = wSum < patchThresh;
        const float inv = 1.0f / wSum;
        out = make_float4(e0 * inv, e1 * inv, e2 * inv, oS * inv);
      } else if (bestPix >= 0) {
        patch = true;
        out = Elo[bestPix];
      } else {
        patch = true;
        int found = -1;
        if (fallbackR > 0) {
          float bestD2 = 1e30f;
          for (int wy = by - fallbackR + 1; wy <= by + fallbackR; ++wy) {
            if (wy < 0 || wy >= hh) continue;
            for (int wx = bx - fallbackR + 1; wx <= bx + fallbackR; ++wx) {
              if (wx < 0 || wx >= hw) continue;
              const int hp = wy * hw + wx;
              if (lo.ne[hp].w == 0.0f) continue;
              const float ddx = float(wx) - sx, ddy = float(wy) - sy;
              const float d2 = ddx * ddx + ddy * ddy;
              if (d2 < bestD2) {
                bestD2 = d2;
                found = hp;
              }
            }
          }
        }
        if (found >= 0) out = Elo[found];
        else hole = true;
      }
      patch = patch && patchOn;
    }
    E[pix] = out;
    if (patchFlag) patchFlag[pix] = patch ? 1 : 0;
  }
  warpCount(holes, hole ? 1u : 0u);
}

// smoothPatchedPixels (pt1_upsample.hpp:214-248): each listed pixel's E
// becomes the guide-weighted mean of its (2r+1)^2 eligible neighbourhood in
// the snapshot (itself at weight 1; neighbour weights below 1e-4 dropped).
__global__ void k_smooth(int W, int H, const uint32_t* list, const uint32_t* count, uint32_t n, const float4* fpd,
                         const float4* fne, float normalPow, float depthScale, int radius, const float4* Esrc,
                         float4* E) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= min(n, *count)) return;
  const uint32_t pix = list[i];
  const int px = int(pix % uint32_t(W)), py = int(pix / uint32_t(W));
  const float4 nf = fne[pix];
  const float zf = fpd[pix].w;
  const float4 e = Esrc[pix];
  float wSum = 1.0f, e0 = e.x, e1 = e.y, e2 = e.z, oS = e.w;
  for (int dy = -radius; dy <= radius; ++dy) {
    const int ny = py + dy;
    if (ny < 0 || ny >= H) continue;
    for (int dx = -radius; dx <= radius; ++dx) {
      if (dx == 0 && dy == 0) continue;
      const int nx = px + dx;
      if (nx < 0 || nx >= W) continue;
      const size_t q = size_t(ny) * W + nx;
      const float4 nn = fne[q];
      if (nn.w == 0.0f) continue;
      const float wn = powf(fmaxf(0.0f, nf.x * nn.x + nf.y * nn.y + nf.z * nn.z), normalPow);
      const float zn = fpd[q].w;
      const float wz = expf(-fabsf(zf - zn) / (depthScale * zf + 1e-6f));
      const float w = wn * wz;
      if (w < 1e-4f) continue;
      const float4 eq = Esrc[q];
      wSum += w;
      e0 += w * eq.x;
      e1 += w * eq.y;
      e2 += w * eq.z;
      oS += w * eq.w;
    }
  }
  const float inv = 1.0f / wSum;
  E[pix] = make_float4(e0 * inv, e1 * inv, e2 * inv, oS * inv);
}

// The [E] composite (embree_renderer.cpp:908-927): every eligible pixel adds
// giIntensity * (kd * pigment) * E.
__global__ void k_composite(uint32_t n, const float4* ne, const float4* refl, const float4* E, float gI,
                            float4* color) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n || ne[p].w == 0.0f) return;
  const float4 rf = refl[p], e = E[p];
  float4 c = color[p];
  c.x += gI * rf.x * e.x;
  c.y += gI * rf.y * e.y;
  c.z += gI * rf.z * e.z;
  color[p] = c;
}

// ---- pt2 adaptive spp (pt2_adaptive.hpp:30-121) ----
// error = |lum(E) - lum(halfSum) / (spp/2)| against threshold x sqrt(lum)
// (dark) or lum; spp < 2 marks every eligible point
__global__ void k_adapt_mask(int W, int H, const float4* E, const float* halfE, const float4* ne, int spp,
                             float threshold, uint8_t* mask) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= uint32_t(W) * uint32_t(H)) return;
  uint8_t m = 0;
  if (ne[p].w != 0.0f) {
    const int nHalf = spp / 2;
    if (nHalf < 1) {
      m = 1;
    } else {
      const float invHalf = 1.0f / float(nHalf);
      const float4 e = E[p];
      const float lumA = 0.2126f * e.x + 0.7152f * e.y + 0.0722f * e.z;
      const float lumH = (0.2126f * halfE[3 * size_t(p)] + 0.7152f * halfE[3 * size_t(p) + 1] +
                          0.0722f * halfE[3 * size_t(p) + 2]) *
                         invHalf;
      const float diff = fabsf(lumA - lumH);
      const float norm = lumA < 1.0f ? sqrtf(fmaxf(lumA, 1.0e-4f)) : lumA;
      m = diff > threshold * norm ? 1 : 0;
    }
  }
  mask[p] = m;
}

// 3x3 dilation over the eligible points
__global__ void k_dilate(int W, int H, const uint8_t* in, const float4* ne, uint8_t* out) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= uint32_t(W) * uint32_t(H)) return;
  uint8_t v = 0;
  if (ne[p].w != 0.0f) {
    const int px = int(p % uint32_t(W)), py = int(p / uint32_t(W));
    v = in[p];
    for (int dy = -1; dy <= 1 && !v; ++dy) {
      const int ny = py + dy;
      if (ny < 0 || ny >= H) continue;
      for (int dx = -1; dx <= 1 && !v; ++dx) {
        const int nx = px + dx;
        if (nx < 0 || nx >= W) continue;
        v = in[size_t(ny) * W + nx];
      }
    }
  }
  out[p] = v;
}

__global__ void k_mask_list(uint32_t n, const uint8_t* mask, uint32_t* list, uint32_t* count) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  const bool on = p < n && mask[p];
  int off;
  const int base = warpPushBase(on, count, off);
  if (on) list[base + off] = p;
}

// E = E * spp / (spp + extra) + Er * (1 - that) on the listed points
__global__ void k_merge(const uint32_t* list, const uint32_t* count, uint32_t n, int spp, int extra,
                        const float4* Er, float4* E) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= min(n, *count)) return;
  const uint32_t p = list[i];
  const float wB = float(spp) / float(spp + extra);
  const float wR = 1.0f - wB;
  const float4 e = E[p], r = Er[p];
  E[p] = make_float4(e.x * wB + r.x * wR, e.y * wB + r.y * wR, e.z * wB + r.z * wR, e.w * wB + r.w * wR);
}

// ---- pt2 ReSTIR spatial resampling (pt2_reservoir.hpp, pt2_spatial.hpp) ----
// pt2_sampler.hpp:71-78 pt2HashHp
UBR_D uint32_t hashHp(uint32_t i) {
  i ^= i >> 16;
  i *= 0x21f0aaadu;
  i ^= i >> 15;
  i *= 0xd35a2d97u;
  i ^= i >> 15;
  return i ^ 0xe6fe3bebu;
}
// pt2TargetPdf (pt2_reservoir.hpp:55-63): luminance times the receiver cosine
UBR_D float targetPdf(f3 P, f3 N, f3 sp, f3 rad) {
  const f3 d{sp.x - P.x, sp.y - P.y, sp.z - P.z};
  const float l2 = dot(d, d);
  if (l2 <= 0.0f) return 0.0f;
  const float c = dot(N, d) / sqrtf(l2);
  if (c <= 0.0f) return 0.0f;
  return lumOf(rad.x, rad.y, rad.z) * c;
}
// pt2Jacobian (pt2_reservoir.hpp:72-89): reconnection Jacobian of moving a
// sample's receiver, cosines at the sample normal, clamped to [0, cap]
UBR_D float reconnectJacobian(f3 recvNew, f3 recvOld, f3 sp, f3 sn, float cap) {
  const f3 a{recvNew.x - sp.x, recvNew.y - sp.y, recvNew.z - sp.z};
  const f3 b{recvOld.x - sp.x, recvOld.y - sp.y, recvOld.z - sp.z};
  const float ra2 = dot(a, a), rb2 = dot(b, b);
  if (ra2 <= 0.0f || rb2 <= 0.0f) return 0.0f;
  const float ca = dot(sn, a) / sqrtf(ra2);
  const float cb = dot(sn, b) / sqrtf(rb2);
  if (ca <= 0.0f || cb <= 0.0f) return 0.0f;
  const float j = (rb2 * ca) / (ra2 * cb);
  if (!isfinite(j) || j < 0.0f) return 0.0f;
  return j > cap ? cap : j;
}

// pt2SpatialRound (pt2_spatial.hpp:66-271), one thread per grid point: the
// point restarts from its own previous-round reservoir and streams in K
// neighbours (8 in round 0, then 5) on a golden-angle spiral rotated per
// point, radius halving per round (floor 3), skipping incompatible normals
// (< 0.5), depths (> 10 %), empty reservoirs and samples nearer than 4x the
// receiver spacing; the selection rule runs in double as the reference's
// wSum does.  W is normalised by the balance-heuristic mixture over the
// contributors; with `unbiased` a contributor that cannot see the selected
// sample counts zero (one any-hit ray each).  The last round writes E.xyz as
// the balance-MIS sum over every contributor's sample.
struct RsvView {
  f3 pos, nrm, rad;
  float M, W;
};
UBR_D RsvView loadRsv(const float4* r, uint32_t q) {
  const float4 a = r[size_t(kRsvF4) * q], b = r[size_t(kRsvF4) * q + 1], c = r[size_t(kRsvF4) * q + 2];
  return RsvView{f3{a.x, a.y, a.z}, f3{b.x, b.y, b.z}, f3{c.x, c.y, c.z}, a.w, b.w};
}

template <int KM>
__global__ void __launch_bounds__(128) k_spatial(GiSpatial sp, DScene sc, GiGrid grid, const float4* in,
                                                 float4* out, int round, float4* E, unsigned long long* overflow) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t n = uint32_t(grid.W) * uint32_t(grid.H);
  uint32_t ovf = 0;
  if (i < n) {
    // a warp's points form an 8 x 4 block (their neighbours overlap)
    const uint32_t pix = tilePixel4(i, uint32_t(grid.W), uint32_t(grid.H));
    const float4 ne = grid.ne[pix];
    float4* o = out + size_t(kRsvF4) * pix;
    if (ne.w == 0.0f) {
      o[0] = o[1] = o[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    } else {
      const int W = grid.W, H = grid.H, px = int(pix % uint32_t(W)), py = int(pix / uint32_t(W));
      const int K = round == 0 ? 8 : 5;
      float radius = sp.radius / float(1 << round);
      if (radius < 3.0f) radius = 3.0f;
      const uint32_t salt = hashHp(sp.seedMix ^ (0x53504154u + uint32_t(round)));
      const float4 pd = grid.pd[pix];
      const f3 P{pd.x, pd.y, pd.z}, N{ne.x, ne.y, ne.z};
      const float d0 = pd.w;
      uint32_t s0 = hashHp(pix ^ salt), s1 = 0x52535452u;
      f3 dPos{0.0f, 0.0f, 0.0f}, dNrm{0.0f, 0.0f, 0.0f}, dRad{0.0f, 0.0f, 0.0f};
      double wSum = 0.0;
      float Mtot = 0.0f;
      // contributors: receiver geometry and the sample each one offered
      f3 cPos[9], cN[9], sPos[9], sRad[9];
      float cM[9], sW[9], sJ[9];
      int nc = 0;
      {
        const RsvView own = loadRsv(in, pix);
        const float m = own.M > sp.mCap ? sp.mCap : own.M;
        const float w = targetPdf(P, N, own.pos, own.rad) * own.W * m;
        tea2(s0, s1);
        wSum += double(w);
        Mtot += m;
        if (w > 0.0f && double(u32ToUnorm(s0)) * wSum <= double(w)) {
          dPos = own.pos;
          dNrm = own.nrm;
          dRad = own.rad;
        }
        cPos[0] = P;
        cN[0] = N;
        cM[0] = m;
        sPos[0] = own.pos;
        sRad[0] = own.rad;
        sW[0] = own.W;
        sJ[0] = 1.0f;
        nc = 1;
      }
      tea2(s0, s1);
      const float rot = u32ToUnorm(s0) * 6.2831853f;
      for (int k = 0; k < K; ++k) {
        const float ang = rot + float(k) * 2.399963230f;
        const float rr = sqrtf((float(k) + 0.5f) / float(K)) * radius;
        const int nx = px + int(lroundf(cosf(ang) * rr));
        const int ny = py + int(lroundf(sinf(ang) * rr));
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        const uint32_t q = uint32_t(ny) * uint32_t(W) + uint32_t(nx);
        if (q == pix) continue;
        const float4 nq = grid.ne[q];
        if (nq.w == 0.0f) continue;
        const f3 Nn{nq.x, nq.y, nq.z};
        if (dot(N, Nn) < 0.5f) continue;
        const float4 pq4 = grid.pd[q];
        if (fabsf(d0 - pq4.w) > 0.1f * d0) continue;
        const RsvView nb = loadRsv(in, q);
        if (nb.M <= 0.0f) continue;
        const f3 Pn{pq4.x, pq4.y, pq4.z};
        const f3 dq{Pn.x - P.x, Pn.y - P.y, Pn.z - P.z};
        const f3 ds{nb.pos.x - Pn.x, nb.pos.y - Pn.y, nb.pos.z - Pn.z};
        if (dot(ds, ds) < 4.0f * 4.0f * dot(dq, dq)) continue;
        const float j = reconnectJacobian(P, Pn, nb.pos, nb.nrm, 10.0f);
        const float m = nb.M > sp.mCap ? sp.mCap : nb.M;
        const float w = targetPdf(P, N, nb.pos, nb.rad) * nb.W * m * j;
        tea2(s0, s1);
        wSum += double(w);
        Mtot += m;
        if (w > 0.0f && double(u32ToUnorm(s0)) * wSum <= double(w)) {
          dPos = nb.pos;
          dNrm = nb.nrm;
          dRad = nb.rad;
        }
        cPos[nc] = Pn;
        cN[nc] = Nn;
        cM[nc] = m;
        sPos[nc] = nb.pos;
        sRad[nc] = nb.rad;
        sW[nc] = nb.W;
        sJ[nc] = j;
        ++nc;
      }
      // W by the balance-heuristic mixture over the contributors
      float piSum = 0.0f;
      if (wSum > 0.0) {
        const TravScene ts = travOf(sc);
        for (int k = 0; k < nc; ++k) {
          float pk = targetPdf(cPos[k], cN[k], dPos, dRad);
          if (pk <= 0.0f) continue;
          if (sp.unbiased) {
            const f3 toS{dPos.x - cPos[k].x, dPos.y - cPos[k].y, dPos.z - cPos[k].z};
            const float dist2 = dot(toS, toS);
            if (dist2 <= 0.0f) continue;
            const float dist = sqrtf(dist2);
            const f3 dir{toS.x / dist, toS.y / dist, toS.z / dist};
            if (dot(cN[k], dir) <= 0.0f) {
              pk = 0.0f;
            } else {
              const float eps = selfIntersectEps(cPos[k], dir, dist);
              const f3 O{cPos[k].x + cN[k].x * eps, cPos[k].y + cN[k].y * eps, cPos[k].z + cN[k].z * eps};
              Ray r{O, dir, eps, dist - 2.0f * eps};
              Hit hh;
              Count cnt;
              if (traverse<false, KM, true>(ts, r, hh, ovf, &cnt, true)) pk = 0.0f;
            }
          }
          piSum += pk * cM[k];
        }
      }
      float Wn = 0.0f;
      if (piSum > 0.0f && wSum > 0.0) Wn = float(wSum) / piSum;
      const float Wd = (sp.wClamp > 0.0f && Wn > sp.wClamp) ? sp.wClamp : Wn;
      const float Md = Mtot > sp.mCap ? sp.mCap : Mtot;
      o[0] = make_float4(dPos.x, dPos.y, dPos.z, Md);
      o[1] = make_float4(dNrm.x, dNrm.y, dNrm.z, Wd);
      o[2] = make_float4(dRad.x, dRad.y, dRad.z, 0.0f);
      if (E) {  // last round: every contributor's sample under balance MIS
        f3 e{0.0f, 0.0f, 0.0f};
        for (int k = 0; k < nc; ++k) {
          if (sW[k] <= 0.0f || sJ[k] <= 0.0f) continue;
          const float pq = targetPdf(P, N, sPos[k], sRad[k]);
          if (pq <= 0.0f) continue;
          float denom = 0.0f;
          for (int j2 = 0; j2 < nc; ++j2) denom += cM[j2] * targetPdf(cPos[j2], cN[j2], sPos[k], sRad[k]);
          if (denom <= 0.0f) continue;
          const float mis = cM[k] * pq / denom;
          const float l = lumOf(sRad[k].x, sRad[k].y, sRad[k].z);
          if (l <= 0.0f) continue;
          const float g = mis * sW[k] * sJ[k] * (pq / l) * (1.0f / kPiF);
          e.x += sRad[k].x * g;
          e.y += sRad[k].y * g;
          e.z += sRad[k].z * g;
        }
        const float4 e0 = E[pix];
        E[pix] = make_float4(e.x, e.y, e.z, e0.w);
      }
    }
  }
  warpCount(overflow, ovf);
}

// ---- pt2 traced reflection (pt2_reflect.hpp, pt2_glossy.hpp) ----
UBR_D f3 schlickF3(f3 F0, float u) {
  float c = 1.0f - u;
  if (c < 0.0f) c = 0.0f;
  if (c > 1.0f) c = 1.0f;
  const float c5 = c * c * c * c * c;
  return f3{F0.x + (1.0f - F0.x) * c5, F0.y + (1.0f - F0.y) * c5, F0.z + (1.0f - F0.z) * c5};
}

// incident direction of the primary ray that reached P
UBR_D f3 incident(const GiCam& cam, f3 P) {
  return cam.ortho ? cam.dir : safeNormalize(f3{P.x - cam.pos.x, P.y - cam.pos.y, P.z - cam.pos.z});
}

// radiance along a reflected ray (origin O, direction d): at a hit its
// NEE direct + albedo x sky (one-bounce ambient cut), the sky on a miss
template <int KM>
UBR_D f3 reflectedRadiance(const GiP& g, const DScene& s, const LightD* lights, int nLights, f3 O, f3 d, float tn,
                           uint32_t r0, uint32_t r1, uint32_t& rays, uint32_t& nee, uint32_t& ovf) {
  Ray r{O, d, tn, kInfF};
  Hit h;
  Count cnt;
  traverse<false, KM>(travOf(s), r, h, ovf, &cnt, false);
  ++rays;
  if (h.ref == kInvalid) return giEnvironment(g, d);
  tea2(r0, r1);
  Vertex v;
  if (!evalVertex<KM>(s, lights, nLights, h, O, d, g.emissive != 0, &r0, &r1, v, nee, ovf))
    return f3{0.0f, 0.0f, 0.0f};
  const f3 sky = giEnvironment(g, d);
  return f3{v.rad.x + v.alb.x * sky.x, v.rad.y + v.alb.y * sky.y, v.rad.z + v.alb.z * sky.z};
}

// pt2ReflectPass: one mirror ray per pixel whose first hit is reflective
// with a mirror lobe; colour += reflection x Schlick(F0, cos) x L.
template <int KM>
__global__ void __launch_bounds__(128) k_reflect(GiP g, DScene s, const LightD* lights, int nLights, GiGrid full,
                                                 ReflD rf, GiCam cam, uint32_t n, float4* color) {
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t rays = 0, nee = 0, ovf = 0;
  if (pix < n) {
    const float4 a = rf.amt[pix];
    if (a.x > 0.0f && !(a.y > 0.0f)) {
      const float4 pd = full.pd[pix], ne = full.ne[pix];
      const f3 P{pd.x, pd.y, pd.z}, N{ne.x, ne.y, ne.z};
      const f3 wi = incident(cam, P);
      const float indot = dot(wi, N);
      const f3 rdir = safeNormalize(f3{wi.x - 2.0f * indot * N.x, wi.y - 2.0f * indot * N.y,
                                       wi.z - 2.0f * indot * N.z});
      const float t0 = pd.w > 0.0f ? pd.w : 1.0f;
      const float eps = selfIntersectEps(P, rdir, t0);
      const f3 O{P.x + N.x * eps, P.y + N.y * eps, P.z + N.z * eps};
      const f3 L = reflectedRadiance<KM>(g, s, lights, nLights, O, rdir, eps, pix ^ 0x52464c54u, 0x4e454531u, rays,
                                         nee, ovf);
      float cosI = -indot;
      if (cosI < 0.0f) cosI = 0.0f;
      if (cosI > 1.0f) cosI = 1.0f;
      const float4 f0 = rf.f0[pix];
      const f3 F = schlickF3(f3{f0.x, f0.y, f0.z}, cosI);
      float4 c = color[pix];
      c.x += a.x * F.x * L.x;
      c.y += a.x * F.y * L.y;
      c.z += a.x * F.z * L.z;
      color[pix] = c;
    }
  }
  warpCount(&g.stats[0], rays);
  warpCount(&g.stats[1], nee);
  warpCount(g.overflow, ovf);
}

// Smith Lambda of GGX, isotropic and anisotropic (pt2_glossy.hpp:41-56)
UBR_D float ggxLambdaIso(float alpha, float cosT) {
  const float c2 = fmaxf(cosT * cosT, 1.0e-12f);
  const float t2 = (1.0f - c2) / c2;
  return 0.5f * (sqrtf(1.0f + alpha * alpha * t2) - 1.0f);
}
UBR_D float ggxLambdaAn(float ax, float ay, f3 w) {
  const float z2 = fmaxf(w.z * w.z, 1.0e-12f);
  const float t2 = (ax * ax * w.x * w.x + ay * ay * w.y * w.y) / z2;
  return 0.5f * (sqrtf(1.0f + t2) - 1.0f);
}
// GGX visible-normal sampling (Heitz, "Sampling the GGX Distribution of
// Visible Normals", JCGT 7(4) 2018) for view wo in the local frame
UBR_D f3 sampleGgxVndf(f3 wo, float ax, float ay, float u1, float u2) {
  const f3 Vh = safeNormalize(f3{ax * wo.x, ay * wo.y, wo.z});
  const f3 T1 = Vh.z < 0.999f ? safeNormalize(cross(f3{0.0f, 0.0f, 1.0f}, Vh)) : f3{1.0f, 0.0f, 0.0f};
  const f3 T2 = cross(Vh, T1);
  const float r = sqrtf(u1);
  const float phi = 2.0f * kPiF * u2;
  const float t1 = r * cosf(phi);
  float t2 = r * sinf(phi);
  const float s = 0.5f * (1.0f + Vh.z);
  t2 = (1.0f - s) * sqrtf(fmaxf(0.0f, 1.0f - t1 * t1)) + s * t2;
  const float t3 = sqrtf(fmaxf(0.0f, 1.0f - t1 * t1 - t2 * t2));
  const f3 Nh{t1 * T1.x + t2 * T2.x + t3 * Vh.x, t1 * T1.y + t2 * T2.y + t3 * Vh.y,
              t1 * T1.z + t2 * T2.z + t3 * Vh.z};
  return safeNormalize(f3{ax * Nh.x, ay * Nh.y, fmaxf(0.0f, Nh.z)});
}

// pt2GlossyPass: spp VNDF-sampled reflection rays per glossy pixel (alpha >
// 0), each weighted G2/G1(wo) x Schlick(F0, wo.wm), mean into Espec (zero
// elsewhere).  Per-pixel Sobol stream hashU32(pix) ^ hashU32(seed ^ 'GLSY').
template <int KM>
__global__ void __launch_bounds__(128) k_glossy(GiP g, DScene s, const LightD* lights, int nLights, GiGrid full,
                                                ReflD rf, GiCam cam, uint32_t n, int spp, uint32_t seedMix,
                                                float4* Espec) {
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t rays = 0, nee = 0, ovf = 0;
  if (pix < n) {
    const float4 a = rf.amt[pix];
    f3 sum{0.0f, 0.0f, 0.0f};
    if (a.x > 0.0f && a.y > 0.0f) {
      const float alpha = a.y;
      const float4 pd = full.pd[pix], ne = full.ne[pix];
      const f3 P{pd.x, pd.y, pd.z}, N{ne.x, ne.y, ne.z};
      const f3 wiV = incident(cam, P);
      bool aniso = false;
      float ax = alpha, ay = alpha;
      Frame3 f;
      if (rf.tan) {
        const float4 t4 = rf.tan[pix];
        const f3 T{t4.x, t4.y, t4.z};
        const float aspect = a.z;
        if (aspect != 1.0f && dot(T, T) > 0.5f) {
          aniso = true;
          f.t = T;
          f.b = cross(N, T);
          f.n = N;
          ax = alpha / aspect;
          if (ax > 1.0f) ax = 1.0f;
          ay = alpha * aspect;
        }
      }
      if (!aniso) f = frameFromNormal(N);
      const f3 woW{-wiV.x, -wiV.y, -wiV.z};
      f3 wo{dot(woW, f.t), dot(woW, f.b), dot(woW, f.n)};
      if (wo.z < 1.0e-4f) wo.z = 1.0e-4f;
      wo = safeNormalize(wo);
      const float lamO = aniso ? ggxLambdaAn(ax, ay, wo) : ggxLambdaIso(alpha, wo.z);
      const float t0 = pd.w > 0.0f ? pd.w : 1.0f;
      const uint32_t seedPix = hashU32(pix) ^ seedMix;
      const float4 f04 = rf.f0[pix];
      const f3 F0{f04.x, f04.y, f04.z};
      for (int sI = 0; sI < spp; ++sI) {
        float u1, u2;
        sobol2D(uint32_t(sI), seedPix, u1, u2);
        const f3 wm = sampleGgxVndf(wo, ax, ay, u1, u2);
        const float owm = dot(wo, wm);
        const f3 wl{2.0f * owm * wm.x - wo.x, 2.0f * owm * wm.y - wo.y, 2.0f * owm * wm.z - wo.z};
        if (wl.z <= 0.0f) continue;
        const float lamI = aniso ? ggxLambdaAn(ax, ay, wl) : ggxLambdaIso(alpha, wl.z);
        const float weight = (1.0f + lamO) / (1.0f + lamO + lamI);
        const f3 rdir = safeNormalize(f3{f.t.x * wl.x + f.b.x * wl.y + f.n.x * wl.z,
                                         f.t.y * wl.x + f.b.y * wl.y + f.n.y * wl.z,
                                         f.t.z * wl.x + f.b.z * wl.y + f.n.z * wl.z});
        const float eps = selfIntersectEps(P, rdir, t0);
        const f3 O{P.x + N.x * eps, P.y + N.y * eps, P.z + N.z * eps};
        const f3 L = reflectedRadiance<KM>(g, s, lights, nLights, O, rdir, eps, pix ^ 0x474c5359u,
                                           0x4e454532u + uint32_t(sI), rays, nee, ovf);
        const f3 F = schlickF3(F0, owm);
        sum.x += weight * F.x * L.x;
        sum.y += weight * F.y * L.y;
        sum.z += weight * F.z * L.z;
      }
      const float invSpp = 1.0f / float(spp);
      sum = f3{sum.x * invSpp, sum.y * invSpp, sum.z * invSpp};
    }
    Espec[pix] = make_float4(sum.x, sum.y, sum.z, 0.0f);
  }
  warpCount(&g.stats[0], rays);
  warpCount(&g.stats[1], nee);
  warpCount(g.overflow, ovf);
}

// glossy-masked box downsample of E_spec and its guides to the output grid
// (embree_renderer.cpp:990-1046): means over the cell's glossy samples, the
// normal renormalised; cells without one stay zero (not valid)
__global__ void k_glossy_down(int W, int H, int ss, ReflD rf, const float4* Espec, const float4* fpd,
                              const float4* fne, float4* Eo, float4* pdo, float4* neo) {
  const int Wo = W / ss, Ho = H / ss;
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= uint32_t(Wo) * uint32_t(Ho)) return;
  const int ox = int(o % uint32_t(Wo)), oy = int(o / uint32_t(Wo));
  f3 eS{0.0f, 0.0f, 0.0f}, nS{0.0f, 0.0f, 0.0f}, pS{0.0f, 0.0f, 0.0f};
  float zS = 0.0f;
  int cnt = 0;
  for (int sy = 0; sy < ss; ++sy)
    for (int sx = 0; sx < ss; ++sx) {
      const size_t pix = size_t(oy * ss + sy) * W + (ox * ss + sx);
      const float4 a = rf.amt[pix];
      if (a.x <= 0.0f || a.y <= 0.0f) continue;
      ++cnt;
      const float4 e = Espec[pix], n = fne[pix], p = fpd[pix];
      eS.x += e.x;
      eS.y += e.y;
      eS.z += e.z;
      nS.x += n.x;
      nS.y += n.y;
      nS.z += n.z;
      pS.x += p.x;
      pS.y += p.y;
      pS.z += p.z;
      zS += p.w;
    }
  if (cnt == 0) {
    Eo[o] = pdo[o] = neo[o] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    return;
  }
  const float inv = 1.0f / float(cnt);
  Eo[o] = make_float4(eS.x * inv, eS.y * inv, eS.z * inv, 0.0f);
  const f3 nAvg = safeNormalize(f3{nS.x * inv, nS.y * inv, nS.z * inv});
  neo[o] = make_float4(nAvg.x, nAvg.y, nAvg.z, 1.0f);
  pdo[o] = make_float4(pS.x * inv, pS.y * inv, pS.z * inv, zS * inv);
}

__global__ void k_glossy_composite(uint32_t n, ReflD rf, const float4* Espec, float4* color) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float4 a = rf.amt[p];
  if (a.x <= 0.0f || a.y <= 0.0f) return;
  const float4 e = Espec[p];
  float4 c = color[p];
  c.x += a.x * e.x;
  c.y += a.x * e.y;
  c.z += a.x * e.z;
  color[p] = c;
}

__global__ void k_glossy_elig(uint32_t n, ReflD rf, const float4* fne, float4* out) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float4 a = rf.amt[p], q = fne[p];
  out[p] = make_float4(q.x, q.y, q.z, (a.x > 0.0f && a.y > 0.0f) ? 1.0f : 0.0f);
}

template <typename F>
void byKind(int km, F&& f) {
  switch (km) {
    case kMaskMesh: f(std::integral_constant<int, kMaskMesh>{}); break;
    case kMaskSphere: f(std::integral_constant<int, kMaskSphere>{}); break;
    // ball-and-stick (spheres + capped cylinders), molecular surface + atoms
    case kMaskSphere | kMaskCone: f(std::integral_constant<int, kMaskSphere | kMaskCone>{}); break;
    case kMaskMesh | kMaskSphere: f(std::integral_constant<int, kMaskMesh | kMaskSphere>{}); break;
    default: f(std::integral_constant<int, kMaskAll>{});
  }
}

inline uint32_t blocks(uint64_t n, uint32_t tb) { return uint32_t((n + tb - 1) / tb); }

}  // namespace

void giGBuffer(int km, cudaStream_t s, const Params& p, const DScene& sc, int w, int h, float4* pd, float4* ne,
               float4* ng, unsigned long long* stats, unsigned long long* overflow) {
  const uint64_t n = uint64_t(w) * uint64_t(h);
  byKind(km, [&](auto K) {
    k_gbuffer<decltype(K)::value><<<blocks(n, 128), 128, 0, s>>>(p, sc, w, h, pd, ne, ng, stats, overflow);
  });
}

// Lanes per gather point: the sample count rounded down to a power of two,
// at most 8 (a warp then holds four points' fans).  The grid is at most 16
// blocks per SM (a list's length is known only on the device).
void giGather(int km, cudaStream_t s, const GiP& g, const DScene& sc, const LightD* lights, int nLights,
              const GiGrid& grid, const uint32_t* list, const uint32_t* listCount, uint32_t n, int spp, float4* E) {
  // a ReSTIR gather streams each point's samples in order: one thread per point
  const int lanes = g.rsv ? 1 : spp >= 8 ? 8 : spp >= 4 ? 4 : spp >= 2 ? 2 : 1;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const uint32_t nb = std::max(1u, std::min(blocks(uint64_t(n) * uint64_t(lanes), 128), uint32_t(std::max(sms, 1)) * 16u));
  byKind(km, [&](auto K) {
    constexpr int k = decltype(K)::value;
    if (lanes == 8)
      k_gather<k, 8><<<nb, 128, 0, s>>>(g, sc, lights, nLights, grid, list, listCount, n, spp, E);
    else if (lanes == 4)
      k_gather<k, 4><<<nb, 128, 0, s>>>(g, sc, lights, nLights, grid, list, listCount, n, spp, E);
    else if (lanes == 2)
      k_gather<k, 2><<<nb, 128, 0, s>>>(g, sc, lights, nLights, grid, list, listCount, n, spp, E);
    else
      k_gather<k, 1><<<nb, 128, 0, s>>>(g, sc, lights, nLights, grid, list, listCount, n, spp, E);
  });
}

void giDenoiseInit(cudaStream_t s, uint32_t n, float4* E, const float4* ne, uint8_t* valid, float4* irr) {
  k_gdn_init<<<blocks(n, 256), 256, 0, s>>>(n, E, ne, valid, irr);
}
void giDenoiseAux(cudaStream_t s, int W, int H, const uint8_t* valid, const float4* irr, const float4* pd,
                  float* var, float* pgrad) {
  k_gdn_aux<<<blocks(uint64_t(W) * H, 256), 256, 0, s>>>(W, H, valid, irr, pd, var, pgrad);
}
void giDenoiseIter(cudaStream_t s, int W, int H, int step, const uint8_t* valid, const float4* ne,
                   const float4* pd, const float4* irr, const float* var, const float* pgrad, float sigmaN,
                   float sigmaZ, float sigmaL, float4* next) {
  k_gdn_iter<<<blocks(uint64_t(W) * H, 256), 256, 0, s>>>(W, H, step, valid, ne, pd, irr, var, pgrad, sigmaN,
                                                           sigmaZ, sigmaL, next);
}
void giDenoiseWrite(cudaStream_t s, uint32_t n, const uint8_t* valid, const float4* irr, float4* E) {
  k_gdn_write<<<blocks(n, 256), 256, 0, s>>>(n, valid, irr, E);
}
// Pixel i of a W x H grid in 16 x 16 tiles (row order inside a tile, tiles in
// row order), the columns and rows past the last whole tile in row order: a
// bijection on [0, W H).  The edge-patch list walks its pixels in this order,
// so the points a warp gathers lie on one stretch of an edge.
struct TileOrder {
  uint32_t W, H;
  UBR_HD uint32_t operator()(uint32_t i) const {
    const uint32_t fw = W & ~15u, fh = H & ~15u, nt = fw * fh;
    if (i < nt) {
      const uint32_t t = i >> 8, k = i & 255u, tx = fw >> 4;
      return ((t / tx) * 16u + (k >> 4)) * W + (t % tx) * 16u + (k & 15u);
    }
    uint32_t j = i - nt;
    const uint32_t rw = W - fw;
    if (j < rw * fh) return (j / rw) * W + fw + j % rw;
    j -= rw * fh;
    return fh * W + j;
  }
};
using TileIt = thrust::transform_iterator<TileOrder, thrust::counting_iterator<uint32_t>>;
using TileFlagIt = thrust::permutation_iterator<const uint8_t*, TileIt>;

size_t giPatchListBytes(uint32_t n) {
  size_t bytes = 0;
  const TileIt in(thrust::counting_iterator<uint32_t>(0), TileOrder{n, 1});
  cub::DeviceSelect::Flagged(nullptr, bytes, in, TileFlagIt(static_cast<const uint8_t*>(nullptr), in),
                             static_cast<uint32_t*>(nullptr), static_cast<uint32_t*>(nullptr), int(n));
  return bytes;
}
cudaError_t giUpsample(cudaStream_t s, int W, int H, const float4* fpd, const float4* fne, const GiGrid& lo,
                       const float4* Elo, float normalPow, float depthScale, int fallbackR, int patchOn,
                       float patchThresh, float4* E, uint8_t* patchFlag, void* listTemp, size_t listTempBytes,
                       uint32_t* patchList, uint32_t* patchCount, unsigned long long* holes) {
  const uint32_t n = uint32_t(W) * uint32_t(H);
  k_upsample<<<blocks(n, 128), 128, 0, s>>>(W, H, fpd, fne, lo, Elo, normalPow, depthScale, fallbackR, patchOn,
                                            patchThresh, E, patchFlag, holes);
  if (!patchOn || !patchFlag) return cudaGetLastError();
  // the pixels to patch, in 16 x 16 tile order (neighbouring rim pixels stay
  // neighbours in the list the patch gather walks)
  const TileIt in(thrust::counting_iterator<uint32_t>(0), TileOrder{uint32_t(W), uint32_t(H)});
  return cub::DeviceSelect::Flagged(listTemp, listTempBytes, in, TileFlagIt(patchFlag, in), patchList, patchCount,
                                    int(n), s);
}
void giSmooth(cudaStream_t s, int W, int H, const uint32_t* list, const uint32_t* count, uint32_t n,
              const float4* fpd, const float4* fne, float normalPow, float depthScale, int radius,
              const float4* Esrc, float4* E) {
  k_smooth<<<blocks(n, 128), 128, 0, s>>>(W, H, list, count, n, fpd, fne, normalPow, depthScale, radius, Esrc, E);
}
void giComposite(cudaStream_t s, uint32_t n, const float4* ne, const float4* refl, const float4* E, float gI,
                 float4* color) {
  k_composite<<<blocks(n, 256), 256, 0, s>>>(n, ne, refl, E, gI, color);
}
void giAdaptiveMask(cudaStream_t s, int W, int H, const float4* E, const float* halfE, const float4* ne, int spp,
                    float threshold, uint8_t* mask) {
  k_adapt_mask<<<blocks(uint64_t(W) * H, 256), 256, 0, s>>>(W, H, E, halfE, ne, spp, threshold, mask);
}
void giDilate(cudaStream_t s, int W, int H, const uint8_t* in, const float4* ne, uint8_t* out) {
  k_dilate<<<blocks(uint64_t(W) * H, 256), 256, 0, s>>>(W, H, in, ne, out);
}
void giMaskList(cudaStream_t s, uint32_t n, const uint8_t* mask, uint32_t* list, uint32_t* count) {
  k_mask_list<<<blocks(n, 256), 256, 0, s>>>(n, mask, list, count);
}
void giMerge(cudaStream_t s, const uint32_t* list, const uint32_t* count, uint32_t n, int spp, int extra,
             const float4* Er, float4* E) {
  k_merge<<<blocks(n, 256), 256, 0, s>>>(list, count, n, spp, extra, Er, E);
}
void giSpatialRound(int km, cudaStream_t s, const GiSpatial& sp, const DScene& sc, const GiGrid& grid,
                    const float4* in, float4* out, int round, float4* E, unsigned long long* overflow) {
  const uint64_t n = uint64_t(grid.W) * uint64_t(grid.H);
  byKind(km, [&](auto K) {
    k_spatial<decltype(K)::value><<<blocks(n, 128), 128, 0, s>>>(sp, sc, grid, in, out, round, E, overflow);
  });
}
void giReflect(int km, cudaStream_t s, const GiP& g, const DScene& sc, const LightD* lights, int nLights,
               const GiGrid& full, const ReflD& r, const GiCam& cam, uint32_t n, float4* color) {
  byKind(km, [&](auto K) {
    k_reflect<decltype(K)::value><<<blocks(n, 128), 128, 0, s>>>(g, sc, lights, nLights, full, r, cam, n, color);
  });
}
void giGlossy(int km, cudaStream_t s, const GiP& g, const DScene& sc, const LightD* lights, int nLights,
              const GiGrid& full, const ReflD& r, const GiCam& cam, uint32_t n, int spp, uint32_t frameSeed,
              float4* Espec) {
  const uint32_t seedMix = hashU32(frameSeed ^ 0x474c5359u);  // 'GLSY'
  byKind(km, [&](auto K) {
    k_glossy<decltype(K)::value><<<blocks(n, 128), 128, 0, s>>>(g, sc, lights, nLights, full, r, cam, n, spp,
                                                                seedMix, Espec);
  });
}
void giGlossyDown(cudaStream_t s, int W, int H, int ss, const ReflD& r, const float4* Espec, const float4* fpd,
                  const float4* fne, float4* Eo, float4* pdo, float4* neo) {
  const uint64_t no = uint64_t(W / ss) * uint64_t(H / ss);
  k_glossy_down<<<blocks(no, 256), 256, 0, s>>>(W, H, ss, r, Espec, fpd, fne, Eo, pdo, neo);
}
void giGlossyComposite(cudaStream_t s, uint32_t n, const ReflD& r, const float4* Espec, float4* color) {
  k_glossy_composite<<<blocks(n, 256), 256, 0, s>>>(n, r, Espec, color);
}
void giGlossyElig(cudaStream_t s, uint32_t n, const ReflD& r, const float4* fne, float4* out) {
  k_glossy_elig<<<blocks(n, 256), 256, 0, s>>>(n, r, fne, out);
}

}  // namespace ubr

// ubr_internal.h -- shared device/host definitions of libubr (not installed).
//
// Vector math, the device scene view, the per-frame parameter block and the
// ray/primitive intersectors used by the BVH build and the trace kernels.
// The library is compiled with --fmad=false so shading arithmetic rounds the
// way the reference's C++ does (each product/sum rounded on its own); the
// traversal slab test and the binary any-hit forms of the sphere and capped
// cone tests opt back into FMA explicitly with fmaf() (the any-hit forms also
// use the approximate division and square root).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cmath>

#include "ubr.h"

#define UBR_HD __host__ __device__ __forceinline__
#define UBR_D __device__ __forceinline__

namespace ubr {

struct f3 {
  float x, y, z;
};
UBR_HD f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
UBR_HD f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
UBR_HD f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
UBR_HD f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
UBR_HD f3 operator*(float s, f3 a) { return {a.x * s, a.y * s, a.z * s}; }
UBR_HD f3 neg(f3 a) { return {-a.x, -a.y, -a.z}; }
UBR_HD float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
UBR_HD f3 cross(f3 a, f3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
UBR_HD float length(f3 a) { return sqrtf(dot(a, a)); }
// Fused forms for the binary any-hit tests: F = true evaluates a dot product
// and a*s + c with one rounding per multiply-add (fewer issued instructions in
// the occlusion kernels); F = false is the separately rounded operation above,
// bit for bit.
template <bool F>
UBR_HD float dotT(f3 a, f3 b) {
  return F ? fmaf(a.x, b.x, fmaf(a.y, b.y, a.z * b.z)) : dot(a, b);
}
template <bool F>
UBR_HD f3 madT(f3 a, float s, f3 c) {
  return F ? f3{fmaf(a.x, s, c.x), fmaf(a.y, s, c.y), fmaf(a.z, s, c.z)} : c + a * s;
}
// Division and square root of the any-hit forms: F = true uses the
// approximate hardware forms (div.approx via __fdividef, sqrt.approx; a few
// ulps) in place of the correctly rounded sequences; F = false is `/` and
// sqrtf.  Host code always takes the correctly rounded form.
template <bool F>
UBR_HD float divT(float a, float b) {
#ifdef __CUDA_ARCH__
  if (F) return __fdividef(a, b);
#endif
  return a / b;
}
template <bool F>
UBR_HD float sqrtT(float x) {
#ifdef __CUDA_ARCH__
  if (F) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
  }
#endif
  return sqrtf(x);
}
// umbreon normalize (scene.hpp:36-39): a * (1/l) when l > 0
UBR_HD f3 normalize(f3 a) {
  float l = length(a);
  return l > 0.0f ? a * (1.0f / l) : a;
}
// scene.hpp:44-49
UBR_HD f3 safeNormalize(f3 a) {
  float s = 1.0f / sqrtf(fmaxf(dot(a, a), 0x1.0p-126f));
  return a * s;
}
// scene.hpp:53-57
UBR_HD f3 safeNormalize(f3 a, f3 fb) {
  float d = dot(a, a);
  if (d < 1.0e-18f) return fb;
  return a * (1.0f / sqrtf(d));
}
UBR_HD float comp(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
UBR_HD float radiansf(float deg) { return deg * 0.01745329252f; }

struct Frame3 {
  f3 t, b, n;
};
// scene.hpp:69-76 frameFromNormal
UBR_HD Frame3 frameFromNormal(f3 n) {
  const f3 seed0{0.0f, n.z, -n.y};
  const f3 seed1{-n.z, 0.0f, n.x};
  const f3 t = safeNormalize(fabsf(n.x) < fabsf(n.y) ? seed0 : seed1, f3{1.0f, 0.0f, 0.0f});
  const f3 b = cross(n, t);
  return {t, b, n};
}

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr int kMesh = 0, kSphere = 1, kRound = 2, kCone = 3;
// A primitive reference packs (kind << 30) | primID.
UBR_HD uint32_t packRef(int kind, uint32_t prim) { return (uint32_t(kind) << 30) | prim; }
UBR_HD int refKind(uint32_t r) { return int(r >> 30); }
UBR_HD uint32_t refPrim(uint32_t r) { return r & 0x3FFFFFFFu; }

// BVH child code: >= 0 internal node, < 0 leaf = ~slot (one primitive).
// Node = 4 float4: (lo_l.x, hi_l.x, lo_l.y, hi_l.y), (lo_r.x, hi_r.x, lo_r.y,
// hi_r.y), (lo_l.z, hi_l.z, lo_r.z, hi_r.z), (child_l, child_r, -, -).
constexpr int kNodeF4 = 4;
// Leaf slot geometry = 3 float4, by kind:
//   mesh   : v0 | v1 | v2          (xyz, w unused)
//   sphere : (c, r)
//   cone   : (p0, r0) | (p1, r1) | (unit axis, length) from segmentAxis
//   round  : (p0, r0) | (p1, r1) | (flags bits, -, -, -)
constexpr int kLeafF4 = 3;

// 8-wide BVH node, 80 B = 5 float4 (compressed child bounds after Ylitie,
// Karras and Laine, "Efficient Incoherent Ray Traversal on GPUs Through
// Compressed Wide BVHs", HPG 2017):
//   [0] origin p.xyz, (ex | ey<<8 | ez<<16 | nInternal<<24 | nChildren<<28):
//       biased exponents of the per-axis power-of-two scale, then the number
//       of internal children (slots 0..nInternal-1, node = childBase + slot)
//       and of all children (leaf slots follow the internal ones)
//   [1] childBase, primBase, meta[0..3], meta[4..7]
//   [2] qlo.x[0..7], qlo.y[0..7]      (8-bit quantised child bounds)
//   [3] qlo.z[0..7], qhi.x[0..7]
//   [4] qhi.y[0..7], qhi.z[0..7]
// meta byte: 0 empty; 0x80|k internal child = node childBase+k;
//            (count<<5)|offset leaf = count (1..3) primitives at primBase+offset.
// Child bound = p + q * scale, evaluated with fmaf in both build and
// traversal so the quantised box is exactly the one the build made
// conservative.
constexpr int kWideF4 = 5;
constexpr int kWideLeafMax = 3;

struct DScene {
  const float4* wnodes = nullptr;  // 8-wide nodes (root = 0)
  uint32_t wideNodes = 0;          // number of 8-wide nodes
  const float4* nodes = nullptr;
  int32_t root = 0;             // child code of the root (when prims > 0)
  uint32_t primCount = 0;       // total primitives
  const uint32_t* leafRef = nullptr;
  const float4* leafGeo = nullptr;
  // mesh shading tables (baked vertices, primID order)
  const float* meshNrm = nullptr;      // 3 per vertex
  const float4* meshCol = nullptr;     // per vertex
  const uint32_t* meshIdx = nullptr;   // 3 per triangle
  const uint32_t* meshTriMat = nullptr;// per base triangle -> material table index
  const uint8_t* meshTriMatId = nullptr;  // per base triangle: the caller's material id (or null)
  uint32_t meshMatCount = 0;           // Mesh::materials.size()
  uint32_t baseSpheres = 0;            // Scene::spheres.size()
  uint32_t roundCount = 0;             // open-cylinder segments (all instances)
  uint32_t meshMat = 0;                // when meshTriMat == nullptr
  uint32_t baseTri = 0;
  // per-kind side tables (primID order); index 0 unused
  const float4* primColor[4] = {nullptr, nullptr, nullptr, nullptr};
  const uint32_t* primMat[4] = {nullptr, nullptr, nullptr, nullptr};
  const uint8_t* primFromEdge[4] = {nullptr, nullptr, nullptr, nullptr};
  const float* primOpacity1[4] = {nullptr, nullptr, nullptr, nullptr};
  const float4* primAxis[4] = {nullptr, nullptr, nullptr, nullptr};  // cylinder unit axis, or null
  const uint16_t* primGroup[4] = {nullptr, nullptr, nullptr, nullptr};  // CueMol section
  const uint16_t* meshTriGroup = nullptr;  // per base triangle (or null: section 0)
  const float4* rcClip = nullptr;      // 2 per round segment (clipL, clipR)
  const float4* sph = nullptr;         // per sphere (centre, radius), primID order
  uint32_t baseSph = 0;                // spheres per instance (primID % baseSph = input sphere)
  const ubr_material* mats = nullptr;
  uint32_t geomID[4] = {kInvalid, kInvalid, kInvalid, kInvalid};
};

// What traversal reads of a scene, compact enough to live in registers (a
// batched kernel loads it once per ray instead of re-reading the frame's
// DScene through global memory inside the traversal loop).
struct TravScene {
  const float4* wnodes;
  const uint32_t* leafRef;
  const float4* leafGeo;
  const float4* rcClip;
  uint32_t primCount;
  uint32_t geomID[4];
};

UBR_HD TravScene travOf(const DScene& s) {
  return TravScene{s.wnodes, s.leafRef, s.leafGeo, s.rcClip, s.primCount,
                   {s.geomID[0], s.geomID[1], s.geomID[2], s.geomID[3]}};
}

struct Hit {
  float t;
  uint32_t ref;  // kInvalid on a miss
  float u, v;
  f3 Ng;
};

struct Ray {
  f3 org, dir;
  float tnear, tfar;
};

// ---------------------------------------------------------------------------
// Intersectors (semantics: a hit is valid for tnear <= t <= tmax)

struct TriPre {
  int kx, ky, kz;
  float Sx, Sy, Sz;
};
UBR_HD TriPre triPre(f3 d) {
  TriPre p;
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  p.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  p.kx = (p.kz + 1) % 3;
  p.ky = (p.kx + 1) % 3;
  if (comp(d, p.kz) < 0.0f) {
    int t = p.kx;
    p.kx = p.ky;
    p.ky = t;
  }
  p.Sx = comp(d, p.kx) / comp(d, p.kz);
  p.Sy = comp(d, p.ky) / comp(d, p.kz);
  p.Sz = 1.0f / comp(d, p.kz);
  return p;
}

// Watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2013): shear into
// ray space, 2-D edge functions U,V,W, double-precision redo when one is 0.
UBR_HD bool isectTriangle(const Ray& r, const TriPre& pre, f3 v0, f3 v1, f3 v2, float tnear,
                          float tmax, Hit& h) {
  const f3 A = v0 - r.org, B = v1 - r.org, C = v2 - r.org;
  const float Ax = comp(A, pre.kx) - pre.Sx * comp(A, pre.kz);
  const float Ay = comp(A, pre.ky) - pre.Sy * comp(A, pre.kz);
  const float Bx = comp(B, pre.kx) - pre.Sx * comp(B, pre.kz);
  const float By = comp(B, pre.ky) - pre.Sy * comp(B, pre.kz);
  const float Cx = comp(C, pre.kx) - pre.Sx * comp(C, pre.kz);
  const float Cy = comp(C, pre.ky) - pre.Sy * comp(C, pre.kz);
  float U = Cx * By - Cy * Bx;
  float V = Ax * Cy - Ay * Cx;
  float W = Bx * Ay - By * Ax;
  if (U == 0.0f || V == 0.0f || W == 0.0f) {
    U = float(double(Cx) * By - double(Cy) * Bx);
    V = float(double(Ax) * Cy - double(Ay) * Cx);
    W = float(double(Bx) * Ay - double(By) * Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
  const float det = U + V + W;
  if (det == 0.0f) return false;
  const float Az = pre.Sz * comp(A, pre.kz);
  const float Bz = pre.Sz * comp(B, pre.kz);
  const float Cz = pre.Sz * comp(C, pre.kz);
  const float T = U * Az + V * Bz + W * Cz;
  const float rcp = 1.0f / det;
  const float t = T * rcp;
  if (!(t >= tnear && t <= tmax)) return false;
  h.t = t;
  h.u = V * rcp;
  h.v = W * rcp;
  h.Ng = cross(v1 - v0, v2 - v0);
  return true;
}

// Sphere, perpendicular-distance form; front root first, back root second.
// ATTR = false (any-hit queries) skips the hit attributes and evaluates the
// same algebra with fused multiply-adds and the approximate division and
// square root: a binary answer, which can differ from the correctly rounded
// one only for a ray that grazes the sphere or ends within a few ulps of it.  Every query that reports a distance, a
// normal or a first hit (ATTR = true) keeps the separately rounded form.
template <bool ATTR = true>
UBR_HD bool isectSphere(const Ray& r, f3 c, float rad, float tnear, float tmax, Hit& h) {
  constexpr bool F = !ATTR;
  const f3 c0 = c - r.org;
  const float rd2 = divT<F>(1.0f, dotT<F>(r.dir, r.dir));
  const float projC0 = dotT<F>(c0, r.dir) * rd2;
  const f3 perp = F ? madT<true>(r.dir, -projC0, c0) : c0 - r.dir * projC0;
  const float l2 = dotT<F>(perp, perp);
  const float r2 = rad * rad;
  if (!(l2 <= r2)) return false;
  const float td = sqrtT<F>((r2 - l2) * rd2);
  const float tf = projC0 - td;
  const float tb = projC0 + td;
  float t;
  if (tf >= tnear && tf <= tmax) t = tf;
  else if (tb >= tnear && tb <= tmax) t = tb;
  else return false;
  h.t = t;
  if (ATTR) {
    h.u = 0.0f;
    h.v = 0.0f;
    h.Ng = r.dir * t - c0;
  }
  return true;
}

// Lateral surface of a frustum on axis (b, unit a), radius k0 + k1*hax over
// axial range [h0, h1].  Solved in float: the ray origin is first moved to
// the point of the ray closest to the frustum's mid-axis point (parameter
// ts0), so the quadratic's coefficients stay small and well conditioned;
// roots are returned in the original ray parameter.  Up to two roots.
// F = true: fused multiply-adds in the dot products and a*s + c terms, the
// approximate division and square root (the any-hit form, as in isectSphere).
template <bool F = false>
UBR_HD int frustumRoots(const Ray& r, f3 b, f3 a, float h0, float h1, float k0, float k1,
                        float* ts, float* hs) {
  const f3 mid = madT<F>(a, 0.5f * (h0 + h1), b);
  const float dd = dotT<F>(r.dir, r.dir);
  const float ts0 = divT<F>(dotT<F>(mid - r.org, r.dir), dd);
  const f3 o = madT<F>(r.dir, ts0, r.org);
  const f3 w = o - b;
  const float wa = dotT<F>(w, a), da = dotT<F>(r.dir, a);
  const f3 wp = F ? madT<true>(a, -wa, w) : w - a * wa;
  const f3 dp = F ? madT<true>(a, -da, r.dir) : r.dir - a * da;
  const float g0 = F ? fmaf(k1, wa, k0) : k0 + k1 * wa, g1 = k1 * da;
  const float A = F ? fmaf(-g1, g1, dotT<true>(dp, dp)) : dot(dp, dp) - g1 * g1;
  const float B = F ? fmaf(-g0, g1, dotT<true>(wp, dp)) : dot(wp, dp) - g0 * g1;  // half the linear coefficient
  const float Cc = F ? fmaf(-g0, g0, dotT<true>(wp, wp)) : dot(wp, wp) - g0 * g0;
  float rr[2];
  int m = 0;
  if (fabsf(A) <= 1e-12f * dd) {
    if (B == 0.0f) return 0;
    rr[m++] = divT<F>(-Cc, 2.0f * B);
  } else {
    const float disc = F ? fmaf(B, B, -(A * Cc)) : B * B - A * Cc;
    if (disc < 0.0f) return 0;
    const float sq = sqrtT<F>(disc);
    const float q = -(B + copysignf(sq, B));
    float r0 = divT<F>(q, A), r1 = q != 0.0f ? divT<F>(Cc, q) : r0;
    if (r0 > r1) {
      const float t = r0;
      r0 = r1;
      r1 = t;
    }
    rr[m++] = r0;
    rr[m++] = r1;
  }
  int n = 0;
  for (int i = 0; i < m; ++i) {
    const float hh = F ? fmaf(rr[i], da, wa) : wa + rr[i] * da;
    if (hh >= h0 && hh <= h1 && (F ? fmaf(k1, hh, k0) : k0 + k1 * hh) >= 0.0f) {
      ts[n] = ts0 + rr[i];
      hs[n] = hh;
      ++n;
    }
  }
  return n;
}

// Unit axis and length of a segment, as the cone intersector derives them
// (the BVH build stores them in the leaf record with these same operations).
UBR_HD void segmentAxis(f3 p0, f3 p1, f3& a, float& L) {
  const f3 ax = p1 - p0;
  L = length(ax);
  a = ax * (1.0f / L);
}

// Capped cone segment (CONE_LINEAR_CURVE): frustum + flat disks at p0, p1,
// with its unit axis `a` and length L precomputed by segmentAxis.
// ATTR = false (any-hit queries) returns at the first valid hit and uses the
// fused forms (as isectSphere does).
template <bool ATTR = true>
UBR_HD bool isectConeCurveAxis(const Ray& r, f3 p0, float r0, f3 p1, float r1, f3 a, float L, float tnear,
                               float tmax, Hit& h) {
  constexpr bool F = !ATTR;
  if (!(L > 0.0f)) return false;
  const float k1 = divT<F>(r1 - r0, L);
  float ts[2], hs[2];
  const int n = frustumRoots<F>(r, p0, a, 0.0f, L, r0, k1, ts, hs);
  bool found = false;
  float best = tmax;
  for (int i = 0; i < n; ++i) {
    if (ts[i] >= tnear && ts[i] <= best) {
      best = ts[i];
      h.t = ts[i];
      if (!ATTR) return true;
      const f3 P = r.org + r.dir * ts[i];
      const f3 rad = (P - p0) - a * hs[i];
      h.u = hs[i] / L;
      h.v = 0.0f;
      h.Ng = rad - a * (k1 * length(rad));
      found = true;
    }
  }
  const float da = dotT<F>(r.dir, a);
  if (da != 0.0f) {
    for (int e = 0; e < 2; ++e) {
      const f3 pc = e == 0 ? p0 : p1;
      const float rc = e == 0 ? r0 : r1;
      const float t = divT<F>(dotT<F>(pc - r.org, a), da);
      if (!(t >= tnear && t <= best)) continue;
      const f3 P = madT<F>(r.dir, t, r.org);
      const f3 d = P - pc;
      if (dotT<F>(d, d) > rc * rc) continue;
      best = t;
      h.t = t;
      if (!ATTR) return true;
      h.u = float(e);
      h.v = 0.0f;
      h.Ng = e == 0 ? a * -1.0f : a;
      found = true;
    }
  }
  return found;
}

UBR_HD bool isectConeCurve(const Ray& r, f3 p0, float r0, f3 p1, float r1, float tnear, float tmax, Hit& h) {
  f3 a;
  float L;
  segmentAxis(p0, p1, a, L);
  return isectConeCurveAxis<true>(r, p0, r0, p1, r1, a, L, tnear, tmax, h);
}

// Round segment (ROUND_LINEAR_CURVE): end spheres + tangent cone, hits kept
// on this segment's side of the bisector plane at each neighbour joint.
UBR_HD bool isectRoundCurve(const Ray& r, f3 p0, float r0, f3 p1, float r1, uint32_t flags,
                            f3 clipL, f3 clipR, float tnear, float tmax, Hit& h) {
  const f3 ax = p1 - p0;
  const float L = length(ax);
  bool found = false;
  float best = tmax;
  float sinA = 0.0f, cosA = 1.0f;
  f3 a{0.0f, 0.0f, 1.0f};
  const bool hasCone = L > fabsf(r0 - r1) && L > 0.0f;
  if (hasCone) {
    a = ax * (1.0f / L);
    sinA = (r0 - r1) / L;
    cosA = sqrtf(fmaxf(0.0f, 1.0f - sinA * sinA));
  }
  const float s0 = r0 * sinA, s1 = L + r1 * sinA;
  for (int e = 0; e < 2; ++e) {
    const f3 c = e == 0 ? p0 : p1;
    const float rad = e == 0 ? r0 : r1;
    if (!hasCone && ((e == 0 && r0 < r1) || (e == 1 && r1 <= r0))) continue;
    const f3 c0 = c - r.org;
    const float rd2 = 1.0f / dot(r.dir, r.dir);
    const float pc = dot(c0, r.dir) * rd2;
    const f3 perp = c0 - r.dir * pc;
    const float l2 = dot(perp, perp), rr = rad * rad;
    if (!(l2 <= rr)) continue;
    const float td = sqrtf((rr - l2) * rd2);
    for (int k = 0; k < 2; ++k) {
      const float t = k == 0 ? pc - td : pc + td;
      const f3 P = r.org + r.dir * t;
      if (hasCone) {
        const float hh = dot(P - p0, a);
        if (e == 0 && hh > s0) continue;
        if (e == 1 && hh < s1) continue;
      }
      if (!(t >= tnear && t <= best)) continue;
      if ((flags & 1u) && dot(P - p0, clipL) < 0.0f) continue;
      if ((flags & 2u) && dot(P - p1, clipR) > 0.0f) continue;
      const float u = hasCone ? fminf(1.0f, fmaxf(0.0f, dot(P - p0, a) / L)) : 0.0f;
      best = t;
      h.t = t;
      h.u = u;
      h.v = 0.0f;
      h.Ng = r.dir * t - c0;
      found = true;
    }
  }
  if (hasCone) {
    const float k0c = r0 * cosA;
    const float k1c = (s1 > s0) ? (r1 * cosA - r0 * cosA) / (s1 - s0) : 0.0f;
    float ts[2], hs[2];
    const int n = frustumRoots(r, p0, a, s0, s1, k0c - k1c * s0, k1c, ts, hs);
    for (int i = 0; i < n; ++i) {
      const float t = ts[i];
      if (!(t >= tnear && t <= best)) continue;
      const f3 P = r.org + r.dir * t;
      if ((flags & 1u) && dot(P - p0, clipL) < 0.0f) continue;
      if ((flags & 2u) && dot(P - p1, clipR) > 0.0f) continue;
      const f3 rad = (P - p0) - a * hs[i];
      best = t;
      h.t = t;
      h.u = fminf(1.0f, fmaxf(0.0f, hs[i] / L));
      h.v = 0.0f;
      h.Ng = rad - a * (k1c * length(rad));
      found = true;
    }
  }
  return found;
}

// Per-frame shading parameters (kernel argument, by value).
constexpr int kMaxLights = 64;
struct LightD {
  f3 L, color;
  uint32_t highlight;
  float radius;
  int32_t samples;      // shadow rays for this light (1 hard, n soft)
  int32_t rayOffset;    // first shadow-ray index within a hit's ray block
  uint32_t soft;        // 1 when sampled through the tea2 stream
};

struct Params {
  int W, H;             // hi-res grid
  int outW, outH, ss;
  f3 camPos, camDir, right, up;
  float halfW, halfH, persHalfW, persHalfH;
  int ortho;
  float clipNear, clipFar;
  f3 ambLight, bg, aoUp;
  int nLights;
  int aoSamples;
  float aoDistance, aoIntensity, aoFalloffPower;
  int aoMultiScale, aoBentNormal, aoMultibounce, aoLowDiscrepancy, aoEnhanced;
  int aoWriteAov;       // first-hit AO AOVs requested (AO rays trace nearest hits)
  int aaMode;           // 1: adaptive AA (first-hit normal and section captured)
  float aaThreshold;
  int aoCoarse;         // coarse-grid AO active: hits look up the grid before casting AO rays
  int cgW, cgH;         // coarse AO grid size
  int reuseAo;          // AO rays 0..reuseAo-1 of a hit are copied from an earlier pass (Bufs::reuseOcc)
  f3 aoSky, aoGround;
  float aoDiffuseFactor;
  int shadowsActive, shadowSamples;
  float specularScale;
  int transparency, transparentBg, maxIters;
  int fogOn;
  f3 fogColor;
  float fogStart, fogEnd;
  float gamma;
  int raysPerHit;       // AO rays + all lights' shadow rays
  int shadowRays;       // sum of LightD::samples (0 when shadows inactive)
  int lightOff;         // first light of this frame in the lights array
  int gi;               // pt1 GI: eligible hits drop their ambient; first hits captured for the gather
  float giIntensity;
  int pt2Refl;          // pt2 traced reflection owns the reflection term (first hits recorded)
  int pt2Glossy;        // ... with GGX lobes for reflective finishes that carry a highlight
};

}  // namespace ubr

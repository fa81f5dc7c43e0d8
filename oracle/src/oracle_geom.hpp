// oracle_geom.hpp -- TEST INFRASTRUCTURE (the oracle), never shipped.
//
// CPU restatement of the ray/primitive queries the reference delegates to
// Intel Embree 4 (pinned 4.4.1, Taskfile.yml:22; not vendored in the
// reference, absent from this machine).  The reference calls them at
// shading/transparency.hpp:382 (rtcIntersect1), shading/secondary_rays.hpp:79-97
// (rtcOccluded1) and shading/hit_shader.hpp:162-165 (rtcInterpolate0), on the
// geometry types built in render/scene_build.cpp:23-128 (TRIANGLE,
// SPHERE_POINT) and render/curve_build.cpp:180-266 (ROUND_LINEAR_CURVE with
// neighbour flags, CONE_LINEAR_CURVE).
//
// Published algorithms restated here:
//   * triangles: watertight ray/triangle test of Woop, Benthin and Wald,
//     "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013 (Embree's robust
//     mode); barycentrics u,v weight v1,v2; Ng = (v1-v0) x (v2-v0).
//   * spheres: perpendicular-distance form (project the centre onto the ray,
//     t = tc -/+ sqrt((r^2 - l^2)/|d|^2)); front hit first, back hit when the
//     front lies outside [tnear, tfar]; Ng = hit - centre.
//   * cone curves: finite cone frustum between the two control points with
//     flat disk caps at both ends; u = axial fraction.
//   * round curves: swept sphere with linear radius (end spheres joined by the
//     tangent cone); where a segment has a neighbour (flag) the hit must lie
//     on this segment's side of the bisector plane through the shared vertex,
//     so a chain renders as one seamless tube with no internal caps.
//   * closest hit: smallest t; equal t resolved to the lowest (geomID, primID)
//     so the answer does not depend on the BVH.
// Interval semantics follow Embree: a hit is valid for tnear <= t <= tfar.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace oracle {

struct V3 {
  float x = 0.0f, y = 0.0f, z = 0.0f;
  V3() = default;
  V3(float a, float b, float c) : x(a), y(b), z(c) {}
};
inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator*(float s, V3 a) { return a * s; }
inline float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 cross(V3 a, V3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline V3 normalize(V3 a) {
  float l = length(a);
  return l > 0.0f ? a * (1.0f / l) : a;
}
inline float comp(const V3& v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

constexpr uint32_t kInvalid = 0xFFFFFFFFu;
constexpr int kMesh = 0, kSphere = 1, kRound = 2, kCone = 3;

struct Hit {
  float t = 0.0f;
  uint32_t geomID = kInvalid;
  uint32_t primID = kInvalid;
  float u = 0.0f, v = 0.0f;
  V3 Ng;
};

struct Ray {
  V3 org, dir;
  float tnear = 0.0f, tfar = std::numeric_limits<float>::infinity();
};

// Geometry in primID order per kind (what the reference hands to Embree).
struct GeomSet {
  std::vector<float> triPos;      // 3 per vertex
  std::vector<uint32_t> triIdx;   // 3 per triangle
  std::vector<float> sph;         // 4 per sphere (x y z r)
  std::vector<float> rcV;         // round curve vertices, 4 floats (x y z r)
  std::vector<uint32_t> rcIdx;    // first vertex of each segment
  std::vector<uint8_t> rcFlags;   // bit0 = neighbour left, bit1 = right
  std::vector<float> ccV;         // cone curve vertices, 4 floats
  std::vector<uint32_t> ccIdx;
  uint32_t geomID[4] = {kInvalid, kInvalid, kInvalid, kInvalid};
  size_t count(int kind) const {
    switch (kind) {
      case kMesh: return triIdx.size() / 3;
      case kSphere: return sph.size() / 4;
      case kRound: return rcIdx.size();
      default: return ccIdx.size();
    }
  }
};

// ---------------------------------------------------------------------------
// Primitive tests.  Each returns the nearest valid hit in [tnear, tbest) and
// writes it into `h` (t, u, v, Ng); the caller owns geomID/primID.

inline V3 triVert(const GeomSet& g, uint32_t vi) {
  return {g.triPos[3 * vi], g.triPos[3 * vi + 1], g.triPos[3 * vi + 2]};
}

struct TriRayPre {
  int kx, ky, kz;
  float Sx, Sy, Sz;
};
inline TriRayPre triPre(const V3& d) {
  TriRayPre p;
  const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
  p.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  p.kx = (p.kz + 1) % 3;
  p.ky = (p.kx + 1) % 3;
  if (comp(d, p.kz) < 0.0f) std::swap(p.kx, p.ky);
  p.Sx = comp(d, p.kx) / comp(d, p.kz);
  p.Sy = comp(d, p.ky) / comp(d, p.kz);
  p.Sz = 1.0f / comp(d, p.kz);
  return p;
}

inline bool intersectTriangle(const Ray& r, const TriRayPre& pre, V3 v0, V3 v1,
                              V3 v2, float tnear, float tmax, Hit& h) {
  const V3 A = v0 - r.org, B = v1 - r.org, C = v2 - r.org;
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
    // Edge-exact case: redo the 2-D edge functions in double (JCGT 2013 sec. 4).
    U = static_cast<float>(static_cast<double>(Cx) * By - static_cast<double>(Cy) * Bx);
    V = static_cast<float>(static_cast<double>(Ax) * Cy - static_cast<double>(Ay) * Cx);
    W = static_cast<float>(static_cast<double>(Bx) * Ay - static_cast<double>(By) * Ax);
  }
  if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f))
    return false;
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

inline bool intersectSphere(const Ray& r, V3 c, float rad, float tnear,
                            float tmax, Hit& h) {
  const V3 c0 = c - r.org;
  const float rd2 = 1.0f / dot(r.dir, r.dir);
  const float projC0 = dot(c0, r.dir) * rd2;
  const V3 perp = c0 - r.dir * projC0;
  const float l2 = dot(perp, perp);
  const float r2 = rad * rad;
  if (!(l2 <= r2)) return false;
  const float td = std::sqrt((r2 - l2) * rd2);
  const float tf = projC0 - td;
  const float tb = projC0 + td;
  float t;
  if (tf >= tnear && tf <= tmax) t = tf;
  else if (tb >= tnear && tb <= tmax) t = tb;
  else return false;
  h.t = t;
  h.u = 0.0f;
  h.v = 0.0f;
  h.Ng = r.dir * t - c0;
  return true;
}

// Ray vs. the lateral surface of a frustum on axis (base b, unit axis a):
// radial distance rho(hax) = k0 + k1*hax for axial coordinate hax in [h0, h1].
// Float quadratic after moving the ray origin to the ray point closest to the
// frustum's mid-axis point (parameter ts0); roots in the original parameter.
inline int frustumRoots(const Ray& r, V3 b, V3 a, float h0, float h1, float k0,
                        float k1, float* ts, float* hs) {
  const V3 mid = b + a * (0.5f * (h0 + h1));
  const float dd = dot(r.dir, r.dir);
  const float ts0 = dot(mid - r.org, r.dir) / dd;
  const V3 o = r.org + r.dir * ts0;
  const V3 w = o - b;
  const float wa = dot(w, a), da = dot(r.dir, a);
  const V3 wp = w - a * wa;
  const V3 dp = r.dir - a * da;
  const float g0 = k0 + k1 * wa, g1 = k1 * da;
  const float A = dot(dp, dp) - g1 * g1;
  const float B = dot(wp, dp) - g0 * g1;
  const float Cc = dot(wp, wp) - g0 * g0;
  float rr[2];
  int m = 0;
  if (std::fabs(A) <= 1e-12f * dd) {
    if (B == 0.0f) return 0;
    rr[m++] = -Cc / (2.0f * B);
  } else {
    const float disc = B * B - A * Cc;
    if (disc < 0.0f) return 0;
    const float sq = std::sqrt(disc);
    const float q = -(B + std::copysign(sq, B));
    float r0 = q / A, r1 = q != 0.0f ? Cc / q : r0;
    if (r0 > r1) std::swap(r0, r1);
    rr[m++] = r0;
    rr[m++] = r1;
  }
  int n = 0;
  for (int i = 0; i < m; ++i) {
    const float hh = wa + rr[i] * da;
    if (hh >= h0 && hh <= h1 && k0 + k1 * hh >= 0.0f) {
      ts[n] = ts0 + rr[i];
      hs[n] = hh;
      ++n;
    }
  }
  return n;
}

// CONE_LINEAR_CURVE: frustum p0 (r0) -> p1 (r1) with flat caps.
inline bool intersectConeCurve(const Ray& r, V3 p0, float r0, V3 p1, float r1,
                               float tnear, float tmax, Hit& h) {
  const V3 ax = p1 - p0;
  const float L = length(ax);
  if (!(L > 0.0f)) return false;
  const V3 a = ax * (1.0f / L);
  const float k1 = (r1 - r0) / L;
  float ts[2], hs[2];
  const int n = frustumRoots(r, p0, a, 0.0f, L, r0, k1, ts, hs);
  bool found = false;
  float best = tmax;
  for (int i = 0; i < n; ++i) {
    if (ts[i] >= tnear && ts[i] <= best) {
      best = ts[i];
      const V3 P = r.org + r.dir * ts[i];
      const V3 rad = (P - p0) - a * hs[i];
      h.t = ts[i];
      h.u = hs[i] / L;
      h.v = 0.0f;
      h.Ng = rad - a * (k1 * length(rad));
      found = true;
    }
  }
  // flat caps: plane (P - p) . a = 0 within radius
  const float da = dot(r.dir, a);
  if (da != 0.0f) {
    for (int e = 0; e < 2; ++e) {
      const V3 pc = e == 0 ? p0 : p1;
      const float rc = e == 0 ? r0 : r1;
      const float t = dot(pc - r.org, a) / da;
      if (!(t >= tnear && t <= best)) continue;
      const V3 P = r.org + r.dir * t;
      const V3 d = P - pc;
      if (dot(d, d) > rc * rc) continue;
      best = t;
      h.t = t;
      h.u = static_cast<float>(e);
      h.v = 0.0f;
      h.Ng = e == 0 ? a * -1.0f : a;
      found = true;
    }
  }
  return found;
}

// ROUND_LINEAR_CURVE segment with optional bisector clipping planes.
// clipL/clipR are the (unit) bisector normals at p0/p1 (valid when the flag
// bit is set); a hit P is kept when dot(P - p0, clipL) >= 0 and
// dot(P - p1, clipR) <= 0.
inline bool intersectRoundCurve(const Ray& r, V3 p0, float r0, V3 p1, float r1,
                                uint8_t flags, V3 clipL, V3 clipR, float tnear,
                                float tmax, Hit& h) {
  const V3 ax = p1 - p0;
  const float L = length(ax);
  bool found = false;
  float best = tmax;
  auto consider = [&](float t, V3 Ng, float u) {
    if (!(t >= tnear && t <= best)) return;
    const V3 P = r.org + r.dir * t;
    if ((flags & 1u) && dot(P - p0, clipL) < 0.0f) return;
    if ((flags & 2u) && dot(P - p1, clipR) > 0.0f) return;
    best = t;
    h.t = t;
    h.u = u;
    h.v = 0.0f;
    h.Ng = Ng;
    found = true;
  };
  // end spheres (both roots); keep only the cap parts outside the tangent cone
  float sinA = 0.0f, cosA = 1.0f;
  V3 a{0.0f, 0.0f, 1.0f};
  const bool hasCone = L > std::fabs(r0 - r1) && L > 0.0f;
  if (hasCone) {
    a = ax * (1.0f / L);
    sinA = (r0 - r1) / L;
    cosA = std::sqrt(std::max(0.0f, 1.0f - sinA * sinA));
  }
  const float s0 = r0 * sinA, s1 = L + r1 * sinA;  // axial range of the cone
  for (int e = 0; e < 2; ++e) {
    const V3 c = e == 0 ? p0 : p1;
    const float rad = e == 0 ? r0 : r1;
    if (!hasCone && ((e == 0 && r0 < r1) || (e == 1 && r1 <= r0))) continue;
    const V3 c0 = c - r.org;
    const float rd2 = 1.0f / dot(r.dir, r.dir);
    const float pc = dot(c0, r.dir) * rd2;
    const V3 perp = c0 - r.dir * pc;
    const float l2 = dot(perp, perp), rr = rad * rad;
    if (!(l2 <= rr)) continue;
    const float td = std::sqrt((rr - l2) * rd2);
    const float cand[2] = {pc - td, pc + td};
    for (float t : cand) {
      const V3 P = r.org + r.dir * t;
      if (hasCone) {
        const float hh = dot(P - p0, a);
        if (e == 0 && hh > s0) continue;
        if (e == 1 && hh < s1) continue;
      }
      const float u = hasCone ? std::min(1.0f, std::max(0.0f, dot(P - p0, a) / L)) : 0.0f;
      consider(t, r.dir * t - c0, u);
    }
  }
  if (hasCone) {
    const float k0c = r0 * cosA, k1c = (s1 > s0) ? (r1 * cosA - r0 * cosA) / (s1 - s0) : 0.0f;
    float ts[2], hs[2];
    const int n = frustumRoots(r, p0, a, s0, s1, k0c - k1c * s0, k1c, ts, hs);
    for (int i = 0; i < n; ++i) {
      const V3 P = r.org + r.dir * ts[i];
      const V3 rad = (P - p0) - a * hs[i];
      consider(ts[i], rad - a * (k1c * length(rad)),
               std::min(1.0f, std::max(0.0f, hs[i] / L)));
    }
  }
  return found;
}

// ---------------------------------------------------------------------------
// Binned-SAH BVH over all primitives (kind, primID) of a GeomSet.

struct Box {
  V3 lo{1e30f, 1e30f, 1e30f}, hi{-1e30f, -1e30f, -1e30f};
  void grow(V3 p) {
    lo = {std::min(lo.x, p.x), std::min(lo.y, p.y), std::min(lo.z, p.z)};
    hi = {std::max(hi.x, p.x), std::max(hi.y, p.y), std::max(hi.z, p.z)};
  }
  void grow(const Box& b) { grow(b.lo); grow(b.hi); }
  float area() const {
    if (lo.x > hi.x) return 0.0f;
    const V3 e = hi - lo;
    return 2.0f * (e.x * e.y + e.y * e.z + e.z * e.x);
  }
};

struct PrimRef {
  uint32_t kind;
  uint32_t id;
};

class Bvh {
 public:
  struct Node {
    Box box;
    uint32_t left = 0;    // internal: left child index (right = left + 1)
    uint32_t first = 0;   // leaf: first ref
    uint32_t count = 0;   // 0 = internal
  };

  // Curve bisector clip normals, filled by build().
  std::vector<V3> rcClipL, rcClipR;

  void build(const GeomSet* g);
  bool closest(const Ray& r, Hit& h) const;
  bool occluded(const Ray& r) const;
  // any hit that `accept(kind, primID, hit)` takes; a sphere whose entry point
  // is refused offers its exit point
  template <class F>
  bool occludedIf(const Ray& r, F accept) const;
  size_t nodeCount() const { return nodes_.size(); }

 private:
  const GeomSet* g_ = nullptr;
  std::vector<Node> nodes_;
  std::vector<PrimRef> refs_;
  Box primBox(const PrimRef& p) const;
  bool testPrim(const PrimRef& p, const Ray& r, const TriRayPre& pre,
                float tnear, float tmax, Hit& h) const;
  void buildRec(uint32_t node, uint32_t first, uint32_t count,
                std::vector<Box>& boxes, std::vector<V3>& cents, int depth);
};

inline V3 rcVert(const GeomSet& g, uint32_t i) {
  return {g.rcV[4 * i], g.rcV[4 * i + 1], g.rcV[4 * i + 2]};
}
inline V3 ccVert(const GeomSet& g, uint32_t i) {
  return {g.ccV[4 * i], g.ccV[4 * i + 1], g.ccV[4 * i + 2]};
}

inline Box Bvh::primBox(const PrimRef& p) const {
  Box b;
  const GeomSet& g = *g_;
  switch (p.kind) {
    case kMesh:
      for (int k = 0; k < 3; ++k) b.grow(triVert(g, g.triIdx[3 * p.id + k]));
      break;
    case kSphere: {
      const V3 c{g.sph[4 * p.id], g.sph[4 * p.id + 1], g.sph[4 * p.id + 2]};
      const float r = g.sph[4 * p.id + 3];
      b.grow(c - V3(r, r, r));
      b.grow(c + V3(r, r, r));
      break;
    }
    case kRound:
    case kCone: {
      const bool rnd = p.kind == kRound;
      const uint32_t v = rnd ? g.rcIdx[p.id] : g.ccIdx[p.id];
      for (uint32_t k = 0; k < 2; ++k) {
        const V3 c = rnd ? rcVert(g, v + k) : ccVert(g, v + k);
        const float r = rnd ? g.rcV[4 * (v + k) + 3] : g.ccV[4 * (v + k) + 3];
        b.grow(c - V3(r, r, r));
        b.grow(c + V3(r, r, r));
      }
      break;
    }
  }
  // pad by a relative epsilon so flat boxes and rounding never cull a hit
  const V3 e = (b.hi - b.lo) * 1e-6f;
  const float m = 1e-6f * std::max({std::fabs(b.lo.x), std::fabs(b.lo.y), std::fabs(b.lo.z),
                                    std::fabs(b.hi.x), std::fabs(b.hi.y), std::fabs(b.hi.z), 1.0f});
  b.lo = b.lo - V3(e.x + m, e.y + m, e.z + m);
  b.hi = b.hi + V3(e.x + m, e.y + m, e.z + m);
  return b;
}

inline void Bvh::build(const GeomSet* g) {
  g_ = g;
  refs_.clear();
  nodes_.clear();
  for (int kind = 0; kind < 4; ++kind)
    for (size_t i = 0; i < g->count(kind); ++i)
      refs_.push_back({static_cast<uint32_t>(kind), static_cast<uint32_t>(i)});
  // bisector planes of chained round curves
  const size_t nrc = g->rcIdx.size();
  rcClipL.assign(nrc, V3());
  rcClipR.assign(nrc, V3());
  for (size_t s = 0; s < nrc; ++s) {
    const uint32_t v = g->rcIdx[s];
    const V3 p0 = rcVert(*g, v), p1 = rcVert(*g, v + 1);
    const V3 dir = normalize(p1 - p0);
    if (g->rcFlags[s] & 1u) rcClipL[s] = normalize(dir + normalize(p0 - rcVert(*g, v - 1)));
    if (g->rcFlags[s] & 2u) rcClipR[s] = normalize(dir + normalize(rcVert(*g, v + 2) - p1));
  }
  if (refs_.empty()) return;
  std::vector<Box> boxes(refs_.size());
  std::vector<V3> cents(refs_.size());
  for (size_t i = 0; i < refs_.size(); ++i) {
    boxes[i] = primBox(refs_[i]);
    cents[i] = (boxes[i].lo + boxes[i].hi) * 0.5f;
  }
  nodes_.reserve(2 * refs_.size());
  nodes_.push_back(Node{});
  buildRec(0, 0, static_cast<uint32_t>(refs_.size()), boxes, cents, 0);
}

inline void Bvh::buildRec(uint32_t node, uint32_t first, uint32_t count,
                          std::vector<Box>& boxes, std::vector<V3>& cents,
                          int depth) {
  Box nb, cb;
  for (uint32_t i = first; i < first + count; ++i) {
    nb.grow(boxes[i]);
    cb.grow(cents[i]);
  }
  nodes_[node].box = nb;
  if (count <= 4 || depth > 48) {
    nodes_[node].first = first;
    nodes_[node].count = count;
    return;
  }
  constexpr int kBins = 16;
  int bestAxis = -1, bestSplit = -1;
  float bestCost = std::numeric_limits<float>::infinity();
  for (int axis = 0; axis < 3; ++axis) {
    const float lo = comp(cb.lo, axis), hi = comp(cb.hi, axis);
    if (!(hi > lo)) continue;
    Box bb[kBins];
    int bc[kBins] = {0};
    const float sc = kBins / (hi - lo);
    for (uint32_t i = first; i < first + count; ++i) {
      int b = static_cast<int>((comp(cents[i], axis) - lo) * sc);
      b = std::min(kBins - 1, std::max(0, b));
      bb[b].grow(boxes[i]);
      ++bc[b];
    }
    Box lb[kBins];
    int lc[kBins];
    Box acc;
    int n = 0;
    for (int b = 0; b < kBins; ++b) {
      acc.grow(bb[b]);
      n += bc[b];
      lb[b] = acc;
      lc[b] = n;
    }
    acc = Box();
    n = 0;
    for (int b = kBins - 1; b > 0; --b) {
      acc.grow(bb[b]);
      n += bc[b];
      if (lc[b - 1] == 0 || n == 0) continue;
      const float cost = lb[b - 1].area() * lc[b - 1] + acc.area() * n;
      if (cost < bestCost) {
        bestCost = cost;
        bestAxis = axis;
        bestSplit = b;
      }
    }
  }
  uint32_t mid = first + count / 2;
  if (bestAxis >= 0) {
    const float lo = comp(cb.lo, bestAxis), hi = comp(cb.hi, bestAxis);
    const float sc = kBins / (hi - lo);
    uint32_t i = first, j = first + count;
    while (i < j) {
      int b = static_cast<int>((comp(cents[i], bestAxis) - lo) * sc);
      b = std::min(kBins - 1, std::max(0, b));
      if (b < bestSplit) {
        ++i;
      } else {
        --j;
        std::swap(refs_[i], refs_[j]);
        std::swap(boxes[i], boxes[j]);
        std::swap(cents[i], cents[j]);
      }
    }
    mid = i;
    if (mid == first || mid == first + count) mid = first + count / 2;
  }
  const uint32_t left = static_cast<uint32_t>(nodes_.size());
  nodes_[node].left = left;
  nodes_[node].count = 0;
  nodes_.push_back(Node{});
  nodes_.push_back(Node{});
  buildRec(left, first, mid - first, boxes, cents, depth + 1);
  buildRec(left + 1, mid, first + count - mid, boxes, cents, depth + 1);
}

inline bool Bvh::testPrim(const PrimRef& p, const Ray& r, const TriRayPre& pre,
                          float tnear, float tmax, Hit& h) const {
  const GeomSet& g = *g_;
  switch (p.kind) {
    case kMesh:
      return intersectTriangle(r, pre, triVert(g, g.triIdx[3 * p.id]),
                               triVert(g, g.triIdx[3 * p.id + 1]),
                               triVert(g, g.triIdx[3 * p.id + 2]), tnear, tmax, h);
    case kSphere:
      return intersectSphere(r, V3(g.sph[4 * p.id], g.sph[4 * p.id + 1], g.sph[4 * p.id + 2]),
                             g.sph[4 * p.id + 3], tnear, tmax, h);
    case kRound: {
      const uint32_t v = g.rcIdx[p.id];
      return intersectRoundCurve(r, rcVert(g, v), g.rcV[4 * v + 3], rcVert(g, v + 1),
                                 g.rcV[4 * v + 7], g.rcFlags[p.id], rcClipL[p.id],
                                 rcClipR[p.id], tnear, tmax, h);
    }
    default: {
      const uint32_t v = g.ccIdx[p.id];
      return intersectConeCurve(r, ccVert(g, v), g.ccV[4 * v + 3], ccVert(g, v + 1),
                                g.ccV[4 * v + 7], tnear, tmax, h);
    }
  }
}

inline bool slab(const Box& b, const V3& o, const V3& inv, float tnear, float tfar,
                 float& tEntry) {
  float t0 = tnear, t1 = tfar;
  for (int k = 0; k < 3; ++k) {
    const float ta = (comp(b.lo, k) - comp(o, k)) * comp(inv, k);
    const float tb = (comp(b.hi, k) - comp(o, k)) * comp(inv, k);
    const float mn = std::min(ta, tb), mx = std::max(ta, tb);
    if (!std::isnan(mn)) t0 = std::max(t0, mn);
    if (!std::isnan(mx)) t1 = std::min(t1, mx);
  }
  tEntry = t0;
  return t0 <= t1;
}

inline V3 safeInv(V3 d) {
  auto f = [](float x) {
    if (std::fabs(x) < 1e-30f) x = std::copysign(1e-30f, x);
    return 1.0f / x;
  };
  return {f(d.x), f(d.y), f(d.z)};
}

inline bool Bvh::closest(const Ray& r, Hit& best) const {
  best.geomID = kInvalid;
  if (nodes_.empty()) return false;
  const V3 inv = safeInv(r.dir);
  const TriRayPre pre = triPre(r.dir);
  float tmax = r.tfar;
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const Node& n = nodes_[stack[--sp]];
    float te;
    if (!slab(n.box, r.org, inv, r.tnear, tmax, te)) continue;
    if (n.count > 0) {
      for (uint32_t i = n.first; i < n.first + n.count; ++i) {
        const PrimRef& p = refs_[i];
        Hit h;
        if (!testPrim(p, r, pre, r.tnear, tmax, h)) continue;
        const uint32_t gid = g_->geomID[p.kind];
        const bool better =
            best.geomID == kInvalid || h.t < best.t ||
            (h.t == best.t && (gid < best.geomID || (gid == best.geomID && p.id < best.primID)));
        if (!better) continue;
        h.geomID = gid;
        h.primID = p.id;
        best = h;
        tmax = h.t;
      }
    } else {
      float tl, tr;
      const bool hl = slab(nodes_[n.left].box, r.org, inv, r.tnear, tmax, tl);
      const bool hr = slab(nodes_[n.left + 1].box, r.org, inv, r.tnear, tmax, tr);
      if (hl && hr) {
        if (tl <= tr) { stack[sp++] = n.left + 1; stack[sp++] = n.left; }
        else { stack[sp++] = n.left; stack[sp++] = n.left + 1; }
      } else if (hl) {
        stack[sp++] = n.left;
      } else if (hr) {
        stack[sp++] = n.left + 1;
      }
    }
  }
  return best.geomID != kInvalid;
}

inline bool Bvh::occluded(const Ray& r) const {
  if (nodes_.empty()) return false;
  if (!(r.tnear <= r.tfar)) return false;
  const V3 inv = safeInv(r.dir);
  const TriRayPre pre = triPre(r.dir);
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const Node& n = nodes_[stack[--sp]];
    float te;
    if (!slab(n.box, r.org, inv, r.tnear, r.tfar, te)) continue;
    if (n.count > 0) {
      for (uint32_t i = n.first; i < n.first + n.count; ++i) {
        Hit h;
        if (testPrim(refs_[i], r, pre, r.tnear, r.tfar, h)) return true;
      }
    } else {
      stack[sp++] = n.left;
      stack[sp++] = n.left + 1;
    }
  }
  return false;
}

template <class F>
inline bool Bvh::occludedIf(const Ray& r, F accept) const {
  if (nodes_.empty()) return false;
  if (!(r.tnear <= r.tfar)) return false;
  const V3 inv = safeInv(r.dir);
  const TriRayPre pre = triPre(r.dir);
  uint32_t stack[128];
  int sp = 0;
  stack[sp++] = 0;
  while (sp > 0) {
    const Node& n = nodes_[stack[--sp]];
    float te;
    if (!slab(n.box, r.org, inv, r.tnear, r.tfar, te)) continue;
    if (n.count > 0) {
      for (uint32_t i = n.first; i < n.first + n.count; ++i) {
        const PrimRef& p = refs_[i];
        Hit h;
        if (!testPrim(p, r, pre, r.tnear, r.tfar, h)) continue;
        if (accept(p.kind, p.id, h)) return true;
        if (p.kind == kSphere) {
          Hit h2;
          if (testPrim(p, r, pre, std::nextafter(h.t, std::numeric_limits<float>::infinity()), r.tfar, h2) &&
              accept(p.kind, p.id, h2))
            return true;
        }
      }
    } else {
      stack[sp++] = n.left;
      stack[sp++] = n.left + 1;
    }
  }
  return false;
}

}  // namespace oracle

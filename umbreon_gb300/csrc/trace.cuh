// trace.cuh -- device building blocks shared by the frame kernels and the
// adjoint: primary rays, 8-wide BVH traversal, shading surface, sample
// streams (tea2, cosine hemisphere, low-discrepancy AO), warp counters.
#pragma once

#include "ubr_context.h"

namespace ubr {
namespace {

constexpr int kStackDepth = 32;  // group entries: one per tree level
constexpr float kInfF = __builtin_huge_valf();

UBR_D f3 ld3(const float4 v) { return f3{v.x, v.y, v.z}; }

UBR_D f3 safeInv(f3 d) {
  auto f = [](float x) {
    if (fabsf(x) < 1e-30f) x = copysignf(1e-30f, x);
    return 1.0f / x;
  };
  return f3{f(d.x), f(d.y), f(d.z)};
}

// Primary ray of hi-res pixel (px, py): embree_renderer.cpp:1399-1414.
UBR_D void primaryRay(const Params& p, int px, int py, f3& org, f3& rd) {
  const float v = 1.0f - 2.0f * (float(py) + 0.5f) / float(p.H);
  const float u = 2.0f * (float(px) + 0.5f) / float(p.W) - 1.0f;
  if (p.ortho) {
    org = p.camPos + p.right * (u * p.halfW) + p.up * (v * p.halfH);
    rd = p.camDir;
  } else {
    org = p.camPos;
    rd = normalize(p.camDir + p.right * (u * p.persHalfW) + p.up * (v * p.persHalfH));
  }
}

// clipRangeT (transparency.hpp:118-129)
UBR_D void clipRange(const Params& p, f3 rd, float& tn, float& tf) {
  tn = 0.0f;
  tf = kInfF;
  if (p.clipNear <= -kInfF && p.clipFar >= kInfF) return;
  const float cosr = dot(rd, p.camDir);
  if (cosr <= 1.0e-6f) return;
  if (p.clipNear > 0.0f) tn = p.clipNear / cosr;
  if (p.clipFar < kInfF) tf = p.clipFar / cosr;
}

// clipRangeT's `on` (transparency.hpp:118-129): clip planes set and the ray
// not degenerate or backward
UBR_D bool clipOn(const Params& p, f3 rd) {
  if (p.clipNear <= -kInfF && p.clipFar >= kInfF) return false;
  return !(dot(rd, p.camDir) <= 1.0e-6f);
}

UBR_D bool slabHit(float lox, float hix, float loy, float hiy, float loz, float hiz, const f3& o,
                   const f3& inv, float tnear, float tmax, float& tEntry) {
  const float t0x = (lox - o.x) * inv.x, t1x = (hix - o.x) * inv.x;
  const float t0y = (loy - o.y) * inv.y, t1y = (hiy - o.y) * inv.y;
  const float t0z = (loz - o.z) * inv.z, t1z = (hiz - o.z) * inv.z;
  const float tmin = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tnear));
  const float tmx = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
  tEntry = tmin;
  return tmin <= tmx;
}

// Kind masks: bit k set when primitives of kind k exist.  Kernels are
// instantiated per mask so a scene only carries the intersectors it needs.
constexpr int kMaskMesh = 1 << kMesh, kMaskSphere = 1 << kSphere, kMaskRound = 1 << kRound,
              kMaskCone = 1 << kCone, kMaskAll = 15;

// Kinds present in a mask: their number, the lowest and the highest.
__host__ __device__ constexpr int kindCount(int km) { return (km & 1) + ((km >> 1) & 1) + ((km >> 2) & 1) + ((km >> 3) & 1); }
__host__ __device__ constexpr int lowKind(int km) { return (km & 1) ? 0 : (km & 2) ? 1 : (km & 4) ? 2 : 3; }
__host__ __device__ constexpr int highKind(int km) { return (km & 8) ? 3 : (km & 4) ? 2 : (km & 2) ? 1 : 0; }

// Test of the primitive in leaf slot `slot` whose kind is known; a round
// segment needs its reference (`ref`, or kInvalid to load it).
template <int KIND, bool ATTR>
UBR_D bool testKnown(const TravScene& s, int slot, const Ray& r, const TriPre& pre, float tnear, float tmax,
                     Hit& h, uint32_t ref) {
  const float4* g = s.leafGeo + kLeafF4 * slot;
  if (KIND == kSphere) {
    const float4 q = __ldg(g);
    return isectSphere<ATTR>(r, f3{q.x, q.y, q.z}, q.w, tnear, tmax, h);
  }
  if (KIND == kMesh) {
    const float4 a = __ldg(g), b = __ldg(g + 1), c = __ldg(g + 2);
    return isectTriangle(r, pre, ld3(a), ld3(b), ld3(c), tnear, tmax, h);
  }
  const float4 a = __ldg(g), b = __ldg(g + 1);
  if (KIND == kCone) {
    const float4 ax = __ldg(g + 2);
    return isectConeCurveAxis<ATTR>(r, ld3(a), a.w, ld3(b), b.w, ld3(ax), ax.w, tnear, tmax, h);
  }
  if (ref == kInvalid) ref = __ldg(&s.leafRef[slot]);
  const uint32_t prim = refPrim(ref);
  const uint32_t flags = __float_as_uint(__ldg(g + 2).x);
  const float4 cl = __ldg(&s.rcClip[2 * prim]), cr = __ldg(&s.rcClip[2 * prim + 1]);
  return isectRoundCurve(r, ld3(a), a.w, ld3(b), b.w, flags, ld3(cl), ld3(cr), tnear, tmax, h);
}

template <int KM, bool ATTR = true>
UBR_D bool testLeaf(const TravScene& s, int slot, const Ray& r, const TriPre& pre, float tnear,
                    float tmax, Hit& h, uint32_t& ref) {
  ref = __ldg(&s.leafRef[slot]);
  const int kind = refKind(ref);
  constexpr bool single = (KM & (KM - 1)) == 0;
  if ((KM & kMaskSphere) && (single || kind == kSphere)) return testKnown<kSphere, ATTR>(s, slot, r, pre, tnear, tmax, h, ref);
  if ((KM & kMaskMesh) && (single || kind == kMesh)) return testKnown<kMesh, ATTR>(s, slot, r, pre, tnear, tmax, h, ref);
  if ((KM & kMaskCone) && (!(KM & kMaskRound) || kind == kCone))
    return testKnown<kCone, ATTR>(s, slot, r, pre, tnear, tmax, h, ref);
  if (KM & kMaskRound) return testKnown<kRound, ATTR>(s, slot, r, pre, tnear, tmax, h, ref);
  return false;
}

// Stack traversal of the binary LBVH, near child first.  ANY: return at the
// first hit in [tnear, tfar].  Closest: smallest t, ties to lowest
// (geomID, primID).
// Bytes of the leaf record fetched for one primitive test, by kind
// (leafRef 4 B + geometry float4s; round segments add their 32 B clip planes).
UBR_D uint32_t leafBytes(int kind) {
  return kind == kSphere ? 20u : kind == kMesh ? 52u : kind == kCone ? 36u : 84u;
}

struct Count {
  uint32_t nodes = 0, primBytes = 0;
};

// One kind's any-hit tests over the primitive slots of `mask` (a phase of
// the kind-split leaf loop): true at the first hit.
template <bool COUNT, int KIND>
UBR_D bool anyHitPhase(const TravScene& s, const Ray& r, const TriPre& pre, int primBase, uint32_t mask, float tmax,
                       Hit& best, Count* cnt) {
  for (; mask; mask &= mask - 1u) {
    const int q = __ffs(mask) - 1;
    if (COUNT) cnt->primBytes += leafBytes(KIND);
    Hit h;
    if (testKnown<KIND, false>(s, primBase + q, r, pre, r.tnear, tmax, h, kInvalid)) {
      best = h;
      best.ref = packRef(KIND, 0);  // a hit marker: binary queries read no ids
      return true;
    }
  }
  return false;
}

// Stack traversal of the 8-wide BVH (node/primitive groups after Ylitie,
// Karras and Laine, HPG 2017).  Visiting a node is branch-free: each child's
// slab planes are one fmaf each from the 8-bit bounds, giving a hit mask;
// the nearest hit internal child is visited next and the other hit internal
// children are pushed as ONE group entry (childBase << 8 | slot mask), so the
// stack depth is the tree depth; hit leaves expand into a mask over the
// node's contiguous primitive block, tested in one loop.  The slab interval
// is widened by a relative 2^-19 so quantised boxes stay conservative under
// float rounding at any camera distance.  any: return at the first hit in
// [tnear, tfar]; otherwise the closest hit, ties to the lowest
// (geomID, primID).
constexpr float kSlabGrow = 1.0f + 0x1.0p-19f;

// Byte b of word q as a float, without an integer->float conversion: place
// the byte in the mantissa of 2^23 (byte permute) and subtract 2^23 (exact).
UBR_D float byteToFloat(uint32_t q, int b) {
  return __uint_as_float(__byte_perm(q, 0x4B000000u, 0x7540u + uint32_t(b))) - 8388608.0f;
}

// Packed pairs of floats for the slab test of two children at once:
// sm_100-family add/mul/fma on .f32x2 round each lane like the scalar
// instruction (round to nearest even), so the pair form gives the same bits
// as two scalar operations with half the instructions issued.
typedef unsigned long long f2x;
UBR_D f2x pk2(float a, float b) {
  f2x r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
UBR_D void up2(f2x v, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
UBR_D f2x fma2(f2x a, f2x b, f2x c) {
  f2x d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
UBR_D f2x add2(f2x a, f2x b) {
  f2x d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
UBR_D f2x mul2(f2x a, f2x b) {
  f2x d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// Bytes b and b+1 of q as a float pair (byteToFloat on both).
UBR_D f2x bytePairToFloat2(uint32_t q, int b, f2x bias) {
  return add2(pk2(__uint_as_float(__byte_perm(q, 0x4B000000u, 0x7540u + uint32_t(b))),
                  __uint_as_float(__byte_perm(q, 0x4B000000u, 0x7540u + uint32_t(b + 1)))),
              bias);
}

// Slot of the nearest hit internal child (-1: none): the smallest key among
// the hit slots, a key being the entry distance's bits with the slot in the
// low three bits (one integer min per child instead of a compare and two
// selects).  Non-negative floats order as unsigned integers; distances within
// 8 ulps go to the lower slot.  The visiting order never changes an answer:
// an any-hit query reports whether some primitive is hit, a closest-hit query
// the nearest hit with ties to the lowest ids.
UBR_D int nearestChild(const float (&tmin)[8], uint32_t hitInt) {
  uint32_t best = 0xFFFFFFFFu;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const uint32_t key = (__float_as_uint(tmin[k]) & ~7u) | uint32_t(k);
    best = ((hitInt >> k) & 1u) ? min(best, key) : best;
  }
  return hitInt ? int(best & 7u) : -1;
}

// Traversal state of one ray, resumable one node at a time (the persistent
// occlusion kernel interleaves rays at node granularity).
struct TravState {
  int node;                      // node to visit next
  int sp;
  uint32_t steps;
  float tmax;
  uint32_t bestGeom, bestPrim;
  uint32_t stack[kStackDepth];   // group entries: (childBase << 8) | slot mask
};

UBR_D void travInit(const Ray& r, TravState& st, Hit& best, int start = 0) {
  st.node = start;
  st.sp = 0;
  st.steps = 0;
  st.tmax = r.tfar;
  st.bestGeom = kInvalid;
  st.bestPrim = kInvalid;
  best.ref = kInvalid;
}

// Visit st.node: test its 8 children, its hit leaves' primitives, choose the
// next node.  Returns true when the ray is finished (any-hit found, stack
// empty, or the step bound reached).
// Candidate-hit filter of the stroke-edge pass's visibility rays
// (excludeFaceFilter, embree_renderer.cpp:76-133): a hit is not an occluder
// when it lies on one of the segment's own mesh faces (primID modulo the base
// triangle count), when the ray meets its face at |cos| <= grazeCos, or when
// the face's plane passes within `coplanar` of the ray origin.
struct HitFilter {
  const int32_t* faces;  // excluded base-triangle ids
  int nFaces;
  uint32_t baseTri;      // triangles per instance (0: not instanced)
  float grazeCos, coplanar;
};
UBR_D bool filterAccept(const HitFilter& f, const Ray& r, const Hit& h, uint32_t ref) {
  if (f.nFaces > 0 && refKind(ref) == kMesh) {
    uint32_t prim = refPrim(ref);
    if (f.baseTri > 0) prim %= f.baseTri;
    for (int k = 0; k < f.nFaces; ++k)
      if (uint32_t(__ldg(&f.faces[k])) == prim) return false;
  }
  if (f.grazeCos > 0.0f || f.coplanar > 0.0f) {
    const float nx = h.Ng.x, ny = h.Ng.y, nz = h.Ng.z;
    const float dx = r.dir.x, dy = r.dir.y, dz = r.dir.z;
    const float nlen = sqrtf(nx * nx + ny * ny + nz * nz);
    const float dlen = sqrtf(dx * dx + dy * dy + dz * dz);
    if (nlen > 0.0f && dlen > 0.0f) {
      const float dDotN = nx * dx + ny * dy + nz * dz;
      const float c = fabsf(dDotN) / (nlen * dlen);
      if (f.grazeCos > 0.0f && c <= f.grazeCos) return false;
      if (f.coplanar > 0.0f) {
        const float perp = h.t * fabsf(dDotN) / nlen;
        if (perp <= f.coplanar) return false;
      }
    }
  }
  return true;
}

// Wide nodes 0..kTopNodes-1 are the root and the two levels below it (the
// collapse numbers nodes level by level); a kernel may stage them in shared
// memory and pass them as `top` (nTop of them).
constexpr int kTopNodes = 73;

template <bool COUNT, int KM, bool ALWAYS_ANY = false, bool FILTER = false>
UBR_D bool travStep(const TravScene& s, const Ray& r, const f3& inv, const TriPre& pre, TravState& st, Hit& best,
                    uint32_t& overflow, Count* cnt, bool any, const float4* top = nullptr, int nTop = 0,
                    const HitFilter* flt = nullptr) {
  if (ALWAYS_ANY) any = true;
  if (++st.steps > s.primCount + 16u) {  // each node at most once per ray in a valid tree
    ++overflow;
    return true;
  }
  if (COUNT) ++cnt->nodes;
  float4 n0, n1, n2, n3, n4;
  if (nTop > 0 && st.node < nTop) {  // folds away where no nodes are staged
    const float4* nd = top + kWideF4 * st.node;
    n0 = nd[0];
    n1 = nd[1];
    n2 = nd[2];
    n3 = nd[3];
    n4 = nd[4];
  } else {
    const float4* nd = s.wnodes + kWideF4 * st.node;
    n0 = __ldg(nd);
    n1 = __ldg(nd + 1);
    n2 = __ldg(nd + 2);
    n3 = __ldg(nd + 3);
    n4 = __ldg(nd + 4);
  }
  const uint32_t hdr = __float_as_uint(n0.w);
  const float sx = __uint_as_float((hdr & 0xFFu) << 23) * inv.x;
  const float sy = __uint_as_float(((hdr >> 8) & 0xFFu) << 23) * inv.y;
  const float sz = __uint_as_float(((hdr >> 16) & 0xFFu) << 23) * inv.z;
  const int nInt = int((hdr >> 24) & 0xFu);
  const float ox = (n0.x - r.org.x) * inv.x, oy = (n0.y - r.org.y) * inv.y, oz = (n0.z - r.org.z) * inv.z;
  const uint32_t childBase = __float_as_uint(n1.x);
  const int primBase = __float_as_int(n1.y);
  const uint32_t meta0 = __float_as_uint(n1.z), meta1 = __float_as_uint(n1.w);
  // near/far planes per axis by the sign of the direction (swap lo/hi words)
  const bool nx = inv.x < 0.0f, ny = inv.y < 0.0f, nz = inv.z < 0.0f;
  const uint32_t qnx[2] = {nx ? __float_as_uint(n3.z) : __float_as_uint(n2.x),
                           nx ? __float_as_uint(n3.w) : __float_as_uint(n2.y)};
  const uint32_t qfx[2] = {nx ? __float_as_uint(n2.x) : __float_as_uint(n3.z),
                           nx ? __float_as_uint(n2.y) : __float_as_uint(n3.w)};
  const uint32_t qny[2] = {ny ? __float_as_uint(n4.x) : __float_as_uint(n2.z),
                           ny ? __float_as_uint(n4.y) : __float_as_uint(n2.w)};
  const uint32_t qfy[2] = {ny ? __float_as_uint(n2.z) : __float_as_uint(n4.x),
                           ny ? __float_as_uint(n2.w) : __float_as_uint(n4.y)};
  const uint32_t qnz[2] = {nz ? __float_as_uint(n4.z) : __float_as_uint(n3.x),
                           nz ? __float_as_uint(n4.w) : __float_as_uint(n3.y)};
  const uint32_t qfz[2] = {nz ? __float_as_uint(n3.x) : __float_as_uint(n4.z),
                           nz ? __float_as_uint(n3.y) : __float_as_uint(n4.w)};
  const f2x bias2 = pk2(-8388608.0f, -8388608.0f), grow2 = pk2(kSlabGrow, kSlabGrow);
  const f2x sx2 = pk2(sx, sx), sy2 = pk2(sy, sy), sz2 = pk2(sz, sz);
  const f2x ox2 = pk2(ox, ox), oy2 = pk2(oy, oy), oz2 = pk2(oz, oz);
  float tminP[8];
  uint32_t gap[8];  // bits of tmax * grow - tmin per slot: sign clear = hit
#pragma unroll
  for (int k = 0; k < 8; k += 2) {
    const int w = k >> 2, b = k & 3;
    float tnx[2], tfx[2], tny[2], tfy[2], tnz[2], tfz[2];
    up2(fma2(bytePairToFloat2(qnx[w], b, bias2), sx2, ox2), tnx[0], tnx[1]);
    up2(fma2(bytePairToFloat2(qfx[w], b, bias2), sx2, ox2), tfx[0], tfx[1]);
    up2(fma2(bytePairToFloat2(qny[w], b, bias2), sy2, oy2), tny[0], tny[1]);
    up2(fma2(bytePairToFloat2(qfy[w], b, bias2), sy2, oy2), tfy[0], tfy[1]);
    up2(fma2(bytePairToFloat2(qnz[w], b, bias2), sz2, oz2), tnz[0], tnz[1]);
    up2(fma2(bytePairToFloat2(qfz[w], b, bias2), sz2, oz2), tfz[0], tfz[1]);
    float tmx[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      tminP[k + j] = fmaxf(fmaxf(tnx[j], tny[j]), fmaxf(tnz[j], r.tnear));
      tmx[j] = fminf(fminf(tfx[j], tfy[j]), fminf(tfz[j], st.tmax));
    }
    float g0, g1;
    up2(fma2(pk2(tmx[0], tmx[1]), grow2, pk2(-tminP[k], -tminP[k + 1])), g0, g1);
    gap[k] = __float_as_uint(g0);
    gap[k + 1] = __float_as_uint(g1);
  }
  // slot mask of the hit children: the sign bytes of the eight gaps gathered
  // into two words, their sign bits moved to bits 28-31 by one multiply
  // (partial products land on distinct bits below 28, so nothing carries).
  const uint32_t sx4 = __byte_perm(__byte_perm(gap[0], gap[1], 0x0073u), __byte_perm(gap[2], gap[3], 0x0073u), 0x5410u);
  const uint32_t sy4 = __byte_perm(__byte_perm(gap[4], gap[5], 0x0073u), __byte_perm(gap[6], gap[7], 0x0073u), 0x5410u);
  const uint32_t neg = (((sx4 & 0x80808080u) * 0x00204081u) >> 28) | ((((sy4 & 0x80808080u) * 0x00204081u) >> 24) & 0xF0u);
  const uint32_t hitMask = ~neg & 0xFFu;
  const uint32_t hitInt = hitMask & ((1u << nInt) - 1u);
  // each hit leaf's meta byte (count << 5 | offset) adds its primitives
  uint32_t primMask = 0;
  for (uint32_t leafHit = hitMask & ~hitInt; leafHit; leafHit &= leafHit - 1u) {
    const int k = __ffs(leafHit) - 1;
    const uint32_t m = __byte_perm(k < 4 ? meta0 : meta1, 0u, 0x4440u | uint32_t(k & 3));
    primMask |= ((1u << (m >> 5)) - 1u) << (m & 31u);
  }
  const int nearK = nearestChild(tminP, hitInt);
  // primitives of the hit leaves.  Binary any-hit queries (no filter) of a
  // scene of two analytic kinds split them by kind: all lanes of a warp test
  // one kind, then the other (a mixed loop runs both intersectors in every
  // step where the lanes' kinds differ; spheres and capped cylinders of a
  // ball-and-stick model mix in most leaves: -1.3 % in the occlusion kernel).
  // Not with triangles: a surface with a few atoms rarely mixes, and the pass
  // over the references costs more than it saves (+3.9 %).  A one-kind scene
  // reads no primitive references.
  constexpr bool kSplit = ALWAYS_ANY && !FILTER && kindCount(KM) == 2 && !(KM & kMaskMesh);
  constexpr bool kKnown = ALWAYS_ANY && !FILTER && kindCount(KM) == 1;
  if (kSplit) {
    uint32_t maskHigh = 0;
    for (uint32_t m = primMask; m; m &= m - 1u) {
      const int q = __ffs(m) - 1;
      if (refKind(__ldg(&s.leafRef[primBase + q])) == highKind(KM)) maskHigh |= 1u << q;
    }
    if (anyHitPhase<COUNT, lowKind(KM)>(s, r, pre, primBase, primMask & ~maskHigh, st.tmax, best, cnt) ||
        anyHitPhase<COUNT, highKind(KM)>(s, r, pre, primBase, maskHigh, st.tmax, best, cnt))
      return true;
    primMask = 0;
  } else if (kKnown) {
    if (anyHitPhase<COUNT, lowKind(KM)>(s, r, pre, primBase, primMask, st.tmax, best, cnt)) return true;
    primMask = 0;
  }
  while (primMask) {
    const int q = __ffs(primMask) - 1;
    primMask &= primMask - 1u;
    Hit h;
    uint32_t ref;
    const bool hitLeaf = testLeaf<KM, !ALWAYS_ANY>(s, primBase + q, r, pre, r.tnear, st.tmax, h, ref);
    if (COUNT) cnt->primBytes += leafBytes(refKind(ref));
    if (!hitLeaf) continue;
    if (FILTER && !filterAccept(*flt, r, h, ref)) {
      // a rejected sphere entry still leaves its exit point as a candidate
      bool second = false;
      if (refKind(ref) == kSphere) {
        const float4 q4 = __ldg(s.leafGeo + kLeafF4 * (primBase + q));
        Hit h2;
        second = isectSphere<true>(r, f3{q4.x, q4.y, q4.z}, q4.w, nextafterf(h.t, kInfF), st.tmax, h2) &&
                 filterAccept(*flt, r, h2, ref);
        if (second) h = h2;
      }
      if (!second) continue;
    }
    if (any) {
      best = h;
      best.ref = ref;
      return true;
    }
    const int kind = refKind(ref);
    const uint32_t gid = s.geomID[kind], prim = refPrim(ref);
    const bool better = best.ref == kInvalid || h.t < best.t ||
                        (h.t == best.t && (gid < st.bestGeom || (gid == st.bestGeom && prim < st.bestPrim)));
    if (better) {
      best = h;
      best.ref = ref;
      st.bestGeom = gid;
      st.bestPrim = prim;
      st.tmax = h.t;
    }
  }
  if (nearK >= 0) {
    const uint32_t rest = hitInt & ~(1u << nearK);
    if (rest) {
      if (st.sp < kStackDepth) st.stack[st.sp++] = (childBase << 8) | rest;
      else ++overflow;
    }
    st.node = int(childBase) + nearK;
    return false;
  }
  if (st.sp == 0) return true;
  const uint32_t g = st.stack[st.sp - 1];
  const uint32_t mask = g & 0xFFu;
  const int k = __ffs(mask) - 1;
  const uint32_t left = mask & (mask - 1u);
  if (left) st.stack[st.sp - 1] = (g & ~0xFFu) | left;
  else --st.sp;
  st.node = int(g >> 8) + k;
  return false;
}

// Whole traversal of one ray (one thread per ray).
template <bool COUNT = false, int KM = kMaskAll, bool ALWAYS_ANY = false, bool FILTER = false>
__device__ bool traverse(const TravScene& s, const Ray& r, Hit& best, uint32_t& overflow, Count* cnt,
                         const bool any, int start = 0, const float4* top = nullptr, int nTop = 0,
                         const HitFilter* flt = nullptr) {
  best.ref = kInvalid;
  if (s.primCount == 0 || start < 0) return false;
  const f3 inv = safeInv(r.dir);
  TriPre pre;
  if (KM & kMaskMesh) pre = triPre(r.dir);
  TravState st;
  travInit(r, st, best, start);
  while (!travStep<COUNT, KM, ALWAYS_ANY, FILTER>(s, r, inv, pre, st, best, overflow, cnt, any, top, nTop, flt)) {
  }
  return best.ref != kInvalid;
}

// Any-hit traversal that interleaves node visits and primitive tests one at
// a time (the "if-if" loop of Aila and Laine, "Understanding the Efficiency of
// Ray Traversal on GPUs", HPG 2009): each iteration a lane either tests ONE
// pending primitive of the leaves it found, or, with none pending, visits one
// node.  A lane with several primitives to test no longer holds the whole
// warp in a leaf loop while the other lanes wait; they make node steps in the
// same iterations.  Same node slab test, visiting order and primitive tests
// as travStep, so the answer is the same.
template <bool COUNT, int KM>
__device__ bool traverseAnyInterleaved(const TravScene& s, const Ray& r, uint32_t& overflow, Count* cnt,
                                       int start) {
  if (s.primCount == 0 || start < 0) return false;
  const f3 inv = safeInv(r.dir);
  TriPre pre;
  if (KM & kMaskMesh) pre = triPre(r.dir);
  int node = start, sp = 0, pendBase = 0;
  uint32_t pendMask = 0, steps = 0;
  uint32_t stack[kStackDepth];
  const bool nx = inv.x < 0.0f, ny = inv.y < 0.0f, nz = inv.z < 0.0f;
  const f2x bias2 = pk2(-8388608.0f, -8388608.0f), grow2 = pk2(kSlabGrow, kSlabGrow);
  for (;;) {
    if (pendMask) {
      const int q = __ffs(pendMask) - 1;
      pendMask &= pendMask - 1u;
      Hit h;
      uint32_t ref;
      const bool hit = testLeaf<KM, false>(s, pendBase + q, r, pre, r.tnear, r.tfar, h, ref);
      if (COUNT) cnt->primBytes += leafBytes(refKind(ref));
      if (hit) return true;
      continue;
    }
    if (node < 0) return false;
    if (++steps > s.primCount + 16u) {
      ++overflow;
      return false;
    }
    if (COUNT) ++cnt->nodes;
    const float4* nd = s.wnodes + kWideF4 * node;
    const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3), n4 = __ldg(nd + 4);
    const uint32_t hdr = __float_as_uint(n0.w);
    const float sx = __uint_as_float((hdr & 0xFFu) << 23) * inv.x;
    const float sy = __uint_as_float(((hdr >> 8) & 0xFFu) << 23) * inv.y;
    const float sz = __uint_as_float(((hdr >> 16) & 0xFFu) << 23) * inv.z;
    const int nInt = int((hdr >> 24) & 0xFu), nCh = int(hdr >> 28);
    const float ox = (n0.x - r.org.x) * inv.x, oy = (n0.y - r.org.y) * inv.y, oz = (n0.z - r.org.z) * inv.z;
    const uint32_t childBase = __float_as_uint(n1.x);
    const int primBase = __float_as_int(n1.y);
    const uint32_t meta0 = __float_as_uint(n1.z), meta1 = __float_as_uint(n1.w);
    const uint32_t qnx[2] = {nx ? __float_as_uint(n3.z) : __float_as_uint(n2.x),
                             nx ? __float_as_uint(n3.w) : __float_as_uint(n2.y)};
    const uint32_t qfx[2] = {nx ? __float_as_uint(n2.x) : __float_as_uint(n3.z),
                             nx ? __float_as_uint(n2.y) : __float_as_uint(n3.w)};
    const uint32_t qny[2] = {ny ? __float_as_uint(n4.x) : __float_as_uint(n2.z),
                             ny ? __float_as_uint(n4.y) : __float_as_uint(n2.w)};
    const uint32_t qfy[2] = {ny ? __float_as_uint(n2.z) : __float_as_uint(n4.x),
                             ny ? __float_as_uint(n2.w) : __float_as_uint(n4.y)};
    const uint32_t qnz[2] = {nz ? __float_as_uint(n4.z) : __float_as_uint(n3.x),
                             nz ? __float_as_uint(n4.w) : __float_as_uint(n3.y)};
    const uint32_t qfz[2] = {nz ? __float_as_uint(n3.x) : __float_as_uint(n4.z),
                             nz ? __float_as_uint(n3.y) : __float_as_uint(n4.w)};
    const f2x sx2 = pk2(sx, sx), sy2 = pk2(sy, sy), sz2 = pk2(sz, sz);
    const f2x ox2 = pk2(ox, ox), oy2 = pk2(oy, oy), oz2 = pk2(oz, oz);
    float tminP[8], tmaxP[8];
#pragma unroll
    for (int k = 0; k < 8; k += 2) {
      const int w = k >> 2, b = k & 3;
      float tnx[2], tfx[2], tny[2], tfy[2], tnz[2], tfz[2];
      up2(fma2(bytePairToFloat2(qnx[w], b, bias2), sx2, ox2), tnx[0], tnx[1]);
      up2(fma2(bytePairToFloat2(qfx[w], b, bias2), sx2, ox2), tfx[0], tfx[1]);
      up2(fma2(bytePairToFloat2(qny[w], b, bias2), sy2, oy2), tny[0], tny[1]);
      up2(fma2(bytePairToFloat2(qfy[w], b, bias2), sy2, oy2), tfy[0], tfy[1]);
      up2(fma2(bytePairToFloat2(qnz[w], b, bias2), sz2, oz2), tnz[0], tnz[1]);
      up2(fma2(bytePairToFloat2(qfz[w], b, bias2), sz2, oz2), tfz[0], tfz[1]);
      float tmx[2];
#pragma unroll
      for (int j = 0; j < 2; ++j) {
        tminP[k + j] = fmaxf(fmaxf(tnx[j], tny[j]), fmaxf(tnz[j], r.tnear));
        tmx[j] = fminf(fminf(tfx[j], tfy[j]), fminf(tfz[j], r.tfar));
      }
      up2(mul2(pk2(tmx[0], tmx[1]), grow2), tmaxP[k], tmaxP[k + 1]);
    }
    uint32_t hitMask = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) hitMask |= tminP[k] <= tmaxP[k] ? (1u << k) : 0u;
    hitMask &= (1u << nCh) - 1u;
    const uint32_t hitInt = hitMask & ((1u << nInt) - 1u);
    uint32_t primMask = 0;
    for (uint32_t leafHit = hitMask & ~hitInt; leafHit; leafHit &= leafHit - 1u) {
      const int k = __ffs(leafHit) - 1;
      const uint32_t m = __byte_perm(k < 4 ? meta0 : meta1, 0u, 0x4440u | uint32_t(k & 3));
      primMask |= ((1u << (m >> 5)) - 1u) << (m & 31u);
    }
    pendBase = primBase;
    pendMask = primMask;
    const int nearK = nearestChild(tminP, hitInt);
    if (nearK >= 0) {
      const uint32_t rest = hitInt & ~(1u << nearK);
      if (rest) {
        if (sp < kStackDepth) stack[sp++] = (childBase << 8) | rest;
        else ++overflow;
      }
      node = int(childBase) + nearK;
    } else if (sp == 0) {
      node = -1;
    } else {
      const uint32_t g = stack[sp - 1];
      const uint32_t mask = g & 0xFFu;
      const int k = __ffs(mask) - 1;
      const uint32_t left = mask & (mask - 1u);
      if (left) stack[sp - 1] = (g & ~0xFFu) | left;
      else --sp;
      node = int(g >> 8) + k;
    }
  }
}

// Start node for rays that stay inside the box [lo, hi] (AO rays: origin
// +- the AO distance): descend from the root while exactly one child's
// quantised box overlaps the box.  Every sibling passed over is disjoint
// from the box, so no primitive outside the returned subtree can meet such
// a ray, and its traversal may start there with the same result.  -1: no
// box overlaps, nothing can be hit.
UBR_D int boxStartNode(const TravScene& s, f3 lo, f3 hi) {
  if (s.primCount == 0) return -1;
  int node = 0;
  for (int depth = 0; depth < kStackDepth; ++depth) {
    const float4* nd = s.wnodes + kWideF4 * node;
    const float4 n0 = __ldg(nd), n1 = __ldg(nd + 1), n2 = __ldg(nd + 2), n3 = __ldg(nd + 3), n4 = __ldg(nd + 4);
    const uint32_t hdr = __float_as_uint(n0.w);
    const float sx = __uint_as_float((hdr & 0xFFu) << 23);
    const float sy = __uint_as_float(((hdr >> 8) & 0xFFu) << 23);
    const float sz = __uint_as_float(((hdr >> 16) & 0xFFu) << 23);
    const int nInt = int((hdr >> 24) & 0xFu), nCh = int(hdr >> 28);
    int count = 0, only = -1;
    for (int k = 0; k < nCh; ++k) {
      const int w = k >> 2, b = k & 3;
      const float lx = fmaf(byteToFloat(__float_as_uint(w ? n2.y : n2.x), b), sx, n0.x);
      const float ly = fmaf(byteToFloat(__float_as_uint(w ? n2.w : n2.z), b), sy, n0.y);
      const float lz = fmaf(byteToFloat(__float_as_uint(w ? n3.y : n3.x), b), sz, n0.z);
      const float hx = fmaf(byteToFloat(__float_as_uint(w ? n3.w : n3.z), b), sx, n0.x);
      const float hy = fmaf(byteToFloat(__float_as_uint(w ? n4.y : n4.x), b), sy, n0.y);
      const float hz = fmaf(byteToFloat(__float_as_uint(w ? n4.w : n4.z), b), sz, n0.z);
      if (lx <= hi.x && hx >= lo.x && ly <= hi.y && hy >= lo.y && lz <= hi.z && hz >= lo.z) {
        ++count;
        only = k;
      }
    }
    if (count == 0) return -1;
    if (count > 1 || only >= nInt) return node;
    node = int(__float_as_uint(n1.x)) + only;
  }
  return node;
}

// The box holding every AO ray of a hit: origin O, length up to R (unit
// directions), with a relative margin for rounding.
UBR_D void aoBox(f3 O, float R, f3& lo, f3& hi) {
  const float m = R * 1.001f + 1.0e-6f * fmaxf(fmaxf(fabsf(O.x), fabsf(O.y)), fabsf(O.z));
  lo = f3{O.x - m, O.y - m, O.z - m};
  hi = f3{O.x + m, O.y + m, O.z + m};
}

// Shading surface of a hit (hit_shader.hpp:147-341 attribute + normal logic).
struct Surf {
  int kind;
  uint32_t prim;
  f3 P, N, Ng, C, V;
  float opacity;
  uint32_t mat;
  float secEps;
  bool aoOn, shOn;
  bool fromEdge;  // outline decoration primitive (no AO, no shadows)
};

// secondary_rays.hpp:38-46
UBR_D float selfIntersectEps(f3 P, f3 dir, float t) {
  const float dirMax = fmaxf(fabsf(dir.x), fmaxf(fabsf(dir.y), fabsf(dir.z)));
  const float epsScale = fmaxf(fmaxf(fabsf(P.x), fabsf(P.y)), fmaxf(fabsf(P.z), dirMax * t));
  return epsScale * 0x1.0fp-21f;
}
// shading.hpp:27-30
UBR_D f3 faceForward(f3 n, f3 rd) { return dot(n, rd) > 0.0f ? neg(n) : n; }

UBR_D Surf surfaceAt(const Params& p, const DScene& s, f3 org, f3 rd, float t, uint32_t ref, float u,
                     float v, f3 Ng) {
  Surf sf;
  sf.kind = refKind(ref);
  sf.prim = refPrim(ref);
  sf.V = normalize(f3{-rd.x, -rd.y, -rd.z});
  sf.Ng = Ng;
  sf.P = f3{org.x + rd.x * t, org.y + rd.y * t, org.z + rd.z * t};
  sf.secEps = selfIntersectEps(sf.P, rd, t);
  const bool shadowsActive = p.shadowsActive != 0;
  if (sf.kind == kMesh) {
    const uint32_t i0 = __ldg(&s.meshIdx[3 * sf.prim]), i1 = __ldg(&s.meshIdx[3 * sf.prim + 1]),
                   i2 = __ldg(&s.meshIdx[3 * sf.prim + 2]);
    const float w0 = 1.0f - u - v;
    float nb[3];
    for (int k = 0; k < 3; ++k)
      nb[k] = w0 * __ldg(&s.meshNrm[3 * i0 + k]) + u * __ldg(&s.meshNrm[3 * i1 + k]) +
              v * __ldg(&s.meshNrm[3 * i2 + k]);
    const float4 c0 = __ldg(&s.meshCol[i0]), c1 = __ldg(&s.meshCol[i1]), c2 = __ldg(&s.meshCol[i2]);
    const float4 cb = make_float4(w0 * c0.x + u * c1.x + v * c2.x, w0 * c0.y + u * c1.y + v * c2.y,
                                  w0 * c0.z + u * c1.z + v * c2.z, w0 * c0.w + u * c1.w + v * c2.w);
    const f3 NgF = faceForward(Ng, rd);
    f3 N = normalize(f3{nb[0], nb[1], nb[2]});
    if (dot(N, NgF) < 0.0f) N = neg(N);
    sf.N = N;
    sf.C = f3{cb.x, cb.y, cb.z};
    sf.opacity = cb.w;
    sf.mat = s.meshTriMat ? __ldg(&s.meshTriMat[s.baseTri ? sf.prim % s.baseTri : 0]) : s.meshMat;
    sf.aoOn = p.aoSamples > 0;
    sf.shOn = shadowsActive;
    sf.fromEdge = false;
  } else {
    const float4 fc = __ldg(&s.primColor[sf.kind][sf.prim]);
    sf.mat = __ldg(&s.primMat[sf.kind][sf.prim]);
    sf.N = faceForward(normalize(Ng), rd);
    sf.C = f3{fc.x, fc.y, fc.z};
    const bool fromEdge = __ldg(&s.primFromEdge[sf.kind][sf.prim]) != 0;
    sf.fromEdge = fromEdge;
    sf.aoOn = !fromEdge && p.aoSamples > 0;
    sf.shOn = !fromEdge && shadowsActive;
    sf.opacity = fc.w;
    if (sf.kind != kSphere) {
      const float op1 = __ldg(&s.primOpacity1[sf.kind][sf.prim]);
      if (op1 >= 0.0f) {
        float uu = u;
        if (uu < 0.0f) uu = 0.0f;
        if (uu > 1.0f) uu = 1.0f;
        sf.opacity = fc.w * (1.0f - uu) + op1 * uu;
      }
    }
  }
  return sf;
}

// secondary_rays.hpp:51-61
UBR_D void tea2(uint32_t& v0, uint32_t& v1) {
  uint32_t sum = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    sum += 0x9E3779B9u;
    v0 += ((v1 << 4) + 0xA341316Cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xC8013EA4u);
    v1 += ((v0 << 4) + 0xAD90777Du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7E95761Eu);
  }
}
UBR_D float u32ToUnorm(uint32_t u) { return float(u >> 8) * 0x1.0p-24f; }
// secondary_rays.hpp:66-73 (Malley's method).  The angle is the reference's
// float product 6.2831853072f * u1: one sincospi of 2 u1 (the exact angle)
// was 0.3 % faster in the occlusion kernel but moved AO directions by up to
// half an ulp of phi, enough to flip a few grazing AO rays per frame against
// the oracle.
UBR_D f3 cosineSampleHemisphere(float u1, float u2, const Frame3& f) {
  const float phi = 6.2831853072f * u1;
  const float r = sqrtf(u2);
  const float z = sqrtf(fmaxf(0.0f, 1.0f - u2));
  const float x = cosf(phi) * r;
  const float y = sinf(phi) * r;
  return f.t * x + f.b * y + f.n * z;
}
// ambient_occlusion.hpp:98-105
UBR_D float radicalInverse2(uint32_t bits) { return float(__brev(bits)) * 0x1.0p-32f; }
// ambient_occlusion.hpp:112-127
UBR_D void aoSample2d(const Params& p, uint32_t base, int i, float cpx, float cpy, float& u1, float& u2) {
  if (p.aoLowDiscrepancy) {
    u1 = float(i) / float(p.aoSamples) + cpx;
    u2 = radicalInverse2(uint32_t(i)) + cpy;
    if (u1 >= 1.0f) u1 -= 1.0f;
    if (u2 >= 1.0f) u2 -= 1.0f;
  } else {
    uint32_t s0 = base, s1 = uint32_t(i);
    tea2(s0, s1);
    u1 = u32ToUnorm(s0);
    u2 = u32ToUnorm(s1);
  }
}
UBR_D void cpShift(int px, int py, float& cpx, float& cpy) {
  uint32_t c0 = uint32_t(px) + 1u, c1 = uint32_t(py) + 1u;
  tea2(c0, c1);
  cpx = u32ToUnorm(c0);
  cpy = u32ToUnorm(c1);
}
// 2-D sample of AO ray i of hi-res pixel (px, py) (legacy: tea2 stream;
// enhanced: also the low-discrepancy set with its per-pixel shift)
UBR_D void aoUV(const Params& p, int px, int py, int i, float& u1, float& u2) {
  const uint32_t base = uint32_t(px) + uint32_t(py) * uint32_t(p.W);
  if (p.aoEnhanced) {
    float cpx = 0.0f, cpy = 0.0f;
    if (p.aoLowDiscrepancy) cpShift(px, py, cpx, cpy);
    aoSample2d(p, base, i, cpx, cpy, u1, u2);
  } else {
    uint32_t s0 = base, s1 = uint32_t(i);
    tea2(s0, s1);
    u1 = u32ToUnorm(s0);
    u2 = u32ToUnorm(s1);
  }
}
// AO direction of sample i
UBR_D f3 aoDir(const Params& p, const Frame3& f, int px, int py, int i) {
  float u1, u2;
  aoUV(p, px, py, i, u1, u2);
  return cosineSampleHemisphere(u1, u2, f);
}
// secondary_rays.hpp:102-109
UBR_D f3 sampleLightDir(const LightD& l, float u1, float u2) {
  if (l.radius <= 0.0f) return l.L;
  const Frame3 f = frameFromNormal(l.L);
  const float phi = 6.2831853072f * u1;
  const float rr = tanf(l.radius) * sqrtf(u2);
  const f3 d = f.n + f.t * (rr * cosf(phi)) + f.b * (rr * sinf(phi));
  return safeNormalize(d, l.L);
}

UBR_D int warpPushBase(bool push, uint32_t* counter, int& offset) {
  const unsigned mask = __ballot_sync(0xFFFFFFFFu, push);
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (mask) {
    const int leader = __ffs(mask) - 1;
    if (lane == leader) base = int(atomicAdd(counter, uint32_t(__popc(mask))));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
  }
  offset = __popc(mask & ((1u << lane) - 1u));
  return base;
}

UBR_D void warpCount(unsigned long long* ctr, uint32_t v) {
  uint32_t s = __reduce_add_sync(0xFFFFFFFFu, v);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(ctr, (unsigned long long)s);
}

UBR_D float blinnExp(float roughness) {
  float r = roughness;
  if (r < 1e-6f) r = 1e-6f;
  float e = 1.0f / r;
  if (e < 1.0f) e = 1.0f;
  if (e > 1.0e6f) e = 1.0e6f;
  return e;
}
UBR_D float aoMultibounce(float ao, float albedo) {
  const float a = 2.0404f * albedo - 0.3324f;
  const float bb = -4.7951f * albedo + 0.6417f;
  const float c = 2.7552f * albedo + 0.6903f;
  return fmaxf(ao, ((ao * a + bb) * ao + c) * ao);
}

// Material::toonLike / diffuseWeight (scene.hpp:171-196).
UBR_D bool toonLike(const ubr_material& m) {
  if (m.model == 2u) return true;
  if (m.model != 0u) return false;
  if (m.specular > 1.0f || m.phong > 1.0f || m.brilliance == 0.0f) return true;
  return m.diffuse <= 0.0f && m.specular <= 0.0f && m.phong <= 0.0f && m.reflection <= 0.0f;
}
UBR_D float diffuseWeight(const ubr_material& m) { return m.model == 1u ? m.diffuse * (1.0f - m.pbr_metallic) : m.diffuse; }

// 32-bit integer hash (irradiance_cache.hpp:176-184): seeds the gather's
// per-pixel stream and the bounce vertices' shadow streams.
UBR_HD uint32_t hashU32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7FEB352Du;
  x ^= x >> 15;
  x *= 0x846CA68Bu;
  x ^= x >> 16;
  return x;
}

UBR_D float lumOf(float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; }

}  // namespace
}  // namespace ubr

// render.cu -- ubr_render: the wavefront ray-cast + shade frame.
//
// One frame is a loop of transparency rounds over a queue of live pixels
// (reference: the layer loop of integratePixel, shading/transparency.hpp:364-467):
//   k_trace_closest   closest hit of each live ray       (rtcIntersect1, :382)
//   k_surface         hit point, shading normal, secondary-ray origin
//                     (hit_shader.hpp:147-341, secondary_rays.hpp:118-124)
//   k_trace_occlusion one thread per AO / shadow ray, rays of a hit
//                     contiguous: AO sample i, then each light's samples
//                     (ambient_occlusion.hpp:33-57 / 171-267,
//                      secondary_rays.hpp:118-134)
//   k_shade           POV local illumination (shading.hpp:76-192) from the
//                     stored visibility, front-to-back "over" compositing,
//                     first-hit capture, epsilon advance, warp-ballot
//                     compaction of the rays that continue
// then one fused pass k_post: linear fog on the hi-res view-z
// (postprocess/fog.cpp:17-36), ss x ss box average with the non-finite guard
// (image_ops.cpp:9-35) and assumed gamma (image_ops.cpp:37-46).
// Per-pixel and per-ray results do not depend on launch order, so a frame is
// bit-reproducible.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "gi.cuh"
#include "trace.cuh"

namespace ubr {

ubr_status buildScene(Context* c, const ubr_scene_desc& d, Scene** out);

namespace {


struct Bufs {
  float4* accum;      // per hi-res pixel: Cf.rgb, Af
  float* tnear;       // per hi-res pixel
  float4* colorHi;    // per hi-res pixel, pre-post colour
  float* depth;       // per hi-res pixel (first-hit t, 0 = background)
  float* viewZ;
  uint32_t* hitGeom;
  uint32_t* hitPrim;
  float4* hitA;       // per queue slot: t, u, v, ref bits
  float4* hitB;       // per queue slot: Ng.xyz
  float4* surfA;      // O.xyz, eps
  float4* surfB;      // N.xyz, AO start node
  float4* surfT;      // AO frame tangent T.xyz (frameFromNormal(N)), written for hits that cast AO
  uint2* surfC;       // pixel, flags (1 hit, 2 AO, 4 shadows)
  uint8_t* occ;       // per slot * raysPerHit
  float* aoT;         // per slot * aoSamples (enhanced AO nearest t)
  float4* aovA;       // per hi-res pixel first-hit AOVs (or null): albedo.rgb, contact
  float4* aovB;       //   normal.xyz, shape
  float4* aovC;       //   bent normal.xyz, mean occluder distance
  float4* aaN;        // per hi-res pixel (adaptive AA, or null): first-hit normal.xyz, section (int bits)
  const uint32_t* coord;  // fine-lattice pass (or null): lattice index of each pixel slot
  const float4* cgN;      // coarse AO grid (or null): shading normal.xyz, primary hit distance
  const float4* cgQ;      //   openness, contact, shape, mean occluder distance
  const float4* cgB;      //   bent normal.xyz (quality estimator only, else null)
  const uint8_t* cgHit;   //   1 = AO-eligible first hit
  float* aoPatch;         // per hi-res pixel (or null): 1 = the first hit gathered its own AO
  // edge G-buffer per hi-res pixel (or null), in the ubr_frame plane layouts
  uint32_t* gbObj;
  uint32_t* gbMat;
  float* gbNrm;           // 3 per pixel
  float* gbAlpha;
  uint8_t* gbClip;        // 0, 1, or 2 = backface first hit awaiting the front check
  float* gbNear;
  float* gbFar;
  // AO results of an earlier pass over the same hits (adaptive AA's boosted
  // centres), indexed by output pixel: ray j of output pixel o at o * reuseR + j
  const uint8_t* reuseOcc;
  const float* reuseAoT;  // stride Params::reuseAo
  uint32_t reuseR;
  const LightD* lights;
  // pt1 GI gather inputs per hi-res pixel (or null): first-hit position.xyz,
  // first-hit t; shading normal.xyz, eligibility (1/0); reflectance kd * C
  float4* giA;
  float4* giB;
  float4* giR;
  ReflD rfl;          // pt2 traced-reflection records per hi-res pixel (or null)
  unsigned long long* stats;  // 0 closest rays, 1 occlusion rays, 2 capped, 3 overflow
  uint32_t* counter;  // [0] next-queue size, [1] occlusion work-queue size
  uint32_t* occQueue; // queue slots of hits that cast AO / shadow rays
  unsigned long long* cursor;  // next ray of the persistent occlusion kernel
};

// Lattice index of pixel slot gpix: the slot itself, or its entry in the
// coordinate table of a fine-lattice pass.
UBR_D uint32_t latticeOf(const Bufs& b, uint32_t gpix) { return b.coord ? __ldg(&b.coord[gpix]) : gpix; }

// Pixel of slot i in a grid frame's first round (all W x H hi-res pixels, no
// queue): 8 x 4 pixel tiles in slot order, so a warp's primary rays are a
// compact bundle and the hits queued after them stay neighbours (a warp of
// one light's shadow rays covers a tile); the columns and rows that do not
// fill a tile follow in row order.  A bijection on [0, W H).
UBR_D uint32_t tiledPixel(uint32_t i, uint32_t W, uint32_t H) {
  const uint32_t fw = W & ~7u, fh = H & ~3u, nt = fw * fh;
  if (i < nt) {
    const uint32_t t = i >> 5, k = i & 31u, tilesX = fw >> 3;
    return ((t / tilesX) * 4u + (k >> 3)) * W + (t % tilesX) * 8u + (k & 7u);
  }
  uint32_t j = i - nt;
  const uint32_t rw = W - fw;  // right strip of rows [0, fh)
  if (j < rw * fh) return (j / rw) * W + fw + j % rw;
  j -= rw * fh;
  return fh * W + j;  // bottom rows
}

// AO of a coarse grid cell or of an interpolated lookup: openness and the
// quality-estimator channels (neutral when not gathered).
struct AoQ {
  float openness = 1.0f, contact = 1.0f, shape = 1.0f, avgHit = 0.0f;
  f3 bent{0.0f, 0.0f, 0.0f};
};

// sampleCoarseAo (ao/ao_coarse.hpp:152-203): the hit at lattice point
// (px, py) of the p.W x p.H lattice, with shading normal N and primary-ray
// distance z, blends the 2x2 surrounding coarse cells with bilinear x
// (N.Nc)^32 x exp(-|z - zc| / (0.02 z + 1e-6)) weights; rejected (false)
// below a weight sum of 0.3.
UBR_D bool coarseAoLookup(const Params& p, const Bufs& b, int px, int py, f3 N, float z, AoQ& q) {
  const float sx = (float(px) + 0.5f) * float(p.cgW) / float(p.W) - 0.5f;
  const float sy = (float(py) + 0.5f) * float(p.cgH) / float(p.H) - 0.5f;
  const int bx = int(floorf(sx)), by = int(floorf(sy));
  const float fx = sx - float(bx), fy = sy - float(by);
  float wSum = 0.0f, opSum = 0.0f, contactSum = 0.0f, shapeSum = 0.0f, ahdSum = 0.0f;
  f3 bentSum{0.0f, 0.0f, 0.0f};
  for (int dy = 0; dy < 2; ++dy) {
    const int cy = by + dy;
    if (cy < 0 || cy >= p.cgH) continue;
    for (int dx = 0; dx < 2; ++dx) {
      const int cx = bx + dx;
      if (cx < 0 || cx >= p.cgW) continue;
      const uint32_t cp = uint32_t(cy) * uint32_t(p.cgW) + uint32_t(cx);
      if (!__ldg(&b.cgHit[cp])) continue;
      const float wb = (dx ? fx : 1.0f - fx) * (dy ? fy : 1.0f - fy);
      const float4 nz = __ldg(&b.cgN[cp]);
      const float nd = dot(N, f3{nz.x, nz.y, nz.z});
      if (nd <= 0.0f) continue;
      const float wn = powf(nd, 32.0f);
      const float wz = expf(-fabsf(z - nz.w) / (0.02f * z + 1e-6f));
      const float wgt = wb * wn * wz;
      if (wgt <= 0.0f) continue;
      const float4 cq = __ldg(&b.cgQ[cp]);
      wSum += wgt;
      opSum += wgt * cq.x;
      if (b.cgB) {
        const float4 cb = __ldg(&b.cgB[cp]);
        bentSum.x += wgt * cb.x;
        bentSum.y += wgt * cb.y;
        bentSum.z += wgt * cb.z;
        contactSum += wgt * cq.y;
        shapeSum += wgt * cq.z;
        ahdSum += wgt * cq.w;
      }
    }
  }
  if (wSum < 0.3f) return false;
  const float inv = 1.0f / wSum;
  q = AoQ{};
  q.openness = opSum * inv;
  if (b.cgB) {
    q.bent = safeNormalize(f3{bentSum.x * inv, bentSum.y * inv, bentSum.z * inv}, N);
    q.contact = contactSum * inv;
    q.shape = shapeSum * inv;
    q.avgHit = ahdSum * inv;
  }
  return true;
}

// Per-frame record of a batched launch (device array): the frame's
// parameters and scene, and where its pixels start in the batch's global
// hi-res pixel and output pixel spaces.
struct FrameDesc {
  Params p;
  DScene s;
  uint32_t pixOff;
  uint32_t outOff;
};

struct Batch {
  const FrameDesc* frames = nullptr;
  const uint32_t* pixOffs = nullptr;  // frames' pixOff, ascending
  const uint32_t* outOffs = nullptr;  // frames' outOff, ascending
  int nFrames = 0;
  uint32_t R = 0;         // AO/shadow-ray stride per hit (max over frames)
  uint32_t aoSplit = 0;   // ray index where shadow rays start in the ray order (min AO count)
  uint32_t aoStride = 0;  // enhanced-AO t stride per hit (max over frames)
  uint32_t nPix = 0;      // hi-res pixels of all frames
};

// Frame owning global index g in an ascending offset table.
UBR_D int frameOf(const uint32_t* offs, int n, uint32_t g) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&offs[mid]) <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Slot -> global pixel of a round: the queue's entry, else, in a full first
// round (every hi-res pixel of the frame or of each frame of a batch), the
// tiled order within each frame, else the slot itself.
template <bool BATCH>
UBR_D uint32_t slotPixel(const Params& p, const Batch& bt, const Bufs& b, const uint32_t* queue, uint32_t i,
                         uint32_t n) {
  if (queue) return queue[i];
  if (b.coord) return i;
  if (BATCH) {
    if (n != bt.nPix) return i;
    const FrameDesc& fd = bt.frames[frameOf(bt.pixOffs, bt.nFrames, i)];
    return fd.pixOff + tiledPixel(i - fd.pixOff, uint32_t(fd.p.W), uint32_t(fd.p.H));
  }
  if (n != uint32_t(p.W) * uint32_t(p.H)) return i;
  return tiledPixel(i, uint32_t(p.W), uint32_t(p.H));
}

// ---------------------------------------------------------------------------
// kernels

template <bool COUNT, int KM, bool BATCH>
__global__ void __launch_bounds__(128, 8) k_trace_closest(Params p1, DScene s1, Batch bt, Bufs b, int layer,
                                                       uint32_t n, const uint32_t* queue) {
  Count cnt;
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t traced = 0, ovf = 0;
  if (i < n) {
    const uint32_t gpix = slotPixel<BATCH>(p1, bt, b, queue, i, n);
    const int f = BATCH ? frameOf(bt.pixOffs, bt.nFrames, gpix) : 0;
    const Params& p = BATCH ? bt.frames[f].p : p1;
    const DScene& s = BATCH ? bt.frames[f].s : s1;
    const uint32_t pix = BATCH ? gpix - bt.frames[f].pixOff : latticeOf(b, gpix);
    const int px = int(pix % uint32_t(p.W)), py = int(pix / uint32_t(p.W));
    f3 org, rd;
    primaryRay(p, px, py, org, rd);
    float ctn, ctf;
    clipRange(p, rd, ctn, ctf);
    Ray r{org, rd, layer == 0 ? ctn : b.tnear[gpix], ctf};
    Hit h;
    const TravScene ts = travOf(s);
    traverse<COUNT, KM>(ts, r, h, ovf, &cnt, false);
    traced = 1;
    b.hitA[i] = make_float4(h.t, h.u, h.v, __uint_as_float(h.ref));
    b.hitB[i] = make_float4(h.Ng.x, h.Ng.y, h.Ng.z, 0.0f);
  }
  warpCount(&b.stats[0], traced);
  warpCount(&b.stats[3], ovf);
  if (COUNT) {
    warpCount(&b.stats[4], cnt.nodes);
    warpCount(&b.stats[5], cnt.primBytes);
  }
}

template <bool BATCH>
__global__ void __launch_bounds__(128) k_surface(Params p1, DScene s1, Batch bt, Bufs b, int layer, uint32_t n,
                                                 const uint32_t* queue) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool cast = false;
  if (i < n) {
    const uint32_t gpix = slotPixel<BATCH>(p1, bt, b, queue, i, n);
    const int f = BATCH ? frameOf(bt.pixOffs, bt.nFrames, gpix) : 0;
    const Params& p = BATCH ? bt.frames[f].p : p1;
    const DScene& s = BATCH ? bt.frames[f].s : s1;
    const uint32_t pix = BATCH ? gpix - bt.frames[f].pixOff : latticeOf(b, gpix);
    const float4 ha = b.hitA[i];
    const uint32_t ref = __float_as_uint(ha.w);
    if (ref == kInvalid) {
      b.surfC[i] = make_uint2(gpix, 0u);
    } else {
      const int px = int(pix % uint32_t(p.W)), py = int(pix / uint32_t(p.W));
      f3 org, rd;
      primaryRay(p, px, py, org, rd);
      const float4 hb = b.hitB[i];
      const Surf sf = surfaceAt(p, s, org, rd, ha.x, ref, ha.y, ha.z, f3{hb.x, hb.y, hb.z});
      // computeAO / computeShadow origin: P + safeNormalize(faceForward-to-N(Ng)) * eps
      f3 ng = dot(sf.Ng, sf.N) < 0.0f ? neg(sf.Ng) : sf.Ng;
      ng = safeNormalize(ng, sf.N);
      const f3 O = sf.P + ng * sf.secEps;
      // coarse-grid AO: a hit the grid lookup accepts casts no AO rays
      // (hit_shader.hpp:129-145)
      bool aoCast = sf.aoOn;
      if (aoCast && p.aoCoarse) {
        AoQ q;
        if (coarseAoLookup(p, b, px, py, sf.N, ha.x, q)) aoCast = false;
      }
      // subtree that holds everything the hit's AO rays can meet
      int start = 0;
      if (aoCast) {
        f3 lo, hi;
        aoBox(O, p.aoDistance, lo, hi);
        start = boxStartNode(travOf(s), lo, hi);
      }
      b.surfA[i] = make_float4(O.x, O.y, O.z, sf.secEps);
      b.surfB[i] = make_float4(sf.N.x, sf.N.y, sf.N.z, __int_as_float(start));
      if (aoCast) {  // the AO rays' frame, once per hit instead of once per ray
        const Frame3 fr = frameFromNormal(sf.N);
        b.surfT[i] = make_float4(fr.t.x, fr.t.y, fr.t.z, 0.0f);
      }
      // flags: 1 hit, 2 casts AO, 4 casts shadows; bits 8.. the frame index
      // bit 3: principled material (its area-light samples use their own stream)
      const bool pbr = __ldg(&s.mats[sf.mat].model) == 1u;
      const uint32_t flags =
          1u | (aoCast ? 2u : 0u) | (sf.shOn ? 4u : 0u) | (pbr ? 8u : 0u) | (uint32_t(f) << 8);
      b.surfC[i] = make_uint2(gpix, flags);
      cast = (flags & 6u) != 0u;
    }
  }
  // compact the hits that cast secondary rays so occlusion warps hold only live rays
  int off;
  const int qb = warpPushBase(cast, b.counter + 1, off);
  if (cast) b.occQueue[qb + off] = i;
}

// The AO / shadow ray j of the hit in queue slot `slot` (rays of a hit: AO
// sample j < aoSamples, then each light's shadow samples in light order).
struct OccRay {
  Ray r;
  bool trace;    // needs a traversal
  bool anyHit;   // binary visibility (false: nearest t, enhanced AO)
  bool grazing;  // AO sample below the 0.01 cosine: counts as occluded
  bool ao;       // this is an AO ray of an AO-receiving hit
  int start;     // traversal start node (-1: provably no hit)
};

UBR_D OccRay occlusionRay(const Params& p, const Bufs& b, uint32_t slot, uint32_t pix, uint32_t flags, int j) {
  OccRay o;
  o.trace = false;
  o.anyHit = true;
  o.grazing = false;
  o.ao = false;
  o.start = 0;
  const LightD* lights = b.lights + p.lightOff;
  const int px = int(pix % uint32_t(p.W)), py = int(pix / uint32_t(p.W));
  const float4 sa = b.surfA[slot], sb = b.surfB[slot];
  const f3 N = ld3(sb);
  f3 dir{0.0f, 0.0f, 0.0f};
  float tfar = kInfF;
  if (j < p.aoSamples) {
    if (flags & 2u) {
      o.ao = true;
      // frameFromNormal(N), its tangent computed once per hit
      const f3 T = ld3(b.surfT[slot]);
      const Frame3 f{T, cross(N, T), N};
      dir = aoDir(p, f, px, py, j);
      o.grazing = dot(dir, N) < 0.01f;
      o.trace = !o.grazing;
      o.anyHit = !(p.aoEnhanced || p.aoWriteAov);
      o.start = __float_as_int(sb.w);
      tfar = p.aoDistance;
    }
  } else if (flags & 4u) {
    const int k = j - p.aoSamples;
    int l = 0;
    while (l + 1 < p.nLights && lights[l + 1].rayOffset <= k) ++l;
    const LightD L = lights[l];
    if (dot(N, L.L) > 0.0f) {
      dir = L.L;
      if (L.soft) {
        // the (px, py) stream is advanced by every earlier lit soft light
        // (shading.hpp:100, secondary_rays.hpp:128-131)
        int consumed = 0;
        for (int q = 0; q < l; ++q) {
          const LightD Q = lights[q];
          if (Q.soft && dot(N, Q.L) > 0.0f) consumed += Q.samples;
        }
        // principled area lights draw from the 'PBRD'-tagged stream
        // (principled.hpp:174-175), advanced the same way
        uint32_t s0 = (flags & 8u) ? (uint32_t(px) ^ 0x50425244u) : uint32_t(px), s1 = uint32_t(py);
        const int stepsRng = consumed + (k - L.rayOffset) + 1;
        for (int q = 0; q < stepsRng; ++q) tea2(s0, s1);
        dir = sampleLightDir(L, u32ToUnorm(s0), u32ToUnorm(s1));
        // a principled sample below the horizon is never queried (:262)
        if ((flags & 8u) && !(dot(N, dir) > 0.0f)) {
          o.r = Ray{ld3(sa), dir, sa.w, tfar};
          return o;
        }
      }
      o.trace = true;
    }
  }
  o.r = Ray{ld3(sa), dir, sa.w, tfar};
  return o;
}

UBR_D void occlusionWrite(const Params& p, const Bufs& b, uint64_t R, uint64_t aoStride, uint32_t slot, int j,
                          const OccRay& o, bool hit, float t) {
  const uint8_t res = o.grazing ? 1 : (hit ? 1 : 0);
  if (o.ao && (p.aoEnhanced || p.aoWriteAov))
    b.aoT[uint64_t(slot) * aoStride + j] = o.grazing ? -1.0f : (hit ? t : kInfF);
  b.occ[uint64_t(slot) * R + j] = res;
}

// Ray (queue position, ray index) of global ray id `rid` among nq hits with
// R rays each: AO rays first, hit-major (a warp holds whole hits' AO samples,
// rays from one origin), then the shadow rays, ray-index-major (a warp holds
// one light's rays of 32 neighbouring hits, one direction).  A bijection onto
// [0, nq) x [0, R) for any split A.
UBR_D void occRayOf(uint64_t rid, uint32_t nq, uint64_t R, uint64_t A, uint32_t& q, int& j) {
  if ((uint64_t(nq) * R) >> 32 == 0) {
    // every ray id of the launch fits 32 bits (warp-uniform): 32-bit division
    const uint32_t r32 = uint32_t(rid), a32 = uint32_t(A), nAo32 = nq * a32;
    if (r32 < nAo32) {
      q = r32 / a32;
      j = int(r32 - q * a32);
    } else {
      const uint32_t t = r32 - nAo32, d = t / nq;
      q = t - d * nq;
      j = int(a32 + d);
    }
    return;
  }
  const uint64_t nAo = uint64_t(nq) * A;
  if (rid < nAo) {
    q = uint32_t(rid / A);
    j = int(rid % A);
  } else {
    const uint64_t t = rid - nAo;
    q = uint32_t(t % nq);
    j = int(A + t / nq);
  }
}

// The occlusion kernel's body: one thread per AO / shadow ray.
template <bool COUNT, int KM, bool BATCH, bool IL>
__device__ __forceinline__ void occlusionBody(const Params& p1, const DScene& s1, const Batch& bt, const Bufs& b) {
  Count cnt;
  const uint64_t tid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint64_t R = BATCH ? uint64_t(bt.R) : uint64_t(p1.raysPerHit);
  const uint64_t aoStride = BATCH ? uint64_t(bt.aoStride) : uint64_t(p1.aoSamples);
  uint32_t traced = 0, ovf = 0;
  const uint32_t nq = *(volatile const uint32_t*)(b.counter + 1);
  if (tid < uint64_t(nq) * R) {
    uint32_t q;
    int j;
    occRayOf(tid, nq, R, BATCH ? uint64_t(bt.aoSplit) : uint64_t(p1.aoSamples), q, j);
    const uint32_t slot = b.occQueue[q];
    const uint2 sc = b.surfC[slot];
    const int f = BATCH ? int(sc.y >> 8) : 0;
    const Params& p = BATCH ? bt.frames[f].p : p1;
    const DScene& s = BATCH ? bt.frames[f].s : s1;
    if (!BATCH && b.reuseOcc && j < p.reuseAo && (sc.y & 2u)) {
      // the same AO ray (origin, direction, range) was traced by the centre
      // pass: copy its result
      const uint32_t pix = latticeOf(b, sc.x);
      const uint32_t px = pix % uint32_t(p.W), py = pix / uint32_t(p.W);
      const uint64_t o = uint64_t(py / uint32_t(p.ss)) * uint32_t(p.outW) + px / uint32_t(p.ss);
      b.occ[uint64_t(slot) * R + j] = b.reuseOcc[o * b.reuseR + j];
      if (p.aoEnhanced || p.aoWriteAov) b.aoT[uint64_t(slot) * aoStride + j] = b.reuseAoT[o * uint64_t(p.reuseAo) + j];
    } else if (j < p.raysPerHit) {
      const OccRay o = occlusionRay(p, b, slot, BATCH ? sc.x - bt.frames[f].pixOff : latticeOf(b, sc.x), sc.y, j);
      bool hit = false;
      Hit h;
      h.t = kInfF;
      if (o.trace) {
        const TravScene ts = travOf(s);
        if (p.aoEnhanced || p.aoWriteAov)
          hit = traverse<COUNT, KM, false>(ts, o.r, h, ovf, &cnt, o.anyHit, o.start);
        else if (IL)
          hit = traverseAnyInterleaved<COUNT, KM>(ts, o.r, ovf, &cnt, o.start);
        else
          hit = traverse<COUNT, KM, true>(ts, o.r, h, ovf, &cnt, true, o.start);
        traced = 1;
      }
      occlusionWrite(p, b, R, aoStride, slot, j, o, hit, h.t);
    }
  }
  warpCount(&b.stats[1], traced);
  warpCount(&b.stats[3], ovf);
  if (COUNT) {
    warpCount(&b.stats[6], cnt.nodes);
    warpCount(&b.stats[7], cnt.primBytes);
  }
}

// One thread per AO / shadow ray, 9 blocks of 128 per SM (56 registers):
// measured best for mesh and for sphere + cylinder scenes.
template <bool COUNT, int KM, bool BATCH>
__global__ void __launch_bounds__(128, 9)
    k_trace_occlusion(Params p1, DScene s1, Batch bt, Bufs b, uint32_t n) {
  occlusionBody<COUNT, KM, BATCH, false>(p1, s1, bt, b);
}

// The same with node visits and primitive tests interleaved one per step
// (traverseAnyInterleaved) for the binary-visibility rays.
template <bool COUNT, int KM, bool BATCH>
__global__ void __launch_bounds__(128, (KM & kMaskMesh) ? 9 : 8)
    k_trace_occlusion_il(Params p1, DScene s1, Batch bt, Bufs b, uint32_t n) {
  occlusionBody<COUNT, KM, BATCH, true>(p1, s1, bt, b);
}

// Resident-grid variant: each CTA stages the top wide nodes (root and the two
// levels below) in shared memory once, then walks the ray list with a grid
// stride in the same order as k_trace_occlusion.  (Batches mix scenes, so
// there the nodes are read from global memory.)
template <bool COUNT, int KM, bool BATCH>
__global__ void __launch_bounds__(128, 8) k_trace_occlusion_gs(Params p1, DScene s1, Batch bt, Bufs b) {
  __shared__ float4 sTop[kTopNodes * kWideF4];
  const int nTop = BATCH ? 0 : min(kTopNodes, int(s1.wideNodes));
  for (int k = threadIdx.x; k < nTop * kWideF4; k += blockDim.x) sTop[k] = __ldg(&s1.wnodes[k]);
  __syncthreads();
  Count cnt;
  const uint64_t R = BATCH ? uint64_t(bt.R) : uint64_t(p1.raysPerHit);
  const uint64_t aoStride = BATCH ? uint64_t(bt.aoStride) : uint64_t(p1.aoSamples);
  uint32_t traced = 0, ovf = 0;
  const uint32_t nq = *(volatile const uint32_t*)(b.counter + 1);
  const uint64_t total = uint64_t(nq) * R;
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t tid = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; tid < total; tid += stride) {
    uint32_t q;
    int j;
    occRayOf(tid, nq, R, BATCH ? uint64_t(bt.aoSplit) : uint64_t(p1.aoSamples), q, j);
    const uint32_t slot = b.occQueue[q];
    const uint2 sc = b.surfC[slot];
    const int f = BATCH ? int(sc.y >> 8) : 0;
    const Params& p = BATCH ? bt.frames[f].p : p1;
    const DScene& s = BATCH ? bt.frames[f].s : s1;
    if (j < p.raysPerHit) {
      const OccRay o = occlusionRay(p, b, slot, BATCH ? sc.x - bt.frames[f].pixOff : latticeOf(b, sc.x), sc.y, j);
      bool hit = false;
      Hit h;
      h.t = kInfF;
      if (o.trace) {
        const TravScene ts = travOf(s);
        hit = (p.aoEnhanced || p.aoWriteAov)
                  ? traverse<COUNT, KM, false>(ts, o.r, h, ovf, &cnt, o.anyHit, o.start, sTop, nTop)
                           : traverse<COUNT, KM, true>(ts, o.r, h, ovf, &cnt, true, o.start, sTop, nTop);
        ++traced;
      }
      occlusionWrite(p, b, R, aoStride, slot, j, o, hit, h.t);
    }
  }
  warpCount(&b.stats[1], traced);
  warpCount(&b.stats[3], ovf);
  if (COUNT) {
    warpCount(&b.stats[6], cnt.nodes);
    warpCount(&b.stats[7], cnt.primBytes);
  }
}

// Persistent variant: a resident grid whose warps keep their lanes busy.
// Each lane advances its ray one BVH node per iteration; when at least
// kRefill lanes of a warp are idle they fetch the next rays of the global
// list with one atomic per warp (dynamic fetch after Aila and Laine,
// "Understanding the Efficiency of Ray Traversal on GPUs", HPG 2009), so
// lanes whose rays end early do not wait for the warp's longest ray.
constexpr int kRefill = 28;  // measured: 8 -> +14 %, 16 -> +6 %, 24 -> 0 %, 32 -> +4 % against 28

template <bool COUNT, int KM, bool BATCH>
__global__ void __launch_bounds__(128, 8) k_trace_occlusion_persistent(Params p1, DScene s1, Batch bt, Bufs b) {
  Count cnt;
  uint32_t traced = 0, ovf = 0;
  const uint64_t R = BATCH ? uint64_t(bt.R) : uint64_t(p1.raysPerHit);
  const uint64_t aoStride = BATCH ? uint64_t(bt.aoStride) : uint64_t(p1.aoSamples);
  int f = 0;
  const uint32_t nqq = *(volatile const uint32_t*)(b.counter + 1);
  const uint64_t total = uint64_t(nqq) * R;
  const int lane = threadIdx.x & 31;
  bool active = false, exhausted = total == 0;
  uint32_t slot = 0;
  int j = 0;
  OccRay o;
  f3 inv{0.0f, 0.0f, 0.0f};
  TriPre pre;
  TravState st;
  Hit best;
  TravScene ts = travOf(s1);
  for (;;) {
    const unsigned idle = __ballot_sync(0xFFFFFFFFu, !active);
    if (!exhausted && (__popc(idle) >= kRefill || idle == 0xFFFFFFFFu)) {
      const int leader = __ffs(idle) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(b.cursor, (unsigned long long)__popc(idle));
      base = __shfl_sync(0xFFFFFFFFu, base, leader);
      if (!active) {
        const uint64_t rid = base + uint64_t(__popc(idle & ((1u << lane) - 1u)));
        if (rid < total) {
          uint32_t q;
          occRayOf(rid, nqq, R, BATCH ? uint64_t(bt.aoSplit) : uint64_t(p1.aoSamples), q, j);
          slot = b.occQueue[q];
          const uint2 sc = b.surfC[slot];
          f = BATCH ? int(sc.y >> 8) : 0;
          const Params& p = BATCH ? bt.frames[f].p : p1;
          const DScene& s = BATCH ? bt.frames[f].s : s1;
          if (j < p.raysPerHit) o = occlusionRay(p, b, slot, BATCH ? sc.x - bt.frames[f].pixOff : latticeOf(b, sc.x), sc.y, j);
          else o.trace = o.grazing = o.ao = false;
          if (j >= p.raysPerHit) {
            // stride padding of a frame with fewer rays per hit: nothing to do
          } else if (o.trace && s.primCount > 0 && o.start >= 0) {
            ts = travOf(s);
            inv = safeInv(o.r.dir);
            if (KM & kMaskMesh) pre = triPre(o.r.dir);
            travInit(o.r, st, best, o.start);
            active = true;
            ++traced;
          } else {
            if (o.trace) ++traced;
            occlusionWrite(p, b, R, aoStride, slot, j, o, false, kInfF);
          }
        }
      }
      if (base + uint64_t(__popc(idle)) >= total) exhausted = true;
    }
    if (!__any_sync(0xFFFFFFFFu, active)) {
      if (exhausted) break;
      continue;
    }
    if (active) {
      const Params& p = BATCH ? bt.frames[f].p : p1;
      if (travStep<COUNT, KM>(ts, o.r, inv, pre, st, best, ovf, &cnt, o.anyHit)) {
        occlusionWrite(p, b, R, aoStride, slot, j, o, best.ref != kInvalid, best.t);
        active = false;
      }
    }
  }
  warpCount(&b.stats[1], traced);
  warpCount(&b.stats[3], ovf);
  if (COUNT) {
    warpCount(&b.stats[6], cnt.nodes);
    warpCount(&b.stats[7], cnt.primBytes);
  }
}

// computeAOQuality accumulation over a hit's stored nearest-hit distances
// (ambient_occlusion.hpp:171-267), sample order preserved: the openness for
// the enhanced estimator and the contact / shape / bent-normal / mean
// occluder distance AOVs.
UBR_D AoQ aoQuality(const Params& p, const float* aoT, uint64_t aoStride, uint32_t i, f3 N, int px, int py,
                    float power, bool multiScale) {
  const float R = p.aoDistance;
  float radius[3], weight[3];
  int K;
  if (multiScale) {
    K = 3;
    radius[0] = 0.08f * R; radius[1] = 0.30f * R; radius[2] = 1.00f * R;
    weight[0] = 0.55f; weight[1] = 0.35f; weight[2] = 0.10f;
  } else {
    K = 1;
    radius[0] = radius[1] = radius[2] = R;
    weight[0] = 1.0f; weight[1] = weight[2] = 0.0f;
  }
  const Frame3 f = frameFromNormal(N);
  float obsScale[3] = {0.0f, 0.0f, 0.0f};
  float weightedObs = 0.0f, hitDistSum = 0.0f;
  int nHit = 0;
  f3 bentAccum{0.0f, 0.0f, 0.0f};
  for (int k = 0; k < p.aoSamples; ++k) {
    const f3 dir = aoDir(p, f, px, py, k);
    if (dot(dir, N) < 0.01f) {
      obsScale[0] += 1.0f; obsScale[1] += 1.0f; obsScale[2] += 1.0f;
      weightedObs += 1.0f;
      continue;
    }
    const float th = aoT[uint64_t(i) * aoStride + k];
    float perSample = 0.0f;
    for (int q = 0; q < K; ++q) {
      if (th < radius[q]) {
        float fk = 1.0f;
        if (power > 0.0f) {
          float a = 1.0f - th / radius[q];
          if (a < 0.0f) a = 0.0f;
          fk = powf(a, power);
        }
        obsScale[q] += fk;
        perSample += weight[q] * fk;
      }
    }
    weightedObs += perSample;
    bentAccum = bentAccum + dir * (1.0f - perSample);
    if (th < R) {
      hitDistSum += th;
      ++nHit;
    }
  }
  AoQ r;
  const float invN = 1.0f / float(p.aoSamples);
  r.openness = 1.0f - weightedObs * invN;
  r.contact = 1.0f - obsScale[0] * invN;
  if (multiScale) {
    const float wMid = weight[1] + weight[2];
    r.shape = 1.0f - (weight[1] * obsScale[1] + weight[2] * obsScale[2]) / (wMid * float(p.aoSamples));
  } else {
    r.shape = r.openness;
  }
  r.bent = safeNormalize(bentAccum, N);
  r.avgHit = nHit > 0 ? hitDistSum / float(nHit) : R;
  return r;
}

// Anisotropy tangent of a principled sphere / cylinder hit (hit_shader.hpp:
// 373-425): the meridian of the world +y pole on a sphere, the axis projected
// onto the tangent plane on a cylinder (none at poles, caps or degenerate
// projections), turned by the material's rotation (in turns).
UBR_D bool anisoTangent(const DScene& s, const Surf& sf, float rotation, f3& t1) {
  const f3 N = sf.N;
  bool valid = false;
  if (sf.kind == kSphere) {
    if (fabsf(N.y) < 0.999f) {
      const f3 tPhi = safeNormalize(cross(f3{0.0f, 1.0f, 0.0f}, N));
      t1 = cross(N, tPhi);
      valid = true;
    }
  } else if (s.primAxis[sf.kind]) {
    const float4 a4 = __ldg(&s.primAxis[sf.kind][sf.prim]);
    const f3 A{a4.x, a4.y, a4.z};
    const f3 ngu = safeNormalize(sf.Ng, N);
    if (fabsf(dot(ngu, A)) < 0.99f) {
      const float andn = dot(A, N);
      const f3 proj{A.x - N.x * andn, A.y - N.y * andn, A.z - N.z * andn};
      if (dot(proj, proj) >= 1.0e-12f) {
        t1 = safeNormalize(proj);
        valid = true;
      }
    }
  }
  if (valid && rotation != 0.0f) {
    const float ang = rotation * 6.2831853072f;
    const f3 t2 = cross(N, t1);
    const float ca = cosf(ang), sa = sinf(ang);
    t1 = f3{ca * t1.x + sa * t2.x, ca * t1.y + sa * t2.y, ca * t1.z + sa * t2.z};
  }
  return valid;
}

// GGX helpers of principled.hpp:35-98.
UBR_D float ggxD(float a2, float ndh) {
  if (ndh <= 0.0f) return 0.0f;
  const float t = ndh * ndh * (a2 - 1.0f) + 1.0f;
  return a2 / (3.14159265358979323846f * t * t);
}
UBR_D float ggxLambda(float a2, float cosT) {
  const float c2 = fmaxf(cosT * cosT, 1.0e-12f);
  const float t2 = (1.0f - c2) / c2;
  return 0.5f * (sqrtf(1.0f + a2 * t2) - 1.0f);
}
UBR_D float ggxDAniso(float ax, float ay, float hx, float hy, float hz) {
  if (hz <= 0.0f) return 0.0f;
  const float sx = hx / ax, sy = hy / ay;
  const float t = sx * sx + sy * sy + hz * hz;
  return 1.0f / (3.14159265358979323846f * ax * ay * t * t);
}
UBR_D float ggxLambdaAniso(float ax, float ay, float vx, float vy, float vz) {
  const float z2 = fmaxf(vz * vz, 1.0e-12f);
  const float t2 = (ax * ax * vx * vx + ay * ay * vy * vy) / z2;
  return 0.5f * (sqrtf(1.0f + t2) - 1.0f);
}

// shadePrincipled (principled.hpp:139-302), direct pass without traced
// reflection: one GGX lobe with Schlick Fresnel; an area light (shadows on,
// samples > 1, radius > 0) weighs visibility x BRDF per cone sample on the
// 'PBRD'-tagged per-pixel stream.  `occ` = this hit's shadow-ray results
// (light order, rayOffset per light).
UBR_D f3 shadePrincipled(const Params& p, const ubr_material& m, const Surf& sf, const LightD* lights,
                         const uint8_t* occ, f3 aoFactor, f3 ambLight, float diffuseAo, int px, int py,
                         const f3* tangent, bool traceRefl) {
  const f3 C = sf.C, N = sf.N, V = sf.V;
  f3 out{m.emission * C.x + aoFactor.x * m.ambient * C.x * ambLight.x,
         m.emission * C.y + aoFactor.y * m.ambient * C.y * ambLight.y,
         m.emission * C.z + aoFactor.z * m.ambient * C.z * ambLight.z};
  const float kd = m.diffuse * (1.0f - m.pbr_metallic);
  const float dd = 0.08f * m.pbr_specular, tm = m.pbr_metallic;
  const f3 F0{dd + (C.x - dd) * tm, dd + (C.y - dd) * tm, dd + (C.z - dd) * tm};
  const float f0max = fmaxf(F0.x, fmaxf(F0.y, F0.z));
  float alpha = m.pbr_roughness * m.pbr_roughness;
  if (alpha < 1.0e-3f) alpha = 1.0e-3f;
  const float a2 = alpha * alpha;
  const float ndv = fmaxf(dot(N, V), 1.0e-4f);
  const float lamV = ggxLambda(a2, ndv);
  const float kPi = 3.14159265358979323846f;
  bool an = false;
  f3 at1{0.0f, 0.0f, 0.0f}, at2{0.0f, 0.0f, 0.0f};
  float ax = 0.0f, ay = 0.0f;
  if (tangent != nullptr && m.pbr_anisotropy != 0.0f) {
    an = true;
    at1 = *tangent;
    at2 = cross(N, at1);
    float aa = fabsf(m.pbr_anisotropy);
    if (aa > 1.0f) aa = 1.0f;
    const float aspect = sqrtf(1.0f - 0.9f * aa);
    ax = alpha / aspect;
    if (ax > 1.0f) ax = 1.0f;
    ay = alpha * aspect;
    if (ax < 1.0e-3f) ax = 1.0e-3f;
    if (ay < 1.0e-3f) ay = 1.0e-3f;
  }
  const float lamVA = an ? ggxLambdaAniso(ax, ay, dot(V, at1), dot(V, at2), ndv) : 0.0f;
  auto specWeight = [&](f3 H, float ndh, f3 w, float ndlw) {
    if (!an) {
      const float G2 = 1.0f / (1.0f + lamV + ggxLambda(a2, ndlw));
      return kPi * ggxD(a2, ndh) * G2 / (4.0f * ndv);
    }
    const float G2 = 1.0f / (1.0f + lamVA + ggxLambdaAniso(ax, ay, dot(w, at1), dot(w, at2), ndlw));
    return kPi * ggxDAniso(ax, ay, dot(H, at1), dot(H, at2), ndh) * G2 / (4.0f * ndv);
  };
  auto schlick = [&](float u) {
    float c = 1.0f - u;
    if (c < 0.0f) c = 0.0f;
    if (c > 1.0f) c = 1.0f;
    const float c5 = c * c * c * c * c;
    return f3{F0.x + (1.0f - F0.x) * c5, F0.y + (1.0f - F0.y) * c5, F0.z + (1.0f - F0.z) * c5};
  };
  uint32_t t0 = uint32_t(px) ^ 0x50425244u, t1 = uint32_t(py);
  for (int l = 0; l < p.nLights; ++l) {
    const LightD L = lights[l];
    const float ndl = dot(N, L.L);
    if (ndl <= 0.0f) continue;
    const bool areaPath = sf.shOn && L.soft;
    if (!areaPath) {
      const float shadowFactor = (sf.shOn && occ[L.rayOffset]) ? 0.0f : 1.0f;
      const f3 Lc{L.color.x * shadowFactor, L.color.y * shadowFactor, L.color.z * shadowFactor};
      const float dk = kd * ndl * diffuseAo;
      out.x += dk * C.x * Lc.x;
      out.y += dk * C.y * Lc.y;
      out.z += dk * C.z * Lc.z;
      if (!L.highlight) continue;
      if (f0max > 0.0f) {
        const f3 H = normalize(f3{L.L.x + V.x, L.L.y + V.y, L.L.z + V.z});
        const float ndh = dot(N, H);
        if (ndh > 0.0f) {
          const float sW = specWeight(H, ndh, L.L, ndl);
          const f3 F = schlick(dot(V, H));
          out.x += sW * F.x * Lc.x;
          out.y += sW * F.y * Lc.y;
          out.z += sW * F.z * Lc.z;
        }
      }
    } else {
      float accD = 0.0f;
      f3 accS{0.0f, 0.0f, 0.0f};
      for (int k = 0; k < L.samples; ++k) {
        tea2(t0, t1);
        const f3 w = sampleLightDir(L, u32ToUnorm(t0), u32ToUnorm(t1));
        const float ndlS = dot(N, w);
        if (ndlS <= 0.0f) continue;
        if (occ[L.rayOffset + k]) continue;
        accD += ndlS;
        if (L.highlight && f0max > 0.0f) {
          const f3 H = normalize(f3{w.x + V.x, w.y + V.y, w.z + V.z});
          const float ndh = dot(N, H);
          if (ndh > 0.0f) {
            const float sW = specWeight(H, ndh, w, ndlS);
            const f3 F = schlick(dot(V, H));
            accS.x += sW * F.x;
            accS.y += sW * F.y;
            accS.z += sW * F.z;
          }
        }
      }
      const float inv = 1.0f / float(L.samples);
      const float dk = kd * diffuseAo * inv * accD;
      out.x += dk * C.x * L.color.x;
      out.y += dk * C.y * L.color.y;
      out.z += dk * C.z * L.color.z;
      out.x += inv * accS.x * L.color.x;
      out.y += inv * accS.y * L.color.y;
      out.z += inv * accS.z * L.color.z;
    }
  }
  // the environment term; pt2's traced reflection owns it instead (:277-302)
  if (!traceRefl) {
    if (m.reflection > 0.0f) {
      out.x += m.reflection * p.bg.x;
      out.y += m.reflection * p.bg.y;
      out.z += m.reflection * p.bg.z;
    } else if (f0max > 0.0f) {
      out.x += F0.x * p.bg.x;
      out.y += F0.y * p.bg.y;
      out.z += F0.z * p.bg.z;
    }
  }
  return out;
}

// pt2GgxAlphaFromRoughness (shading.hpp:48-60): the GGX alpha matched to the
// Blinn highlight width, sqrt(2 / (blinnExp + 2)); below 0.015 a mirror (0).
UBR_D float ggxAlphaFromRoughness(float roughness) {
  const float e = blinnExp(roughness);
  const float a = sqrtf(2.0f / (e + 2.0f));
  if (a < 0.015f) return 0.0f;
  return a < 1.0f ? a : 1.0f;
}

template <bool BATCH>
__global__ void __launch_bounds__(128) k_shade(Params p1, DScene s1, Batch bt, Bufs b, int layer, uint32_t n,
                                               const uint32_t* queue, uint32_t* outQueue) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  bool push = false;
  uint32_t gpix = 0, capped = 0;
  if (i < n) {
    gpix = slotPixel<BATCH>(p1, bt, b, queue, i, n);
    const int f = BATCH ? frameOf(bt.pixOffs, bt.nFrames, gpix) : 0;
    const Params& p = BATCH ? bt.frames[f].p : p1;
    const DScene& s = BATCH ? bt.frames[f].s : s1;
    const LightD* lights = b.lights + p.lightOff;
    const uint64_t R = BATCH ? uint64_t(bt.R) : uint64_t(p.raysPerHit);
    const uint64_t aoStride = BATCH ? uint64_t(bt.aoStride) : uint64_t(p.aoSamples);
    const uint32_t pix = BATCH ? gpix - bt.frames[f].pixOff : latticeOf(b, gpix);
    const int px = int(pix % uint32_t(p.W)), py = int(pix / uint32_t(p.W));
    float4 acc = layer == 0 ? make_float4(0, 0, 0, 0) : b.accum[gpix];
    f3 base = p.bg;
    float baseCov = p.transparentBg ? 0.0f : 1.0f;
    bool done = true;
    const float4 ha = b.hitA[i];
    const uint32_t ref = __float_as_uint(ha.w);
    if (ref != kInvalid) {
      f3 org, rd;
      primaryRay(p, px, py, org, rd);
      const float4 hb = b.hitB[i];
      const float t = ha.x;
      const Surf sf = surfaceAt(p, s, org, rd, t, ref, ha.y, ha.z, f3{hb.x, hb.y, hb.z});
      const ubr_material m = s.mats[sf.mat];
      // --- ambient occlusion factors (ao_shade.hpp:44-141) ---
      f3 aoFactor{1.0f, 1.0f, 1.0f};
      f3 ambLight = p.ambLight;
      float diffuseAo = 1.0f;
      const uint64_t rb = uint64_t(i) * R;
      AoQ aq;  // AOVs of this hit (neutral unless computed)
      bool patched = false;
      bool giElig = false;
      if (sf.aoOn) {
        float openness;
        f3 bent = sf.N;
        AoQ cq;
        const bool coarse = p.aoCoarse && coarseAoLookup(p, b, px, py, sf.N, ha.x, cq);
        patched = p.aoCoarse && !coarse;
        if (coarse) {
          // interpolated grid values (legacy grids leave the AOV defaults)
          aq = cq;
          openness = cq.openness;
          bent = cq.bent;
        } else if (!p.aoEnhanced) {
          int hits = 0;
          for (int k = 0; k < p.aoSamples; ++k) hits += b.occ[rb + k];
          openness = 1.0f - float(hits) / float(p.aoSamples);
          // aoWriteAov on the legacy estimator: one single-scale quality pass
          // over the same sample stream (ao_shade.hpp:58-70)
          if (p.aoWriteAov && sf.kind == kMesh) aq = aoQuality(p, b.aoT, aoStride, i, sf.N, px, py, 0.0f, false);
        } else {
          aq = aoQuality(p, b.aoT, aoStride, i, sf.N, px, py, p.aoFalloffPower, p.aoMultiScale != 0);
          openness = aq.openness;
          bent = aq.bent;
        }
        if (p.aoEnhanced && p.aoBentNormal) {
          const float w = 0.5f * (dot(bent, p.aoUp) + 1.0f);
          ambLight = f3{p.ambLight.x * (p.aoGround.x + (p.aoSky.x - p.aoGround.x) * w),
                        p.ambLight.y * (p.aoGround.y + (p.aoSky.y - p.aoGround.y) * w),
                        p.ambLight.z * (p.aoGround.z + (p.aoSky.z - p.aoGround.z) * w)};
        }
        if (p.aoMultibounce) {
          const float ox = aoMultibounce(openness, sf.C.x);
          const float oy = aoMultibounce(openness, sf.C.y);
          const float oz = aoMultibounce(openness, sf.C.z);
          aoFactor = f3{1.0f - p.aoIntensity * (1.0f - ox), 1.0f - p.aoIntensity * (1.0f - oy),
                        1.0f - p.aoIntensity * (1.0f - oz)};
        } else {
          const float sv = 1.0f - p.aoIntensity * (1.0f - openness);
          aoFactor = f3{sv, sv, sv};
        }
        if (p.aoDiffuseFactor > 0.0f) diffuseAo = 1.0f - p.aoDiffuseFactor * (1.0f - openness);
      }
      // --- GI (hit_shader.hpp:221-242, 351-365): an eligible hit (mesh, or a
      // real primitive) drops its constant ambient for the gathered indirect
      // the post-pass adds; toon finishes keep a unit ambient and no indirect ---
      if (p.gi && (sf.kind == kMesh || !sf.fromEdge)) {
        if (toonLike(m)) {
          ambLight = f3{1.0f, 1.0f, 1.0f};
        } else {
          giElig = true;
          ambLight = f3{0.0f, 0.0f, 0.0f};
        }
      }
      const f3 C = sf.C, N = sf.N, V = sf.V;
      f3 out;
      // pt2 traced reflection of this hit (HitShade::reflectivity / reflAlpha
      // / reflF0 / reflTangent / reflAspect)
      bool traceRefl = false;
      float rAmt = 0.0f, rAlpha = 0.0f, rAspect = 1.0f;
      f3 rF0{1.0f, 1.0f, 1.0f}, rTan{0.0f, 0.0f, 0.0f};
      if (m.model == 1u) {
        // --- principled direct pass (shading.hpp:88-91 -> principled.hpp) ---
        f3 anisoT{0.0f, 0.0f, 0.0f};
        const bool tanValid = sf.kind != kMesh && !sf.fromEdge && m.pbr_anisotropy != 0.0f &&
                              anisoTangent(s, sf, m.pbr_anisotropy_rotation, anisoT);
        // traced-reflection ownership (hit_shader.hpp:243-270, 426-452): a
        // specular lobe (metallic or dielectric F0 > 0) reflects, Fresnel
        // folded into the pass, alpha = roughness^2 (a mirror below 0.015)
        if (p.pt2Refl && (sf.kind == kMesh || !sf.fromEdge) &&
            (m.pbr_metallic > 1e-4f || m.pbr_specular > 1e-4f)) {
          traceRefl = true;
          rAmt = 1.0f;
          const float dd = 0.08f * m.pbr_specular, tm = m.pbr_metallic;
          rF0 = f3{dd + (C.x - dd) * tm, dd + (C.y - dd) * tm, dd + (C.z - dd) * tm};
          if (p.pt2Glossy) {
            const float a = m.pbr_roughness * m.pbr_roughness;
            rAlpha = a >= 0.015f ? a : 0.0f;
            if (tanValid) {
              rTan = anisoT;
              float an = fabsf(m.pbr_anisotropy);
              if (an > 1.0f) an = 1.0f;
              rAspect = sqrtf(1.0f - 0.9f * an);
            }
          }
        }
        out = shadePrincipled(p, m, sf, lights, b.occ + rb + p.aoSamples, aoFactor, ambLight, diffuseAo, px, py,
                              tanValid ? &anisoT : nullptr, traceRefl);
      } else {
      // --- shadeLocal, POV branch (shading.hpp:96-191) ---
      out = f3{m.emission * C.x + aoFactor.x * m.ambient * C.x * ambLight.x,
               m.emission * C.y + aoFactor.y * m.ambient * C.y * ambLight.y,
               m.emission * C.z + aoFactor.z * m.ambient * C.z * ambLight.z};
      const float ex = blinnExp(m.roughness);
      for (int l = 0; l < p.nLights; ++l) {
        const LightD L = lights[l];
        const float ndl = dot(N, L.L);
        if (ndl <= 0.0f) continue;
        float shadowFactor = 1.0f;
        if (sf.shOn) {
          const uint8_t* o = b.occ + rb + p.aoSamples + L.rayOffset;
          if (!L.soft) {
            shadowFactor = o[0] ? 0.0f : 1.0f;
          } else {
            int hits = 0;
            for (int q = 0; q < L.samples; ++q) hits += o[q];
            shadowFactor = 1.0f - float(hits) / float(L.samples);
          }
        }
        const f3 Lc{L.color.x * shadowFactor, L.color.y * shadowFactor, L.color.z * shadowFactor};
        float d;
        if (m.brilliance == 1.0f) d = ndl;
        else if (m.brilliance == 0.0f) d = 1.0f;
        else d = powf(ndl, m.brilliance);
        const float dk = m.diffuse * d * diffuseAo;
        out.x += dk * C.x * Lc.x;
        out.y += dk * C.y * Lc.y;
        out.z += dk * C.z * Lc.z;
        if (!L.highlight) continue;
        f3 hl;
        if (m.metallic) {
          float c = ndl;
          if (c > 1.0f) c = 1.0f;
          const float x = acosf(c) * 0.63661977f;
          float fr = 0.014567225f / ((x - 1.12f) * (x - 1.12f)) - 0.011612903f;
          if (fr < 0.0f) fr = 0.0f;
          if (fr > 1.0f) fr = 1.0f;
          hl = f3{Lc.x * (fr + (1.0f - fr) * C.x), Lc.y * (fr + (1.0f - fr) * C.y),
                  Lc.z * (fr + (1.0f - fr) * C.z)};
        } else {
          hl = Lc;
        }
        float specW = 0.0f;
        if (m.specular > 0.0f) {
          const f3 H = normalize(f3{L.L.x + V.x, L.L.y + V.y, L.L.z + V.z});
          const float nh = dot(N, H);
          if (nh > 0.0f) specW += m.specular * powf(nh, ex);
        }
        if (m.phong > 0.0f) {
          const f3 Rr = 2.0f * ndl * N - L.L;
          const float rv = dot(Rr, V);
          if (rv > 0.0f && (m.phong_size < 60.0f || rv > 0.0008f)) specW += m.phong * powf(rv, m.phong_size);
        }
        if (specW > 0.0f) {
          const float sc = specW * p.specularScale;
          out.x += sc * hl.x;
          out.y += sc * hl.y;
          out.z += sc * hl.z;
        }
      }
      if (p.pt2Refl && (sf.kind == kMesh || !sf.fromEdge) && m.reflection > 0.0f) {
        traceRefl = true;
        rAmt = m.reflection;
        if (p.pt2Glossy && m.specular > 0.0f) rAlpha = ggxAlphaFromRoughness(m.roughness);
      }
      if (m.reflection > 0.0f && !traceRefl) {
        out.x += m.reflection * p.bg.x;
        out.y += m.reflection * p.bg.y;
        out.z += m.reflection * p.bg.z;
      }
      }
      // --- first-hit capture + compositing (transparency.hpp:394-467) ---
      if (b.depth[gpix] == 0.0f) {
        if (b.aovA && p.aoWriteAov) {
          // first-hit AO AOVs (hit_shader.hpp:207-213: mesh hits only)
          if (sf.kind == kMesh) {
            b.aovA[gpix] = make_float4(sf.C.x, sf.C.y, sf.C.z, aq.contact);
            b.aovB[gpix] = make_float4(sf.N.x, sf.N.y, sf.N.z, aq.shape);
            b.aovC[gpix] = make_float4(aq.bent.x, aq.bent.y, aq.bent.z, aq.avgHit);
          }
        }
        if (b.aaN && p.aaMode == 1) {
          // first-hit shading normal and section for the adaptive-AA mask
          // (hit_shader.hpp:214-220, 277, 321, 457)
          int grp = 0;
          if (sf.kind == kMesh) {
            if (s.meshTriGroup) grp = __ldg(&s.meshTriGroup[s.baseTri ? sf.prim % s.baseTri : sf.prim]);
          } else if (s.primGroup[sf.kind]) {
            grp = __ldg(&s.primGroup[sf.kind][sf.prim]);
          }
          b.aaN[gpix] = make_float4(sf.N.x, sf.N.y, sf.N.z, __int_as_float(grp));
        }
        if (b.aoPatch) b.aoPatch[gpix] = patched ? 1.0f : 0.0f;
        if (b.giA) {
          // first-hit gather seed (transparency.hpp:407-415): position, the
          // face-forwarded shading normal, eligibility and kd * pigment
          const float kd = diffuseWeight(m);
          b.giA[gpix] = make_float4(sf.P.x, sf.P.y, sf.P.z, t);
          b.giB[gpix] = make_float4(sf.N.x, sf.N.y, sf.N.z, giElig ? 1.0f : 0.0f);
          b.giR[gpix] = make_float4(kd * sf.C.x, kd * sf.C.y, kd * sf.C.z, 0.0f);
          if (b.rfl.amt) {
            // the first hit's traced-reflection record (storeShadingChannels,
            // embree_renderer.cpp:194-216)
            b.rfl.amt[gpix] = make_float4(rAmt, rAlpha, rAspect, 0.0f);
            b.rfl.f0[gpix] = make_float4(rF0.x, rF0.y, rF0.z, 0.0f);
            if (b.rfl.tan) b.rfl.tan[gpix] = make_float4(rTan.x, rTan.y, rTan.z, 0.0f);
          }
        }
        if (b.gbObj) {
          // edge G-buffer (hit_shader.hpp:278-300, 460-478; transparency.hpp:394-428)
          uint32_t grp = 0, mat;
          if (sf.kind == kMesh) {
            const uint32_t bt = s.baseTri ? sf.prim % s.baseTri : sf.prim;
            if (s.meshTriGroup) grp = __ldg(&s.meshTriGroup[bt]);
            mat = s.meshTriMatId ? uint32_t(__ldg(&s.meshTriMatId[bt])) : 0u;
          } else {
            if (s.primGroup[sf.kind]) grp = __ldg(&s.primGroup[sf.kind][sf.prim]);
            mat = s.meshMatCount + sf.prim;
            if (sf.kind != kSphere) mat += s.baseSpheres;
            if (sf.kind == kCone) mat += s.roundCount;
          }
          b.gbObj[gpix] = (grp << 2) | uint32_t(sf.kind);
          b.gbMat[gpix] = mat;
          b.gbNrm[3 * size_t(gpix)] = sf.N.x;
          b.gbNrm[3 * size_t(gpix) + 1] = sf.N.y;
          b.gbNrm[3 * size_t(gpix) + 2] = sf.N.z;
          b.gbAlpha[gpix] = sf.opacity;
          float ctn, ctf;
          clipRange(p, rd, ctn, ctf);
          if (b.gbClip && clipOn(p, rd) && ctn > 0.0f && dot(sf.Ng, rd) > 0.0f) b.gbClip[gpix] = 2;
        }
        b.depth[gpix] = t;
        b.viewZ[gpix] = t * dot(rd, p.camDir);
        b.hitGeom[gpix] = s.geomID[sf.kind];
        b.hitPrim[gpix] = sf.prim;
      }
      const float kOpaque = 1.0f - 1e-4f;
      if (!p.transparency || sf.opacity >= kOpaque) {
        base = out;
        baseCov = 1.0f;
      } else {
        const float w = (1.0f - acc.w) * sf.opacity;
        acc.x += w * out.x;
        acc.y += w * out.y;
        acc.z += w * out.z;
        acc.w += w;
        if (!(acc.w >= kOpaque)) {
          const f3 hitP{org.x + rd.x * t, org.y + rd.y * t, org.z + rd.z * t};
          const float dirMax = fmaxf(fabsf(rd.x), fmaxf(fabsf(rd.y), fabsf(rd.z)));
          const float epsScale =
              fmaxf(fmaxf(fabsf(hitP.x), fabsf(hitP.y)), fmaxf(fabsf(hitP.z), dirMax * t));
          const float tn = t + epsScale * 0x1.0fp-21f;
          if (layer == p.maxIters - 1) {
            capped = 1;
          } else {
            b.tnear[gpix] = tn;
            b.accum[gpix] = acc;
            done = false;
            push = true;
          }
        }
      }
    }
    if (done) {
      const float floorW = (1.0f - acc.w) * baseCov;
      float outA = acc.w + floorW;
      outA = fminf(1.0f, fmaxf(0.0f, outA));
      b.colorHi[gpix] = make_float4(acc.x + floorW * base.x, acc.y + floorW * base.y,
                                    acc.z + floorW * base.z, outA);
    }
  }
  int off;
  const int qb = warpPushBase(push, b.counter, off);
  if (push) outQueue[qb + off] = gpix;
  warpCount(&b.stats[2], capped);
}

// Fused finishing pass: fog (fog.cpp:7-36) on each hi-res sample, ss x ss box
// average with the non-finite guard (image_ops.cpp:9-35; only when ss > 1,
// as renderFrame skips the downsample at ss == 1), assumed gamma
// (image_ops.cpp:37-46).
template <bool BATCH>
__global__ void k_post(Params p1, Batch bt, uint32_t nOut, const float4* colorHi, const float* viewZ,
                       float4* out) {
  const uint32_t go = blockIdx.x * blockDim.x + threadIdx.x;
  if (go >= nOut) return;
  const int f = BATCH ? frameOf(bt.outOffs, bt.nFrames, go) : 0;
  const Params& p = BATCH ? bt.frames[f].p : p1;
  const size_t pixOff = BATCH ? bt.frames[f].pixOff : 0u;
  const int o = int(go - (BATCH ? bt.frames[f].outOff : 0u));
  const int ox = o % p.outW, oy = o / p.outW;
  const int ss = p.ss;
  auto fogged = [&](int hx, int hy) {
    const size_t hp = pixOff + size_t(hy) * p.W + hx;
    float4 c = colorHi[hp];
    if (p.fogOn) {
      const float z = viewZ[hp];
      if (z > 0.0f) {
        float f;
        const float denom = p.fogEnd - p.fogStart;
        if (denom <= 0.0f) {
          f = z < p.fogEnd ? 1.0f : 0.0f;
        } else {
          f = (p.fogEnd - z) / denom;
          if (f < 0.0f) f = 0.0f;
          if (f > 1.0f) f = 1.0f;
        }
        if (p.transparentBg) {
          c.w *= f;
        } else {
          c.x = p.fogColor.x * (1.0f - f) + c.x * f;
          c.y = p.fogColor.y * (1.0f - f) + c.y * f;
          c.z = p.fogColor.z * (1.0f - f) + c.z * f;
        }
      }
    }
    return c;
  };
  float4 r;
  if (ss == 1) {
    r = fogged(ox, oy);
  } else {
    float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int dy = 0; dy < ss; ++dy)
      for (int dx = 0; dx < ss; ++dx) {
        const float4 c = fogged(ox * ss + dx, oy * ss + dy);
        a[0] += isfinite(c.x) ? c.x : 0.0f;
        a[1] += isfinite(c.y) ? c.y : 0.0f;
        a[2] += isfinite(c.z) ? c.z : 0.0f;
        a[3] += isfinite(c.w) ? c.w : 0.0f;
      }
    const float inv = 1.0f / float(ss * ss);
    r = make_float4(a[0] * inv, a[1] * inv, a[2] * inv, a[3] * inv);
  }
  const float g = p.gamma;
  if (!(fabsf(g - 1.0f) <= 1.0e-4f)) {
    r.x = r.x > 0.0f ? powf(r.x, g) : 0.0f;
    r.y = r.y > 0.0f ? powf(r.y, g) : 0.0f;
    r.z = r.z > 0.0f ? powf(r.z, g) : 0.0f;
  }
  out[go] = r;
}

// First-hit state of a pixel before its primary ray (all pixels, or the
// pixels of a list when `list` is set).
__global__ void k_init_pixels(uint32_t npix, float* depth, float* viewZ, uint32_t* hg, uint32_t* hp, float4* aovA,
                              float4* aovB, float4* aovC, float4* aaN = nullptr, const uint32_t* list = nullptr,
                              float* aoPatch = nullptr) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= npix) return;
  const uint32_t i = list ? list[k] : k;
  if (aaN) aaN[i] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(-1));
  if (aoPatch) aoPatch[i] = 0.0f;
  depth[i] = 0.0f;
  viewZ[i] = 0.0f;
  hg[i] = kInvalid;
  hp[i] = kInvalid;
  if (aovA) {  // neutral AOVs of a pixel without a mesh first hit
    aovA[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    aovB[i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);
    aovC[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}

// AO AOVs to the output resolution: box average with the non-finite guard
// (pipeline.cpp:182-206 boxDownsample of albedo / normal / contact / shape /
// avgHitDist / bentNormal; a copy at ss == 1), unpacked into the FrameResult
// plane layouts (3, 3, 3, 1, 1, 1 floats per pixel).
template <bool BATCH>
__global__ void k_post_aov(Params p1, Batch bt, uint32_t nOut, const float4* aovA, const float4* aovB,
                           const float4* aovC, float* alb, float* nrm, float* bent, float* con, float* shp,
                           float* avg) {
  const uint32_t go = blockIdx.x * blockDim.x + threadIdx.x;
  if (go >= nOut) return;
  const int f = BATCH ? frameOf(bt.outOffs, bt.nFrames, go) : 0;
  const Params& p = BATCH ? bt.frames[f].p : p1;
  const size_t pixOff = BATCH ? bt.frames[f].pixOff : 0u;
  const int o = int(go - (BATCH ? bt.frames[f].outOff : 0u));
  const int ox = o % p.outW, oy = o / p.outW;
  const int ss = p.ss;
  float a[12];
  if (ss == 1) {
    const size_t hp = pixOff + size_t(oy) * p.W + ox;
    const float4 A = aovA[hp], B = aovB[hp], C = aovC[hp];
    const float v[12] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w, C.x, C.y, C.z, C.w};
    for (int k = 0; k < 12; ++k) a[k] = v[k];
  } else {
    for (int k = 0; k < 12; ++k) a[k] = 0.0f;
    for (int dy = 0; dy < ss; ++dy)
      for (int dx = 0; dx < ss; ++dx) {
        const size_t hp = pixOff + size_t(oy * ss + dy) * p.W + size_t(ox * ss + dx);
        const float4 A = aovA[hp], B = aovB[hp], C = aovC[hp];
        const float v[12] = {A.x, A.y, A.z, A.w, B.x, B.y, B.z, B.w, C.x, C.y, C.z, C.w};
        for (int k = 0; k < 12; ++k) a[k] += isfinite(v[k]) ? v[k] : 0.0f;
      }
    const float inv = 1.0f / float(ss * ss);
    for (int k = 0; k < 12; ++k) a[k] *= inv;
  }
  alb[3 * size_t(go)] = a[0]; alb[3 * size_t(go) + 1] = a[1]; alb[3 * size_t(go) + 2] = a[2];
  con[go] = a[3];
  nrm[3 * size_t(go)] = a[4]; nrm[3 * size_t(go) + 1] = a[5]; nrm[3 * size_t(go) + 2] = a[6];
  shp[go] = a[7];
  bent[3 * size_t(go)] = a[8]; bent[3 * size_t(go) + 1] = a[9]; bent[3 * size_t(go) + 2] = a[10];
  avg[go] = a[11];
}

// ---- Adaptive AA (embree_renderer.cpp:1379-1670, render/adaptive_aa.hpp) ----
// Phase 1 shades the centre subpixel (ss/2, ss/2) of each output pixel; the
// refinement mask compares 4-neighbour centre pairs and is dilated once; the
// flagged blocks shade their remaining subpixels, the others replicate their
// centre (re-shaded first with ss^2 AO / soft-shadow samples).
struct AaGrid {
  const float4* color;  // hi-res colour before fog
  const float* viewZ;
  const uint32_t* geom;
  const float4* nrm;    // first-hit normal.xyz, section id (int bits)
  int W, ss, cSub, Wf, Hf;
  float thr, pixelWorldSize;
  int persp;
};

UBR_D uint32_t aaCentre(const AaGrid& g, int x, int y) {
  return uint32_t(y * g.ss + g.cSub) * uint32_t(g.W) + uint32_t(x * g.ss + g.cSub);
}

// aaPairNeedsRefine (adaptive_aa.hpp:65-111): a and b are neighbouring
// centres, za0 / zb1 the view z one step beyond each (or extrapolated).
UBR_D bool aaPairRefine(const AaGrid& g, uint32_t a, uint32_t b, float za0, float zb1) {
  const uint32_t ga = g.geom[a], gb = g.geom[b];
  const float4 na = g.nrm[a], nb = g.nrm[b];
  if (ga != gb || __float_as_int(na.w) != __float_as_int(nb.w)) return true;
  const float4 ca = g.color[a], cb = g.color[b];
  if (fabsf(ca.x - cb.x) > g.thr || fabsf(ca.y - cb.y) > g.thr || fabsf(ca.z - cb.z) > g.thr ||
      fabsf(ca.w - cb.w) > g.thr)
    return true;
  if (ga == kInvalid || gb == kInvalid) return false;
  const float la = na.x * na.x + na.y * na.y + na.z * na.z;
  const float lb = nb.x * nb.x + nb.y * nb.y + nb.z * nb.z;
  if (la > 0.0f && lb > 0.0f) {
    const float dd = na.x * nb.x + na.y * nb.y + na.z * nb.z;
    if (1.0f - dd > 0.3f) return true;
  }
  const float za = g.viewZ[a], zb = g.viewZ[b];
  const float step = fabsf(zb - za);
  const float sa = fabsf(za - za0), sb = fabsf(zb1 - zb);
  const float slope = sa < sb ? sa : sb;
  float absTerm = 12.0f * g.pixelWorldSize;
  if (g.persp) absTerm *= fabsf(za) < fabsf(zb) ? fabsf(za) : fabsf(zb);
  const float th = 3.0f * slope > absTerm ? 3.0f * slope : absTerm;
  return step > th;
}

// Horizontal pair (x0, x0 + 1) or vertical pair (y0, y0 + 1) of buildAaMask
// (adaptive_aa.hpp:132-161).
UBR_D bool aaPairH(const AaGrid& g, int x0, int y) {
  const uint32_t a = aaCentre(g, x0, y), b = aaCentre(g, x0 + 1, y);
  const float za = g.viewZ[a], zb = g.viewZ[b];
  const float za0 = x0 > 0 ? g.viewZ[aaCentre(g, x0 - 1, y)] : 2.0f * za - zb;
  const float zb1 = x0 + 2 < g.Wf ? g.viewZ[aaCentre(g, x0 + 2, y)] : 2.0f * zb - za;
  return aaPairRefine(g, a, b, za0, zb1);
}
UBR_D bool aaPairV(const AaGrid& g, int x, int y0) {
  const uint32_t a = aaCentre(g, x, y0), b = aaCentre(g, x, y0 + 1);
  const float za = g.viewZ[a], zb = g.viewZ[b];
  const float za0 = y0 > 0 ? g.viewZ[aaCentre(g, x, y0 - 1)] : 2.0f * za - zb;
  const float zb1 = y0 + 2 < g.Hf ? g.viewZ[aaCentre(g, x, y0 + 2)] : 2.0f * zb - za;
  return aaPairRefine(g, a, b, za0, zb1);
}

// centre subpixel of every output pixel, in output raster order
__global__ void k_aa_centres(AaGrid g, uint32_t* list) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= uint32_t(g.Wf) * uint32_t(g.Hf)) return;
  list[o] = aaCentre(g, int(o % uint32_t(g.Wf)), int(o / uint32_t(g.Wf)));
}

// raw mask: an output pixel is flagged when any of its (up to four) pairs is
__global__ void k_aa_raw(AaGrid g, uint8_t* raw) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= uint32_t(g.Wf) * uint32_t(g.Hf)) return;
  const int x = int(o % uint32_t(g.Wf)), y = int(o / uint32_t(g.Wf));
  bool r = (x > 0 && aaPairH(g, x - 1, y)) || (x + 1 < g.Wf && aaPairH(g, x, y)) ||
           (y > 0 && aaPairV(g, x, y - 1)) || (y + 1 < g.Hf && aaPairV(g, x, y));
  raw[o] = r ? 1 : 0;
}

// dilateMask3x3 (adaptive_aa.hpp:35-56), then the work lists: every
// non-centre subpixel of a flagged block (every subpixel when `withCentre`,
// for the fine lattice), and the centre of every other block; `maskOut`
// (output resolution, 1 = refined) when requested.
__global__ void k_aa_lists(AaGrid g, const uint8_t* raw, uint32_t* flagged, uint32_t* centres,
                           uint32_t* counts, float* maskOut, bool withCentre) {
  const uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = o < uint32_t(g.Wf) * uint32_t(g.Hf);
  int x = 0, y = 0;
  bool m = false;
  if (valid) {
    x = int(o % uint32_t(g.Wf));
    y = int(o / uint32_t(g.Wf));
    for (int dy = -1; dy <= 1 && !m; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int xx = x + dx, yy = y + dy;
        if (xx < 0 || yy < 0 || xx >= g.Wf || yy >= g.Hf) continue;
        if (raw[uint32_t(yy) * uint32_t(g.Wf) + uint32_t(xx)]) {
          m = true;
          break;
        }
      }
    if (maskOut) maskOut[o] = m ? 1.0f : 0.0f;
  }
  const uint32_t c = valid ? aaCentre(g, x, y) : 0u;
  int off;
  int base = warpPushBase(valid && !m, &counts[1], off);
  if (valid && !m) centres[base + off] = c;
  // subpixel k of each flagged block in this warp lands in one contiguous run
  const int n2 = g.ss * g.ss;
  for (int k = 0; k < n2; ++k) {
    const int i = k % g.ss, j = k / g.ss;
    const bool push = valid && m && (withCentre || !(i == g.cSub && j == g.cSub));
    base = warpPushBase(push, &counts[0], off);
    if (push) flagged[base + off] = uint32_t(y * g.ss + j) * uint32_t(g.W) + uint32_t(x * g.ss + i);
  }
}

// unflagged blocks: the centre's first-hit state and colour to every subpixel
__global__ void k_aa_replicate(AaGrid g, const uint32_t* centres, const uint32_t* counts, float4* color,
                               float* depth, float* viewZ, uint32_t* hg, uint32_t* hp, float4* aovA, float4* aovB,
                               float4* aovC, float* aoPatch) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= counts[1]) return;
  const uint32_t c = centres[k];
  const int cx = int(c % uint32_t(g.W)), cy = int(c / uint32_t(g.W));
  const int x0 = cx - g.cSub, y0 = cy - g.cSub;
  const float4 col = color[c];
  const float d = depth[c], z = viewZ[c];
  const uint32_t gi = hg[c], pi = hp[c];
  const float patch = aoPatch ? aoPatch[c] : 0.0f;
  float4 a = make_float4(0, 0, 0, 0), b2 = a, c3 = a;
  if (aovA) {
    a = aovA[c];
    b2 = aovB[c];
    c3 = aovC[c];
  }
  for (int j = 0; j < g.ss; ++j)
    for (int i = 0; i < g.ss; ++i) {
      const uint32_t t = uint32_t(y0 + j) * uint32_t(g.W) + uint32_t(x0 + i);
      if (t == c) continue;
      color[t] = col;
      depth[t] = d;
      viewZ[t] = z;
      hg[t] = gi;
      hp[t] = pi;
      if (aoPatch) aoPatch[t] = patch;
      if (aovA) {
        aovA[t] = a;
        aovB[t] = b2;
        aovC[t] = c3;
      }
    }
}

// Fine-lattice samples of the flagged cells (embree_renderer.cpp:1542-1590):
// chunk sample t is point (t % k, t / k % k) of cell cell0 + t / k^2 on the
// (W k) x (H k) lattice.
__global__ void k_aa_fine_coords(AaGrid g, const uint32_t* cells, uint32_t cell0, uint32_t n, int k,
                                 uint32_t* coord) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const uint32_t uk = uint32_t(k), k2 = uk * uk;
  const uint32_t cell = cells[cell0 + t / k2], sub = t % k2;
  const uint32_t cx = cell % uint32_t(g.W), cy = cell / uint32_t(g.W);
  coord[t] = (cy * uk + sub / uk) * (uint32_t(g.W) * uk) + cx * uk + sub % uk;
}

// Box average of each cell's k^2 samples into the hi-res buffers: colour,
// depth and view z summed in sample order then scaled by 1 / k^2; first hit
// and AOVs from the first sample.
__global__ void k_aa_fine_reduce(const uint32_t* cells, uint32_t cell0, uint32_t nCells, int k, Bufs fine, Bufs b) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nCells) return;
  const uint32_t k2 = uint32_t(k) * uint32_t(k);
  const uint32_t c = cells[cell0 + t];
  const uint32_t s0 = t * k2;
  float4 acc = fine.colorHi[s0];
  float d = fine.depth[s0], z = fine.viewZ[s0];
  for (uint32_t q = 1; q < k2; ++q) {
    const float4 v = fine.colorHi[s0 + q];
    acc.x += v.x;
    acc.y += v.y;
    acc.z += v.z;
    acc.w += v.w;
    d += fine.depth[s0 + q];
    z += fine.viewZ[s0 + q];
  }
  const float inv = 1.0f / float(k2);
  b.colorHi[c] = make_float4(acc.x * inv, acc.y * inv, acc.z * inv, acc.w * inv);
  b.depth[c] = d * inv;
  b.viewZ[c] = z * inv;
  b.hitGeom[c] = fine.hitGeom[s0];
  b.hitPrim[c] = fine.hitPrim[s0];
  if (b.aoPatch) b.aoPatch[c] = fine.aoPatch[s0];
  if (b.aovA) {
    b.aovA[c] = fine.aovA[s0];
    b.aovB[c] = fine.aovB[s0];
    b.aovC[c] = fine.aovC[s0];
  }
}

// ---- Coarse-grid AO pre-pass (embree_renderer.cpp:527-553) ----
// The first-hit G-buffer of the coarse grid (pt1_gbuffer.hpp:83-196: primary
// rays through the cell centres of the same camera plane, no clip range; mesh
// hits with the interpolated normal, non-outline primitives with the
// geometric one, both turned toward the viewer) and, per eligible cell, the
// surface record of its AO gather (ao_coarse.hpp:73-140: epsilon from the hit
// distance with N in place of the ray direction).  `pc` is the frame's
// parameters with W x H = the coarse grid, so AO seeds live on that lattice.
template <bool COUNT, int KM, bool BATCH>
__global__ void __launch_bounds__(128) k_cao_trace(Params pc, DScene s, Bufs b, float4* cgN, uint8_t* cgHit) {
  const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nc = uint32_t(pc.W) * uint32_t(pc.H);
  bool cast = false;
  if (cell < nc) {
    const int cx = int(cell % uint32_t(pc.W)), cy = int(cell / uint32_t(pc.W));
    f3 org, rd;
    primaryRay(pc, cx, cy, org, rd);
    Ray r{org, rd, 0.0f, kInfF};
    Hit h;
    uint32_t ovf = 0;
    Count cnt;
    traverse<false, KM>(travOf(s), r, h, ovf, &cnt, false);
    uint8_t eligible = 0;
    f3 N{0.0f, 0.0f, 0.0f}, Ng{0.0f, 0.0f, 0.0f};
    if (h.ref != kInvalid) {
      const int kind = refKind(h.ref);
      const uint32_t prim = refPrim(h.ref);
      if (kind == kMesh) {
        const uint32_t i0 = __ldg(&s.meshIdx[3 * prim]), i1 = __ldg(&s.meshIdx[3 * prim + 1]),
                       i2 = __ldg(&s.meshIdx[3 * prim + 2]);
        const float w0 = 1.0f - h.u - h.v;
        float nb[3];
        for (int k = 0; k < 3; ++k)
          nb[k] = w0 * __ldg(&s.meshNrm[3 * i0 + k]) + h.u * __ldg(&s.meshNrm[3 * i1 + k]) +
                  h.v * __ldg(&s.meshNrm[3 * i2 + k]);
        N = safeNormalize(f3{nb[0], nb[1], nb[2]});
        Ng = safeNormalize(h.Ng);
        eligible = 1;
      } else if (!__ldg(&s.primFromEdge[kind][prim])) {
        N = safeNormalize(h.Ng);
        Ng = N;
        eligible = 1;
      }
    }
    cgHit[cell] = eligible;
    if (eligible) {
      if (dot(N, rd) > 0.0f) N = neg(N);
      if (dot(Ng, rd) > 0.0f) Ng = neg(Ng);
      const float t = h.t;
      cgN[cell] = make_float4(N.x, N.y, N.z, t);
      const f3 P{org.x + rd.x * t, org.y + rd.y * t, org.z + rd.z * t};
      const float eps = selfIntersectEps(P, N, t);
      f3 ng = dot(Ng, N) < 0.0f ? neg(Ng) : Ng;
      ng = safeNormalize(ng, N);
      const f3 O = P + ng * eps;
      f3 lo, hi;
      aoBox(O, pc.aoDistance, lo, hi);
      const int start = boxStartNode(travOf(s), lo, hi);
      b.surfA[cell] = make_float4(O.x, O.y, O.z, eps);
      b.surfB[cell] = make_float4(N.x, N.y, N.z, __int_as_float(start));
      const Frame3 fr = frameFromNormal(N);
      b.surfT[cell] = make_float4(fr.t.x, fr.t.y, fr.t.z, 0.0f);
      b.surfC[cell] = make_uint2(cell, 3u);
      cast = true;
    }
  }
  int off;
  const int qb = warpPushBase(cast, b.counter + 1, off);
  if (cast) b.occQueue[qb + off] = cell;
}

// Per eligible cell, the AO estimate from its rays (aoGather,
// ao_shade.hpp:44-72): binary openness, or the quality estimator when AO is
// enhanced; with AOVs requested the legacy openness plus a single-scale
// quality pass.
__global__ void k_cao_finish(Params pc, Bufs b, const uint8_t* cgHit, float4* cgQ, float4* cgB) {
  const uint32_t cell = blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= uint32_t(pc.W) * uint32_t(pc.H) || !cgHit[cell]) return;
  const int cx = int(cell % uint32_t(pc.W)), cy = int(cell / uint32_t(pc.W));
  const uint64_t n = uint64_t(pc.aoSamples);
  const f3 N = ld3(b.surfB[cell]);
  AoQ q;
  if (!pc.aoEnhanced) {
    int hits = 0;
    for (uint64_t k = 0; k < n; ++k) hits += b.occ[uint64_t(cell) * n + k];
    const float openness = 1.0f - float(hits) / float(pc.aoSamples);
    if (pc.aoWriteAov) q = aoQuality(pc, b.aoT, n, cell, N, cx, cy, 0.0f, false);
    q.openness = openness;
  } else {
    q = aoQuality(pc, b.aoT, n, cell, N, cx, cy, pc.aoFalloffPower, pc.aoMultiScale != 0);
  }
  cgQ[cell] = make_float4(q.openness, q.contact, q.shape, q.avgHit);
  if (cgB) cgB[cell] = make_float4(q.bent.x, q.bent.y, q.bent.z, 0.0f);
}

// ---- Edge G-buffer (transparency.hpp:131-186, 394-428, 470-481) ----
__global__ void k_gb_init(uint32_t npix, Bufs b) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  b.gbObj[i] = kInvalid;
  b.gbMat[i] = kInvalid;
  b.gbNrm[3 * size_t(i)] = 0.0f;
  b.gbNrm[3 * size_t(i) + 1] = 0.0f;
  b.gbNrm[3 * size_t(i) + 2] = 0.0f;
  b.gbAlpha[i] = 1.0f;
  if (b.gbClip) {
    b.gbClip[i] = 0;
    b.gbNear[i] = 0.0f;
    b.gbFar[i] = 0.0f;
  }
}

// With clip planes: a backface first hit is a clip-cut interior when an
// any-hit ray finds the clipped-away front over [max(1e-4, 1e-4 tn),
// tn (1 - 1e-4)); a background pixel records the view z of the first
// surface removed in front of the near plane and beyond the far plane.
template <int KM>
__global__ void __launch_bounds__(128) k_gb_clip(Params p, DScene s, Bufs b, uint32_t npix) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npix) return;
  const int px = int(i % uint32_t(p.W)), py = int(i / uint32_t(p.W));
  f3 org, rd;
  primaryRay(p, px, py, org, rd);
  if (!clipOn(p, rd)) return;
  float ctn, ctf;
  clipRange(p, rd, ctn, ctf);
  const TravScene ts = travOf(s);
  uint32_t ovf = 0;
  Count cnt;
  if (b.gbClip[i] == 2) {
    const float tn = fmaxf(1.0e-4f, 1.0e-4f * ctn), tf = ctn * (1.0f - 1.0e-4f);
    bool front = false;
    if (tn < tf) {
      Hit h;
      front = traverse<false, KM>(ts, Ray{org, rd, tn, tf}, h, ovf, &cnt, true);
    }
    b.gbClip[i] = front ? 1 : 0;
  } else if (b.hitGeom[i] == kInvalid) {
    const float camCos = dot(rd, p.camDir);
    if (ctn > 0.0f) {
      const float t0 = fmaxf(1.0e-4f, 1.0e-6f * ctn), t1 = ctn * (1.0f - 1.0e-6f);
      if (t0 < t1) {
        Hit h;
        if (traverse<false, KM>(ts, Ray{org, rd, t0, t1}, h, ovf, &cnt, false)) b.gbNear[i] = h.t * camCos;
      }
    }
    if (ctf < kInfF) {
      const float t0 = ctf * (1.0f + 1.0e-6f);
      if (t0 < kInfF) {
        Hit h;
        if (traverse<false, KM>(ts, Ray{org, rd, t0, kInfF}, h, ovf, &cnt, false)) b.gbFar[i] = h.t * camCos;
      }
    }
  }
}

// ---- A-trous denoiser (experimental/irradiance_cache/denoise_atrous.cpp:27-220,
// pipeline.cpp:224-252) on the final-resolution linear colour, guided by the
// AO AOV normal (and albedo, demodulated); no position guide without GI ----
__global__ void k_dn_init(uint32_t n, const float4* color, const float* nrm, const float* alb, uint8_t* valid,
                          float* irr) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float nx = nrm[3 * size_t(p)], ny = nrm[3 * size_t(p) + 1], nz = nrm[3 * size_t(p) + 2];
  valid[p] = (nx * nx + ny * ny + nz * nz) > 0.25f ? 1 : 0;
  const float4 c = color[p];
  const float cv[3] = {c.x, c.y, c.z};
  for (int k = 0; k < 3; ++k) {
    float v = cv[k];
    if (alb) {
      const float a = alb[3 * size_t(p) + k];
      v /= (a > 1.0e-3f ? a : 1.0e-3f);
    }
    irr[3 * size_t(p) + k] = v;
  }
}

// luminance variance over the valid 3x3 neighbourhood
__global__ void k_dn_var(int W, int H, const uint8_t* valid, const float* irr, float* var) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= uint32_t(W) * uint32_t(H)) return;
  float v = 0.0f;
  if (valid[p]) {
    const int x = int(p % uint32_t(W)), y = int(p / uint32_t(W));
    float sm = 0.0f, s2 = 0.0f;
    int n = 0;
    for (int dy = -1; dy <= 1; ++dy)
      for (int dx = -1; dx <= 1; ++dx) {
        const int qx = x + dx, qy = y + dy;
        if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
        const size_t q = size_t(qy) * W + qx;
        if (!valid[q]) continue;
        const float l = lumOf(irr[3 * q], irr[3 * q + 1], irr[3 * q + 2]);
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
}

__global__ void k_dn_lum(uint32_t n, const float* irr, float* lum) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) lum[p] = lumOf(irr[3 * size_t(p)], irr[3 * size_t(p) + 1], irr[3 * size_t(p) + 2]);
}

// one a-trous iteration: 5x5 B3 taps at 2^it spacing, normal^sigmaN and
// exp(-|dl| / (sigmaL sqrt(var) + 1e-3)) edge-stops
__global__ void k_dn_iter(int W, int H, int step, const uint8_t* valid, const float* nrm, const float* irr,
                          const float* lum, const float* var, float sigmaN, float sigmaL, float* next) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= uint32_t(W) * uint32_t(H)) return;
  if (!valid[p]) {
    next[3 * size_t(p)] = irr[3 * size_t(p)];
    next[3 * size_t(p) + 1] = irr[3 * size_t(p) + 1];
    next[3 * size_t(p) + 2] = irr[3 * size_t(p) + 2];
    return;
  }
  const float h5[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
  const int x = int(p % uint32_t(W)), y = int(p / uint32_t(W));
  const f3 np{nrm[3 * size_t(p)], nrm[3 * size_t(p) + 1], nrm[3 * size_t(p) + 2]};
  const float lp = lum[p];
  const float lDenom = sigmaL * sqrtf(var[p]) + 1.0e-3f;
  float sum[3] = {0.0f, 0.0f, 0.0f};
  float wsum = 0.0f;
  for (int dy = -2; dy <= 2; ++dy) {
    const int qy = y + dy * step;
    if (qy < 0 || qy >= H) continue;
    for (int dx = -2; dx <= 2; ++dx) {
      const int qx = x + dx * step;
      if (qx < 0 || qx >= W) continue;
      const size_t q = size_t(qy) * W + qx;
      if (!valid[q]) continue;
      float w = h5[dx + 2] * h5[dy + 2];
      const f3 nq{nrm[3 * q], nrm[3 * q + 1], nrm[3 * q + 2]};
      const float nd = fmaxf(0.0f, dot(np, nq));
      w *= powf(nd, sigmaN);
      w *= expf(-fabsf(lp - lum[q]) / lDenom);
      sum[0] += w * irr[3 * q];
      sum[1] += w * irr[3 * q + 1];
      sum[2] += w * irr[3 * q + 2];
      wsum += w;
    }
  }
  for (int k = 0; k < 3; ++k) next[3 * size_t(p) + k] = wsum > 0.0f ? sum[k] / wsum : irr[3 * size_t(p) + k];
}

__global__ void k_dn_write(uint32_t n, const uint8_t* valid, const float* irr, const float* alb, float4* color) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n || !valid[p]) return;
  float v[3];
  for (int k = 0; k < 3; ++k) {
    v[k] = irr[3 * size_t(p) + k];
    if (alb) v[k] *= alb[3 * size_t(p) + k];
    v[k] = fmaxf(0.0f, v[k]);
  }
  color[p] = make_float4(v[0], v[1], v[2], color[p].w);
}

// applyAssumedGamma (image_ops.cpp:37-46) after the denoiser
__global__ void k_gamma(uint32_t n, float4* color, float g) {
  const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  float4 r = color[p];
  r.x = r.x > 0.0f ? powf(r.x, g) : 0.0f;
  r.y = r.y > 0.0f ? powf(r.y, g) : 0.0f;
  r.z = r.z > 0.0f ? powf(r.z, g) : 0.0f;
  color[p] = r;
}

}  // namespace

// Host-side parameter setup: computeCameraBasis (embree_renderer.cpp:375-386),
// buildSceneLights (:436-458) and buildEnvDomeLights (ao/env_dome.hpp:33-64),
// evaluated in float on the host exactly as the reference does.
ubr_status makeParams(Context* c, const ubr_render_desc& d, Params& p, std::vector<LightD>& lights) {
  if (d.abi_version != UBR_ABI_VERSION) return setError(c, UBR_INVALID_ARGUMENT, "render desc: abi_version mismatch");
  if (d.width <= 0 || d.height <= 0) return setError(c, UBR_INVALID_ARGUMENT, "render desc: width/height must be > 0");
  const int ss = d.supersample < 1 ? 1 : d.supersample;
  if (d.gi) {
    if (d.gi_integrator != 1 && d.gi_integrator != 2)
      return setError(c, UBR_INVALID_ARGUMENT, "render desc: gi needs gi_integrator 1 (pt1) or 2 (pt2)");
    if (d.gi_integrator == 2 && (d.pt2_pattern < 0 || d.pt2_pattern > 1))
      return setError(c, UBR_INVALID_ARGUMENT, "render desc: pt2_pattern must be 0 (Sobol) or 1 (blue noise)");
    if (d.gi_integrator == 2 && d.pt2_reflect && d.pt2_glossy && d.pt2_glossy_spp < 1)
      return setError(c, UBR_INVALID_ARGUMENT, "render desc: pt2_glossy_spp must be >= 1");
    if (d.pt1_spp < 1 || d.gi_bounces < 1)
      return setError(c, UBR_INVALID_ARGUMENT, "render desc: gi needs pt1_spp >= 1 and gi_bounces >= 1");
    if (d.pt1_gather_div < -1)
      return setError(c, UBR_INVALID_ARGUMENT, "render desc: pt1_gather_div must be -1, 0 or a divisor >= 1");
    if (d.aa_mode == 1) return setError(c, UBR_INVALID_ARGUMENT, "render desc: adaptive AA is not supported with gi");
    if ((d.ao_res_div < 0 ? ss : d.ao_res_div) > 1 && d.ao_samples > 0)
      return setError(c, UBR_INVALID_ARGUMENT, "render desc: coarse-grid AO is not supported with gi");
  }
  if (int64_t(d.width) * ss * int64_t(d.height) * ss >= (1ll << 31))
    return setError(c, UBR_INVALID_ARGUMENT, "render desc: supersampled frame too large");
  if (d.light_count && !d.lights) return setError(c, UBR_INVALID_ARGUMENT, "render desc: lights is NULL");
  if (d.ao_samples < 0) return setError(c, UBR_INVALID_ARGUMENT, "render desc: ao_samples < 0");
  std::memset(&p, 0, sizeof(p));
  p.ss = ss;
  p.outW = d.width;
  p.outH = d.height;
  p.W = d.width * ss;
  p.H = d.height * ss;
  const float aspect = float(p.W) / float(p.H);
  p.camPos = f3{d.cam_position[0], d.cam_position[1], d.cam_position[2]};
  p.camDir = normalize(f3{d.cam_direction[0], d.cam_direction[1], d.cam_direction[2]});
  p.right = normalize(cross(p.camDir, f3{d.cam_up[0], d.cam_up[1], d.cam_up[2]}));
  p.up = normalize(cross(p.right, p.camDir));
  p.halfH = d.cam_height * 0.5f;
  p.halfW = p.halfH * aspect;
  p.persHalfH = std::tan(radiansf(d.cam_fovy) * 0.5f);
  p.persHalfW = p.persHalfH * aspect;
  p.ortho = d.cam_orthographic ? 1 : 0;
  p.clipNear = d.clip_near;
  p.clipFar = d.clip_far;
  p.ambLight = f3{d.ambient_color[0], d.ambient_color[1], d.ambient_color[2]};
  p.bg = f3{d.background[0], d.background[1], d.background[2]};
  p.aoUp = d.ao_use_camera_up ? p.up : safeNormalize(f3{d.ao_up[0], d.ao_up[1], d.ao_up[2]}, p.up);
  p.aoSamples = d.ao_samples;
  p.aoDistance = d.ao_distance;
  p.aoIntensity = d.ao_intensity;
  p.aoFalloffPower = d.ao_falloff_power;
  p.aoMultiScale = d.ao_multiscale != 0;
  p.aoBentNormal = d.ao_bent_normal != 0;
  p.aoMultibounce = d.ao_multibounce != 0;
  p.aoLowDiscrepancy = d.ao_low_discrepancy != 0;
  p.aoSky = f3{d.ao_sky_color[0], d.ao_sky_color[1], d.ao_sky_color[2]};
  p.aoGround = f3{d.ao_ground_color[0], d.ao_ground_color[1], d.ao_ground_color[2]};
  p.aoDiffuseFactor = d.ao_diffuse_factor;
  p.aoWriteAov = d.ao_write_aov ? 1 : 0;
  p.gi = d.gi ? 1 : 0;
  p.giIntensity = d.gi_intensity;
  p.pt2Refl = (d.gi && d.gi_integrator == 2 && d.pt2_reflect) ? 1 : 0;
  p.pt2Glossy = (p.pt2Refl && d.pt2_glossy) ? 1 : 0;
  p.aaMode = d.aa_mode == 1 ? 1 : 0;  // any other value renders the full grid
  p.aaThreshold = d.aa_threshold;
  p.aoEnhanced = (d.ao_falloff_power > 0.0f || d.ao_multiscale || d.ao_bent_normal || d.ao_multibounce ||
                  d.ao_low_discrepancy || d.ao_diffuse_factor > 0.0f)
                     ? 1
                     : 0;
  p.shadowsActive = (d.shadows || d.env_lights > 0) ? 1 : 0;
  p.shadowSamples = d.shadow_samples;
  p.specularScale = d.specular_scale;
  p.transparency = d.transparency ? 1 : 0;
  p.transparentBg = d.transparent_background ? 1 : 0;
  p.maxIters = d.transparency ? (d.max_transparent_layers + 1) : 1;
  if (p.maxIters < 1) p.maxIters = 1;
  p.fogOn = d.fog_enabled ? 1 : 0;
  p.fogColor = f3{d.fog_color[0], d.fog_color[1], d.fog_color[2]};
  p.fogStart = d.fog_start;
  p.fogEnd = d.fog_end;
  p.gamma = d.assumed_gamma;
  // lights
  lights.clear();
  for (uint32_t i = 0; i < d.light_count; ++i) {
    const ubr_light& dl = d.lights[i];
    LightD l{};
    l.L = normalize(f3{-dl.direction[0], -dl.direction[1], -dl.direction[2]});
    l.color = f3{dl.color[0] * dl.intensity, dl.color[1] * dl.intensity, dl.color[2] * dl.intensity};
    l.highlight = dl.casts_highlight ? 1u : 0u;
    l.radius = (d.gi_integrator == 2 && dl.angular_radius > 0.0f) ? dl.angular_radius : radiansf(d.light_radius_deg);
    lights.push_back(l);
  }
  if (d.env_lights > 0) {
    for (LightD& l : lights) l.color = l.color * d.env_key_scale;
    const int n = d.env_lights;
    const float cosMax = std::cos(radiansf(d.env_angle));
    const float ga = 3.14159265f * (3.0f - std::sqrt(5.0f));
    float cosSum = 0.0f;
    std::vector<f3> dirs;
    for (int i = 0; i < n; ++i) {
      const float z = 1.0f - (1.0f - cosMax) * ((i + 0.5f) / n);
      const float r = std::sqrt(std::max(0.0f, 1.0f - z * z));
      const float t = ga * i;
      dirs.push_back(normalize(p.camDir * z + p.right * (r * std::cos(t)) + p.up * (r * std::sin(t))));
      cosSum += z;
    }
    const float perLight = cosSum > 0.0f ? d.env_intensity / cosSum : 0.0f;
    for (const f3& dd : dirs) {
      LightD l{};
      l.L = f3{-dd.x, -dd.y, -dd.z};
      l.color = f3{perLight, perLight, perLight};
      l.highlight = 0u;
      l.radius = radiansf(d.light_radius_deg);
      lights.push_back(l);
    }
  }
  if (lights.size() > size_t(kMaxLights)) return setError(c, UBR_INVALID_ARGUMENT, "too many lights (max 64)");
  int off = 0;
  for (LightD& l : lights) {
    l.soft = (d.shadow_samples > 1 && l.radius > 0.0f) ? 1u : 0u;
    l.samples = l.soft ? d.shadow_samples : 1;
    l.rayOffset = off;
    off += l.samples;
  }
  p.nLights = int(lights.size());
  p.shadowRays = p.shadowsActive ? off : 0;
  p.raysPerHit = p.aoSamples + p.shadowRays;
  return UBR_OK;
}

namespace {

// EmbreeRenderer::occluded plain any-hit branch (embree_renderer.cpp:294-315):
// the open segment (p, q) trimmed by max(eps*len, eps) and len*(1-eps).
__global__ void k_occluded_segments(DScene s, const float* segs, uint64_t n, float eps, uint8_t* out,
                                    unsigned long long* stats) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint32_t ovf = 0;
  if (i < n) {
    const float* q = segs + 6 * i;
    const f3 a{q[0], q[1], q[2]}, bq{q[3], q[4], q[5]};
    const f3 d = bq - a;
    const float len = length(d);
    uint8_t res = 0;
    if (len > 0.0f) {
      const f3 dir{d.x / len, d.y / len, d.z / len};
      const float tnear = fmaxf(eps * len, eps);
      const float tfar = len * (1.0f - eps);
      if (tnear < tfar) {
        Ray r{a, dir, tnear, tfar};
        Hit h;
        res = traverse<false, kMaskAll, true>(travOf(s), r, h, ovf, nullptr, true) ? 1 : 0;
      }
    }
    out[i] = res;
  }
  warpCount(&stats[3], ovf);
}

// EmbreeRenderer::occluded with its argument filter (embree_renderer.cpp:
// 294-357): the same trimmed open segment, any hit that the segment's filter
// accepts (own mesh faces, grazing faces and coincident planes are skipped;
// the plain any-hit test when nothing is filtered).
__global__ void k_occluded_filtered(DScene s, const float* segs, uint64_t n, float eps, float grazeCos,
                                    float coplanar, const uint32_t* offs, const int32_t* faces, int meshPresent,
                                    uint8_t* out, unsigned long long* stats) {
  const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  uint32_t ovf = 0;
  if (i < n) {
    const float* q = segs + 6 * i;
    const f3 a{q[0], q[1], q[2]}, bq{q[3], q[4], q[5]};
    const f3 d = bq - a;
    const float len = length(d);
    uint8_t res = 0;
    if (len > 0.0f) {
      const f3 dir{d.x / len, d.y / len, d.z / len};
      const float tnear = fmaxf(eps * len, eps);
      const float tfar = len * (1.0f - eps);
      if (tnear < tfar) {
        HitFilter f;
        f.faces = faces && offs ? faces + offs[i] : nullptr;
        f.nFaces = (faces && offs && meshPresent) ? int(offs[i + 1] - offs[i]) : 0;
        f.baseTri = s.baseTri;
        f.grazeCos = grazeCos;
        f.coplanar = coplanar;
        const Ray r{a, dir, tnear, tfar};
        Hit h;
        const TravScene ts = travOf(s);
        if (f.nFaces == 0 && grazeCos <= 0.0f && coplanar <= 0.0f)
          res = traverse<false, kMaskAll, true>(ts, r, h, ovf, nullptr, true) ? 1 : 0;
        else
          res = traverse<false, kMaskAll, false, true>(ts, r, h, ovf, nullptr, true, 0, nullptr, 0, &f) ? 1 : 0;
      }
    }
    out[i] = res;
  }
  warpCount(&stats[3], ovf);
}

// Kind bits of a scene, and the instantiated variant that covers a set of kinds.
int kindMaskBits(const Scene& sc) {
  int m = 0;
  for (int k = 0; k < 4; ++k)
    if (sc.primCount[k]) m |= 1 << k;
  return m;
}

int roundKindMask(int m) {
  switch (m) {
    case kMaskMesh:
    case kMaskSphere:
    case kMaskMesh | kMaskSphere:
    case kMaskSphere | kMaskCone:
      return m;
    default:
      return kMaskAll;
  }
}

#define UBR_LAUNCH3(KERNEL, KM, count, batch, grid, tb, stream, ...)                  \
  do {                                                                                \
    if (count) {                                                                      \
      if (batch) KERNEL<true, KM, true><<<grid, tb, 0, stream>>>(__VA_ARGS__);        \
      else KERNEL<true, KM, false><<<grid, tb, 0, stream>>>(__VA_ARGS__);             \
    } else {                                                                          \
      if (batch) KERNEL<false, KM, true><<<grid, tb, 0, stream>>>(__VA_ARGS__);       \
      else KERNEL<false, KM, false><<<grid, tb, 0, stream>>>(__VA_ARGS__);            \
    }                                                                                 \
  } while (0)

#define UBR_KM_DISPATCH(KERNEL, km, count, batch, grid, tb, stream, ...)                                     \
  do {                                                                                                       \
    switch (km) {                                                                                            \
      case kMaskMesh: UBR_LAUNCH3(KERNEL, kMaskMesh, count, batch, grid, tb, stream, __VA_ARGS__); break;  \
      case kMaskSphere: UBR_LAUNCH3(KERNEL, kMaskSphere, count, batch, grid, tb, stream, __VA_ARGS__); break; \
      case kMaskMesh | kMaskSphere:                                                                          \
        UBR_LAUNCH3(KERNEL, kMaskMesh | kMaskSphere, count, batch, grid, tb, stream, __VA_ARGS__);           \
        break;                                                                                               \
      case kMaskSphere | kMaskCone:                                                                          \
        UBR_LAUNCH3(KERNEL, kMaskSphere | kMaskCone, count, batch, grid, tb, stream, __VA_ARGS__);           \
        break;                                                                                               \
      default: UBR_LAUNCH3(KERNEL, kMaskAll, count, batch, grid, tb, stream, __VA_ARGS__);                   \
    }                                                                                                        \
  } while (0)

// kind-mask dispatch of a kernel templated on the mask alone
#define UBR_KM_DISPATCH1(KERNEL, km, grid, tb, stream, ...)                                   \
  do {                                                                                      \
    switch (km) {                                                                           \
      case kMaskMesh: KERNEL<kMaskMesh><<<grid, tb, 0, stream>>>(__VA_ARGS__); break;       \
      case kMaskSphere: KERNEL<kMaskSphere><<<grid, tb, 0, stream>>>(__VA_ARGS__); break;   \
      default: KERNEL<kMaskAll><<<grid, tb, 0, stream>>>(__VA_ARGS__);                      \
    }                                                                                       \
  } while (0)

void launchClosest(int km, bool count, bool batch, uint32_t grid, int tb, cudaStream_t st, const Params& p,
                   const DScene& s, const Batch& bt, const Bufs& b, int layer, uint32_t n, const uint32_t* queue) {
  UBR_KM_DISPATCH(k_trace_closest, km, count, batch, grid, tb, st, p, s, bt, b, layer, n, queue);
}

void launchOcclusion(int km, bool count, bool batch, uint32_t grid, int tb, cudaStream_t st, const Params& p,
                     const DScene& s, const Batch& bt, const Bufs& b, uint32_t n, bool il = false) {
  if (il) UBR_KM_DISPATCH(k_trace_occlusion_il, km, count, batch, grid, tb, st, p, s, bt, b, n);
  else UBR_KM_DISPATCH(k_trace_occlusion, km, count, batch, grid, tb, st, p, s, bt, b, n);
}

// Resident grid of the persistent occlusion kernel: SMs x resident blocks.
uint32_t persistentGrid(int device) {
  static int cached[64] = {};
  if (device >= 0 && device < 64 && cached[device]) return uint32_t(cached[device]);
  int sms = 0, perSm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_trace_occlusion_persistent<false, kMaskAll, false>, 128,
                                                0);
  const int g = std::max(1, sms) * std::max(1, perSm);
  if (device >= 0 && device < 64) cached[device] = g;
  return uint32_t(g);
}

uint32_t gridStrideGrid(int device) {
  static int cached[64] = {};
  if (device >= 0 && device < 64 && cached[device]) return uint32_t(cached[device]);
  int sms = 0, perSm = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSm, k_trace_occlusion_gs<false, kMaskAll, false>, 128, 0);
  const int g = std::max(1, sms) * std::max(1, perSm);
  if (device >= 0 && device < 64) cached[device] = g;
  return uint32_t(g);
}

void launchOcclusionGridStride(int km, bool count, bool batch, uint32_t grid, int tb, cudaStream_t st,
                               const Params& p, const DScene& s, const Batch& bt, const Bufs& b) {
  UBR_KM_DISPATCH(k_trace_occlusion_gs, km, count, batch, grid, tb, st, p, s, bt, b);
}

void launchOcclusionPersistent(int km, bool count, bool batch, uint32_t grid, int tb, cudaStream_t st,
                               const Params& p, const DScene& s, const Batch& bt, const Bufs& b) {
  UBR_KM_DISPATCH(k_trace_occlusion_persistent, km, count, batch, grid, tb, st, p, s, bt, b);
}

}  // namespace

// One frame of a (possibly single-frame) launch.
struct Job {
  const Scene* scene;
  const ubr_render_desc* desc;
  ubr_frame* frame;
};

// Run N frames through one set of launches over a global pixel / ray space
// (N = 1 is the per-frame path, BATCH = false, parameters in the constant
// bank).  When every frame is one layer deep (opaque scene or transparency
// off) and nothing is profiled, the device work is a fixed sequence: it is
// captured once into a CUDA graph and replayed (re-captured and updated in
// place when the parameters change).
ubr_status runFrames(Context* c, const std::vector<Job>& jobs, ubr_frame* total, const volatile int32_t* cancel,
                     uint64_t* progress) {
  const size_t nf = jobs.size();
  if (nf == 0) return UBR_OK;
  const bool batch = nf > 1;
  std::vector<FrameDesc> fds(nf);
  std::vector<LightD> lights;
  std::vector<uint32_t> pixOffs(nf), outOffs(nf);
  uint64_t npix64 = 0, nout64 = 0;
  uint32_t R = 0, aoStride = 0, aoMin = 0xFFFFFFFFu;
  int km = 0, maxIters = 1;
  bool secondary = false, enhanced = false, singleLayer = true, aov = false;
  for (size_t f = 0; f < nf; ++f) {
    std::vector<LightD> fl;
    Params& p = fds[f].p;
    ubr_status st = makeParams(c, *jobs[f].desc, p, fl);
    if (st != UBR_OK) return st;
    p.lightOff = int(lights.size());
    lights.insert(lights.end(), fl.begin(), fl.end());
    fds[f].s = jobs[f].scene->view;
    fds[f].pixOff = uint32_t(npix64);
    fds[f].outOff = uint32_t(nout64);
    pixOffs[f] = fds[f].pixOff;
    outOffs[f] = fds[f].outOff;
    npix64 += uint64_t(p.W) * uint64_t(p.H);
    nout64 += uint64_t(p.outW) * uint64_t(p.outH);
    R = std::max(R, uint32_t(p.raysPerHit));
    aoMin = std::min(aoMin, uint32_t(p.aoSamples));
    if ((p.aoEnhanced || p.aoWriteAov) && p.aoSamples > 0) {
      enhanced = true;
      aoStride = std::max(aoStride, uint32_t(p.aoSamples));
    }
    secondary = secondary || p.raysPerHit > 0;
    aov = aov || p.aoWriteAov;
    if (!(p.maxIters == 1 || jobs[f].scene->opaque)) singleLayer = false;
    maxIters = std::max(maxIters, jobs[f].scene->opaque ? 1 : p.maxIters);
    km |= kindMaskBits(*jobs[f].scene);
  }
  if (npix64 >= (1ull << 31) || nout64 >= (1ull << 31))
    return setError(c, UBR_INVALID_ARGUMENT, "render: more than 2^31 pixels in one launch");
  if (lights.size() > size_t(kMaxLights) * nf) return setError(c, UBR_INVALID_ARGUMENT, "too many lights");
  km = roundKindMask(km);
  const uint32_t npix = uint32_t(npix64), nout = uint32_t(nout64);
  const Params& p1 = fds[0].p;
  const DScene& s1 = fds[0].s;
  ubr_status st = UBR_OK;
  // adaptive AA (one frame per call): supersampled, or a fine lattice at ss 1
  const ubr_render_desc& d0 = *jobs[0].desc;
  const bool adaptive = !batch && p1.aaMode == 1 && (p1.ss > 1 || d0.aa_depth > 1);
  if (batch)
    for (size_t f = 0; f < nf; ++f)
      if (fds[f].p.aaMode == 1 && (fds[f].p.ss > 1 || jobs[f].desc->aa_depth > 1))
        return setError(c, UBR_INVALID_ARGUMENT, "render batch: adaptive AA renders one frame per call");
  // fine lattice of flagged cells: kFine^2 samples per hi-res cell
  const int kFine = adaptive ? std::max(1, (d0.aa_depth + p1.ss - 1) / p1.ss) : 1;
  const uint32_t k2 = uint32_t(kFine) * uint32_t(kFine);
  if (kFine > 1 && (uint64_t(p1.W) * kFine * uint64_t(p1.H) * kFine >= (1ull << 32) || k2 > (1u << 16)))
    return setError(c, UBR_INVALID_ARGUMENT, "render desc: aa_depth lattice too large");
  // per-slot buffers hold a full frame, or one chunk of fine samples
  const uint32_t nslot = std::max(npix, k2);
  Bufs b{};
  b.accum = scratchT<float4>(c, 16, npix, st);
  b.tnear = scratchT<float>(c, 17, npix, st);
  b.colorHi = scratchT<float4>(c, 18, npix, st);
  const bool giOn = p1.gi != 0;
  GiP gp{};
  b.rfl = ReflD{nullptr, nullptr, nullptr};
  if (giOn) {
    if (batch) return setError(c, UBR_INVALID_ARGUMENT, "render desc: gi renders one frame per call");
    b.giA = scratchT<float4>(c, 112, npix, st);
    b.giB = scratchT<float4>(c, 113, npix, st);
    b.giR = scratchT<float4>(c, 114, npix, st);
    // embree_renderer.cpp:581-612: gather sky (uniform, or gradient toward
    // ao_ground_color), up axis = the AO up axis, tfar = giMaxDistance or inf
    gp.spp = d0.pt1_spp;
    gp.bounces = d0.gi_bounces;
    gp.ld = d0.pt1_ld ? 1 : 0;
    gp.maxDist = d0.gi_max_distance > 0.0f ? d0.gi_max_distance : kInfF;
    gp.clampLum = d0.pt1_clamp;
    gp.seedMix = hashU32(d0.pt1_seed);
    gp.envI = d0.gi_env_intensity;
    gp.amb = p1.ambLight;
    gp.envUp = p1.aoUp;
    gp.sky = f3{d0.pt1_sky_radiance[0], d0.pt1_sky_radiance[1], d0.pt1_sky_radiance[2]};
    gp.ground = d0.pt1_sky_mode == 1 ? f3{d0.ao_ground_color[0], d0.ao_ground_color[1], d0.ao_ground_color[2]} : gp.sky;
    gp.stats = scratchT<unsigned long long>(c, 115, 4, st);
    if (p1.pt2Refl) {
      b.rfl.amt = scratchT<float4>(c, 141, npix, st);
      b.rfl.f0 = scratchT<float4>(c, 142, npix, st);
      if (p1.pt2Glossy && jobs[0].scene->anisoPrincipled) b.rfl.tan = scratchT<float4>(c, 143, npix, st);
    }
  }
  b.depth = scratchT<float>(c, 19, npix, st);
  b.viewZ = scratchT<float>(c, 20, npix, st);
  b.hitGeom = scratchT<uint32_t>(c, 21, npix, st);
  b.hitPrim = scratchT<uint32_t>(c, 22, npix, st);
  b.hitA = scratchT<float4>(c, 23, nslot, st);
  b.hitB = scratchT<float4>(c, 24, nslot, st);
  uint32_t* q0 = scratchT<uint32_t>(c, 25, nslot, st);
  uint32_t* q1 = scratchT<uint32_t>(c, 26, nslot, st);
  if (secondary) {
    b.surfA = scratchT<float4>(c, 27, nslot, st);
    b.surfB = scratchT<float4>(c, 28, nslot, st);
    b.surfT = scratchT<float4>(c, 146, nslot, st);
    b.surfC = scratchT<uint2>(c, 29, nslot, st);
    b.occQueue = scratchT<uint32_t>(c, 36, nslot, st);
    b.cursor = scratchT<unsigned long long>(c, 37, 1, st);
    b.occ = scratchT<uint8_t>(c, 30, size_t(nslot) * R, st);
    if (enhanced) b.aoT = scratchT<float>(c, 31, size_t(nslot) * aoStride, st);
  }
  LightD* dl = scratchT<LightD>(c, 32, lights.size() + 1, st);
  b.lights = dl;
  b.stats = scratchT<unsigned long long>(c, 33, 8, st);
  b.counter = scratchT<uint32_t>(c, 34, 4, st);
  float4* outColor = scratchT<float4>(c, 35, nout, st);
  float* outAov = nullptr;  // albedo 3, normal 3, bent 3, contact, shape, avg per output pixel
  if (aov) {
    b.aovA = scratchT<float4>(c, 70, npix, st);
    b.aovB = scratchT<float4>(c, 71, npix, st);
    b.aovC = scratchT<float4>(c, 72, npix, st);
    outAov = scratchT<float>(c, 73, size_t(nout) * 12, st);
  }
  // coarse-grid AO (one frame per call; pipeline.cpp:68 resolves -1 to ss;
  // embree_renderer.cpp:531 needs AO and a mesh or a non-outline primitive)
  if (batch)
    for (size_t f = 0; f < nf; ++f) {
      const int dv = jobs[f].desc->ao_res_div < 0 ? fds[f].p.ss : jobs[f].desc->ao_res_div;
      if (dv > 1 && fds[f].p.aoSamples > 0)
        return setError(c, UBR_INVALID_ARGUMENT, "render batch: coarse-grid AO renders one frame per call");
    }
  Params pCoarse{};
  bool coarseOn = false;
  uint32_t nCell = 0;
  float4 *cgN = nullptr, *cgQ = nullptr, *cgB = nullptr;
  uint8_t* cgHit = nullptr;
  if (!batch) {
    const int div = d0.ao_res_div < 0 ? p1.ss : d0.ao_res_div;
    if (div > 1 && p1.aoSamples > 0 && jobs[0].scene->aoReceivers) {
      coarseOn = true;
      Params& pm = fds[0].p;
      pm.aoCoarse = 1;
      pm.cgW = (p1.W + div - 1) / div;
      pm.cgH = (p1.H + div - 1) / div;
      nCell = uint32_t(pm.cgW) * uint32_t(pm.cgH);
      cgN = scratchT<float4>(c, 92, nCell, st);
      cgQ = scratchT<float4>(c, 93, nCell, st);
      cgHit = scratchT<uint8_t>(c, 94, nCell, st);
      if (p1.aoEnhanced || p1.aoWriteAov) cgB = scratchT<float4>(c, 95, nCell, st);
      if (jobs[0].frame->ao_patch_mask) b.aoPatch = scratchT<float>(c, 96, npix, st);
      b.cgN = cgN;
      b.cgQ = cgQ;
      b.cgB = cgB;
      b.cgHit = cgHit;
      // the coarse lattice: AO rays only, seeds on the grid
      pCoarse = p1;
      pCoarse.aoCoarse = 0;
      pCoarse.W = p1.cgW;
      pCoarse.H = p1.cgH;
      pCoarse.raysPerHit = p1.aoSamples;
      pCoarse.shadowRays = 0;
      pCoarse.shadowsActive = 0;
      pCoarse.nLights = 0;
    }
  }
  // edge G-buffer (one frame per call, grid frames)
  for (size_t f = 0; f < nf; ++f)
    if (jobs[f].desc->edge_gbuffer && (batch || adaptive))
      return setError(c, UBR_INVALID_ARGUMENT,
                      "render: the edge G-buffer needs a single grid frame (no batch, no adaptive AA)");
  const bool edgeGb = !batch && d0.edge_gbuffer != 0;
  const bool clipPlanes = !(p1.clipNear <= -kInfF && p1.clipFar >= kInfF);
  if (edgeGb) {
    b.gbObj = scratchT<uint32_t>(c, 98, npix, st);
    b.gbMat = scratchT<uint32_t>(c, 99, npix, st);
    b.gbNrm = scratchT<float>(c, 100, size_t(npix) * 3, st);
    b.gbAlpha = scratchT<float>(c, 101, npix, st);
    if (clipPlanes) {
      b.gbClip = scratchT<uint8_t>(c, 102, npix, st);
      b.gbNear = scratchT<float>(c, 103, npix, st);
      b.gbFar = scratchT<float>(c, 104, npix, st);
    }
  }
  // a-trous denoiser: one grid frame with the AO AOV guides
  const bool denoise = !batch && aov && d0.denoiser != 0 && d0.denoise_iters > 0;
  uint8_t* dnValid = nullptr;
  float *dnIrr[2] = {nullptr, nullptr}, *dnLum = nullptr, *dnVar = nullptr;
  if (denoise) {
    dnValid = scratchT<uint8_t>(c, 107, nout, st);
    dnIrr[0] = scratchT<float>(c, 108, size_t(nout) * 3, st);
    dnIrr[1] = scratchT<float>(c, 109, size_t(nout) * 3, st);
    dnLum = scratchT<float>(c, 110, nout, st);
    dnVar = scratchT<float>(c, 111, nout, st);
  }
  const uint32_t nCentre = uint32_t(p1.outW) * uint32_t(p1.outH);
  uint32_t *aaList0 = nullptr, *aaList1 = nullptr, *aaCounts = nullptr;
  uint8_t* aaRaw = nullptr;
  float* aaMaskOut = nullptr;
  Params pBoost{}, pFine{};
  uint8_t* reuseOccBuf = nullptr;
  float* reuseAoTBuf = nullptr;
  std::vector<LightD> lightsBoost;
  LightD* dlBoost = nullptr;
  bool needBoost = false;
  Bufs bFine{};
  uint32_t fineCap = 0;  // fine samples per chunk (a multiple of kFine^2)
  uint32_t* fineCoord = nullptr;
  if (adaptive) {
    const int ss = p1.ss;
    b.aaN = scratchT<float4>(c, 74, npix, st);
    aaList0 = scratchT<uint32_t>(c, 75, nCentre, st);
    aaList1 = scratchT<uint32_t>(c, 76, size_t(nCentre) * size_t(ss * ss), st);
    aaRaw = scratchT<uint8_t>(c, 77, nCentre, st);
    aaCounts = scratchT<uint32_t>(c, 78, 2, st);
    if (jobs[0].frame->aa_mask) aaMaskOut = scratchT<float>(c, 79, nCentre, st);
    // replication context (embree_renderer.cpp:1592-1608): ss^2 AO samples,
    // ss^2 soft-shadow samples when shadows are stochastic
    const bool soft = d0.shadow_samples > 1 && d0.light_radius_deg > 0.0f;
    needBoost = ss > 1 && ((d0.ao_samples > 0 && !coarseOn) || soft);
    if (needBoost) {
      ubr_render_desc db = d0;
      if (!coarseOn) db.ao_samples = d0.ao_samples * ss * ss;  // the grid is smooth already
      if (soft) db.shadow_samples = d0.shadow_samples * ss * ss;
      st = makeParams(c, db, pBoost, lightsBoost);
      if (st != UBR_OK) return st;
      pBoost.aoCoarse = p1.aoCoarse;
      pBoost.cgW = p1.cgW;
      pBoost.cgH = p1.cgH;
      // the boosted centre's first aoSamples AO rays are the centre pass's
      // own (the tea2 stream does not depend on the sample count; the
      // low-discrepancy set does): copy them instead of tracing, for single
      // layer frames and the per-ray occlusion kernel
      if (p1.aoSamples > 0 && !p1.aoLowDiscrepancy && !coarseOn && singleLayer &&
          (c->traceMode == 1 || c->traceMode == 4)) {
        pBoost.reuseAo = p1.aoSamples;
        reuseOccBuf = scratchT<uint8_t>(c, 105, size_t(nCentre) * R, st);
        if (p1.aoEnhanced || p1.aoWriteAov) reuseAoTBuf = scratchT<float>(c, 106, size_t(nCentre) * p1.aoSamples, st);
      }
      dlBoost = scratchT<LightD>(c, 80, lightsBoost.size() + 1, st);
    }
    if (kFine > 1) {
      // the (W k) x (H k) lattice: same camera, seeds on the finer grid
      pFine = p1;
      pFine.W = p1.W * kFine;
      pFine.H = p1.H * kFine;
      fineCap = (nslot / k2) * k2;
      bFine = b;
      bFine.lights = dl;
      bFine.aaN = nullptr;
      bFine.accum = scratchT<float4>(c, 81, fineCap, st);
      bFine.tnear = scratchT<float>(c, 82, fineCap, st);
      bFine.colorHi = scratchT<float4>(c, 83, fineCap, st);
      bFine.depth = scratchT<float>(c, 84, fineCap, st);
      bFine.viewZ = scratchT<float>(c, 85, fineCap, st);
      bFine.hitGeom = scratchT<uint32_t>(c, 86, fineCap, st);
      bFine.hitPrim = scratchT<uint32_t>(c, 87, fineCap, st);
      fineCoord = scratchT<uint32_t>(c, 88, fineCap, st);
      bFine.coord = fineCoord;
      bFine.aoPatch = b.aoPatch ? scratchT<float>(c, 97, fineCap, st) : nullptr;
      if (aov) {
        bFine.aovA = scratchT<float4>(c, 89, fineCap, st);
        bFine.aovB = scratchT<float4>(c, 90, fineCap, st);
        bFine.aovC = scratchT<float4>(c, 91, fineCap, st);
      }
    }
  }
  Batch bt{};
  if (batch) {
    FrameDesc* dfd = scratchT<FrameDesc>(c, 38, nf, st);
    uint32_t* doffs = scratchT<uint32_t>(c, 39, 2 * nf, st);
    if (st != UBR_OK) return st;
    UBR_CUDA(c, cudaMemcpyAsync(dfd, fds.data(), nf * sizeof(FrameDesc), cudaMemcpyHostToDevice, c->stream));
    UBR_CUDA(c, cudaMemcpyAsync(doffs, pixOffs.data(), nf * 4, cudaMemcpyHostToDevice, c->stream));
    UBR_CUDA(c, cudaMemcpyAsync(doffs + nf, outOffs.data(), nf * 4, cudaMemcpyHostToDevice, c->stream));
    bt.frames = dfd;
    bt.pixOffs = doffs;
    bt.outOffs = doffs + nf;
    bt.nFrames = int(nf);
    bt.R = R;
    bt.aoSplit = aoMin;
    bt.aoStride = aoStride;
    bt.nPix = uint32_t(npix64);
  }
  if (st != UBR_OK) return st;
  cudaStream_t s = c->stream;
  uint32_t kernels = 0;
  const uint32_t flags = total ? total->flags : 0u;
  const bool prof = (flags & UBR_FRAME_PROFILE) != 0;
  const bool count = (flags & UBR_FRAME_COUNT) != 0;
  // phase timing: pairs of events per launch, summed per phase after the sync
  std::vector<std::pair<int, int>> marks;  // (phase, event index of the start)
  auto mark = [&](int phase, bool start) {
    if (!prof) return;
    if (start) {
      const int e = int(marks.size()) * 2;
      if (size_t(e + 2) > c->pev.size()) {
        const size_t old = c->pev.size();
        c->pev.resize(old + 64);
        for (size_t i = old; i < c->pev.size(); ++i) cudaEventCreate(&c->pev[i]);
      }
      marks.push_back({phase, e});
      cudaEventRecord(c->pev[size_t(e)], s);
    } else {
      cudaEventRecord(c->pev[size_t(marks.back().second + 1)], s);
    }
  };
  const int TB = 128;
  // one transparency round of device work
  auto round = [&](const Params& pr, const Bufs& br, uint32_t Rr, int layer, uint32_t n, const uint32_t* queue,
                   uint32_t* outQ) -> ubr_status {
    UBR_CUDA(c, cudaMemsetAsync(br.counter, 0, 2 * sizeof(uint32_t), s));
    const uint32_t grid = (n + TB - 1) / TB;
    mark(0, true);
    launchClosest(km, count, batch, grid, TB, s, pr, s1, bt, br, layer, n, queue);
    mark(0, false);
    ++kernels;
    if (secondary) {
      mark(1, true);
      if (batch) k_surface<true><<<grid, TB, 0, s>>>(pr, s1, bt, br, layer, n, queue);
      else k_surface<false><<<grid, TB, 0, s>>>(pr, s1, bt, br, layer, n, queue);
      mark(1, false);
      const uint64_t nr = uint64_t(n) * uint64_t(Rr);
      mark(2, true);
      if (c->traceMode == 1 || c->traceMode == 4) {
        launchOcclusion(km, count, batch, uint32_t((nr + TB - 1) / TB), TB, s, pr, s1, bt, br, n,
                        c->traceMode == 4);
      } else if (c->traceMode == 3) {
        launchOcclusionGridStride(km, count, batch, gridStrideGrid(c->device), TB, s, pr, s1, bt, br);
      } else {
        UBR_CUDA(c, cudaMemsetAsync(br.cursor, 0, sizeof(unsigned long long), s));
        launchOcclusionPersistent(km, count, batch, persistentGrid(c->device), TB, s, pr, s1, bt, br);
      }
      mark(2, false);
      kernels += 2;
    }
    mark(3, true);
    if (batch) k_shade<true><<<grid, TB, 0, s>>>(pr, s1, bt, br, layer, n, queue, outQ);
    else k_shade<false><<<grid, TB, 0, s>>>(pr, s1, bt, br, layer, n, queue, outQ);
    mark(3, false);
    ++kernels;
    UBR_CUDA(c, cudaGetLastError());
    return UBR_OK;
  };
  // coarse-grid AO pre-pass: G-buffer + AO rays of the grid cells, then the
  // per-cell estimate (device-only, so graph capture keeps it)
  auto coarsePrepass = [&]() -> ubr_status {
    if (!coarseOn) return UBR_OK;
    UBR_CUDA(c, cudaMemsetAsync(b.counter, 0, 2 * sizeof(uint32_t), s));
    const uint32_t grid = (nCell + TB - 1) / TB;
    mark(1, true);
    UBR_KM_DISPATCH(k_cao_trace, km, false, false, grid, TB, s, pCoarse, s1, b, cgN, cgHit);
    mark(1, false);
    const uint64_t nr = uint64_t(nCell) * uint64_t(pCoarse.raysPerHit);
    mark(2, true);
    if (c->traceMode == 1 || c->traceMode == 4) {
      launchOcclusion(km, count, false, uint32_t((nr + TB - 1) / TB), TB, s, pCoarse, s1, bt, b, nCell,
                      c->traceMode == 4);
    } else if (c->traceMode == 3) {
      launchOcclusionGridStride(km, count, false, gridStrideGrid(c->device), TB, s, pCoarse, s1, bt, b);
    } else {
      UBR_CUDA(c, cudaMemsetAsync(b.cursor, 0, sizeof(unsigned long long), s));
      launchOcclusionPersistent(km, count, false, persistentGrid(c->device), TB, s, pCoarse, s1, bt, b);
    }
    mark(2, false);
    mark(3, true);
    k_cao_finish<<<(nCell + 255) / 256, 256, 0, s>>>(pCoarse, b, cgHit, cgQ, cgB);
    mark(3, false);
    kernels += 3;
    UBR_CUDA(c, cudaGetLastError());
    return UBR_OK;
  };
  auto gbInit = [&]() {
    if (!edgeGb) return;
    k_gb_init<<<(npix + 255) / 256, 256, 0, s>>>(npix, b);
    ++kernels;
  };
  auto gbClip = [&]() {
    if (!edgeGb || !clipPlanes) return;
    UBR_KM_DISPATCH1(k_gb_clip, km, (npix + 127) / 128, 128, s, p1, s1, b, npix);
    ++kernels;
  };
  auto post = [&]() -> ubr_status {
    mark(4, true);
    // with the denoiser the gamma waits until after it
    Params pp = p1;
    if (denoise) pp.gamma = 1.0f;
    if (batch) k_post<true><<<(nout + 255) / 256, 256, 0, s>>>(p1, bt, nout, b.colorHi, b.viewZ, outColor);
    else k_post<false><<<(nout + 255) / 256, 256, 0, s>>>(pp, bt, nout, b.colorHi, b.viewZ, outColor);
    if (aov) {
      float* o = outAov;
      const size_t n = nout;
      if (batch)
        k_post_aov<true><<<(nout + 255) / 256, 256, 0, s>>>(p1, bt, nout, b.aovA, b.aovB, b.aovC, o, o + 3 * n,
                                                             o + 6 * n, o + 9 * n, o + 10 * n, o + 11 * n);
      else
        k_post_aov<false><<<(nout + 255) / 256, 256, 0, s>>>(p1, bt, nout, b.aovA, b.aovB, b.aovC, o, o + 3 * n,
                                                              o + 6 * n, o + 9 * n, o + 10 * n, o + 11 * n);
      ++kernels;
    }
    if (denoise) {
      const int W = p1.outW, H = p1.outH;
      const uint32_t g = (nout + 255) / 256;
      const float* nrm = outAov + 3 * size_t(nout);
      const float* alb = d0.denoise_demodulate_albedo ? outAov : nullptr;
      k_dn_init<<<g, 256, 0, s>>>(nout, outColor, nrm, alb, dnValid, dnIrr[0]);
      k_dn_var<<<g, 256, 0, s>>>(W, H, dnValid, dnIrr[0], dnVar);
      kernels += 2;
      const int iters = std::max(0, d0.denoise_iters);
      const float sigmaL = std::max(1.0e-4f, d0.denoise_sigma_l);
      int cur = 0;
      for (int it = 0; it < iters; ++it) {
        k_dn_lum<<<g, 256, 0, s>>>(nout, dnIrr[cur], dnLum);
        k_dn_iter<<<g, 256, 0, s>>>(W, H, 1 << it, dnValid, nrm, dnIrr[cur], dnLum, dnVar, d0.denoise_sigma_n, sigmaL,
                                    dnIrr[cur ^ 1]);
        cur ^= 1;
        kernels += 2;
      }
      k_dn_write<<<g, 256, 0, s>>>(nout, dnValid, dnIrr[cur], alb, outColor);
      ++kernels;
      if (!(fabsf(p1.gamma - 1.0f) <= 1.0e-4f)) {
        k_gamma<<<g, 256, 0, s>>>(nout, outColor, p1.gamma);
        ++kernels;
      }
    }
    mark(4, false);
    ++kernels;
    UBR_CUDA(c, cudaGetLastError());
    return UBR_OK;
  };
  // a cancel raised before the call renders nothing (embree_renderer.cpp:
  // 1395-1398 bails before the first chunk of rows)
  if (cancel && *cancel) return setError(c, UBR_CANCELLED, "render cancelled");
  cudaEventRecord(c->ev[0], s);
  if (!lights.empty())
    UBR_CUDA(c, cudaMemcpyAsync(dl, lights.data(), lights.size() * sizeof(LightD), cudaMemcpyHostToDevice, s));
  if (dlBoost && !lightsBoost.empty())
    UBR_CUDA(c, cudaMemcpyAsync(dlBoost, lightsBoost.data(), lightsBoost.size() * sizeof(LightD),
                                cudaMemcpyHostToDevice, s));
  int layer = 0;
  bool cancelled = false;
  uint32_t* hostCount = static_cast<uint32_t*>(c->pinned);
  // all transparency rounds of one set of pixels: the first round over
  // `list` (all pixels when null), later rounds over the survivors
  auto runLayers = [&](const Params& pr, const Bufs& br, uint32_t Rr, const uint32_t* list,
                       uint32_t n) -> ubr_status {
    const uint32_t* queue = list;
    uint32_t* qs[2] = {q0, q1};
    int l = 0;
    for (; l < maxIters && n > 0; ++l) {
      uint32_t* outQ = qs[l & 1];
      const ubr_status rs = round(pr, br, Rr, l, n, queue, outQ);
      if (rs != UBR_OK) return rs;
      if (l + 1 >= maxIters) {
        ++l;
        break;
      }
      UBR_CUDA(c, cudaMemcpyAsync(hostCount, br.counter, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
      UBR_CUDA(c, cudaStreamSynchronize(s));
      n = *hostCount;
      queue = outQ;
      if (progress) *progress = uint64_t(l + 1);
      if (cancel && *cancel) {
        cancelled = true;
        ++l;
        break;
      }
    }
    layer = std::max(layer, l);
    return UBR_OK;
  };
  // adaptive AA passes: centres, mask, flagged subpixels, re-shaded centres,
  // replication (embree_renderer.cpp:1379-1670)
  auto runAdaptive = [&]() -> ubr_status {
    AaGrid g{};
    g.color = b.colorHi;
    g.viewZ = b.viewZ;
    g.geom = b.hitGeom;
    g.nrm = b.aaN;
    g.W = p1.W;
    g.ss = p1.ss;
    g.cSub = p1.ss / 2;
    g.Wf = p1.outW;
    g.Hf = p1.outH;
    g.thr = p1.aaThreshold;
    g.persp = d0.cam_orthographic ? 0 : 1;
    g.pixelWorldSize = d0.cam_orthographic ? d0.cam_height / float(g.Hf) : 2.0f * p1.persHalfH / float(g.Hf);
    const uint32_t gridC = (nCentre + 255) / 256;
    k_aa_centres<<<gridC, 256, 0, s>>>(g, aaList0);
    ++kernels;
    ubr_status rs = runLayers(p1, b, R, aaList0, nCentre);
    if (rs != UBR_OK || cancelled) return rs;
    if (reuseOccBuf) {  // the centre pass's AO results, slot = output pixel
      UBR_CUDA(c, cudaMemcpyAsync(reuseOccBuf, b.occ, size_t(nCentre) * R, cudaMemcpyDeviceToDevice, s));
      if (reuseAoTBuf)
        UBR_CUDA(c, cudaMemcpyAsync(reuseAoTBuf, b.aoT, size_t(nCentre) * p1.aoSamples * sizeof(float),
                                    cudaMemcpyDeviceToDevice, s));
    }
    k_aa_raw<<<gridC, 256, 0, s>>>(g, aaRaw);
    UBR_CUDA(c, cudaMemsetAsync(aaCounts, 0, 2 * sizeof(uint32_t), s));
    k_aa_lists<<<gridC, 256, 0, s>>>(g, aaRaw, aaList1, aaList0, aaCounts, aaMaskOut, kFine > 1);
    kernels += 2;
    uint32_t* hc = hostCount + 2;
    UBR_CUDA(c, cudaMemcpyAsync(hc, aaCounts, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    UBR_CUDA(c, cudaStreamSynchronize(s));
    const uint32_t nFlagged = hc[0], nCentres = hc[1];
    if (kFine == 1) {
      rs = runLayers(p1, b, R, aaList1, nFlagged);
      if (rs != UBR_OK || cancelled) return rs;
    } else {
      // flagged cells in chunks of fineCap / k^2 cells
      const uint32_t cellsPerChunk = fineCap / k2;
      for (uint32_t cell0 = 0; cell0 < nFlagged; cell0 += cellsPerChunk) {
        const uint32_t nc = std::min(cellsPerChunk, nFlagged - cell0), n = nc * k2;
        k_aa_fine_coords<<<(n + 255) / 256, 256, 0, s>>>(g, aaList1, cell0, n, kFine, fineCoord);
        k_init_pixels<<<(n + 255) / 256, 256, 0, s>>>(n, bFine.depth, bFine.viewZ, bFine.hitGeom, bFine.hitPrim,
                                                      bFine.aovA, bFine.aovB, bFine.aovC, nullptr, nullptr,
                                                      bFine.aoPatch);
        kernels += 2;
        rs = runLayers(pFine, bFine, R, nullptr, n);
        if (rs != UBR_OK || cancelled) return rs;
        k_aa_fine_reduce<<<(nc + 255) / 256, 256, 0, s>>>(aaList1, cell0, nc, kFine, bFine, b);
        ++kernels;
      }
    }
    if (needBoost && nCentres > 0) {
      k_init_pixels<<<(nCentres + 255) / 256, 256, 0, s>>>(nCentres, b.depth, b.viewZ, b.hitGeom, b.hitPrim,
                                                           b.aovA, b.aovB, b.aovC, b.aaN, aaList0, b.aoPatch);
      ++kernels;
      Bufs bb = b;
      bb.lights = dlBoost;
      bb.reuseOcc = reuseOccBuf;
      bb.reuseAoT = reuseAoTBuf;
      bb.reuseR = R;
      rs = runLayers(pBoost, bb, uint32_t(pBoost.raysPerHit), aaList0, nCentres);
      if (rs != UBR_OK || cancelled) return rs;
    }
    if (nCentres > 0) {
      k_aa_replicate<<<(nCentres + 255) / 256, 256, 0, s>>>(g, aaList0, aaCounts, b.colorHi, b.depth, b.viewZ,
                                                            b.hitGeom, b.hitPrim, b.aovA, b.aovB, b.aovC, b.aoPatch);
      ++kernels;
    }
    UBR_CUDA(c, cudaGetLastError());
    return UBR_OK;
  };
  // runPt1GiPass (embree_renderer.cpp:560-934): the gather on the render grid,
  // or on a grid reduced by k with its own primary rays, then the denoise of
  // E at gather resolution, the joint-bilateral upsample, the silhouette edge
  // patch and the [E] composite.
  int giDiv = 1;
  if (giOn) {
    giDiv = d0.pt1_gather_div;
    if (giDiv < 0) giDiv = p1.ss;  // "output resolution" (pipeline.cpp resolves -1 to the supersample factor)
    if (giDiv == 0) giDiv = d0.pt1_half_res ? 2 : 1;
    if (giDiv < 1) giDiv = 1;
  }
  auto giPass = [&]() -> ubr_status {
    ubr_status gs = UBR_OK;
    for (cudaEvent_t& e : c->giEv)
      if (!e) UBR_CUDA(c, cudaEventCreate(&e));
    gp.overflow = b.stats + 3;
    UBR_CUDA(c, cudaMemsetAsync(gp.stats, 0, 4 * sizeof(unsigned long long), s));
    const LightD* lt = b.lights + p1.lightOff;
    const int nL = p1.nLights;
    const int spp = d0.pt1_spp;
    const GiGrid full{p1.W, p1.H, b.giA, b.giB, nullptr};
    // pt2's gather configuration (embree_renderer.cpp:620-660): the sampler,
    // emission at vertices, emissive NEE when the scene emits; adaptive spp
    // (spp >= 2) adds spp * (mul - 1) samples where the estimate is noisy
    const bool pt2 = d0.gi_integrator == 2;
    gp.pt2 = pt2 ? 1 : 0;
    gp.pattern = d0.pt2_pattern;
    gp.emissive = (pt2 && d0.pt2_emissive) ? 1 : 0;
    gp.em = (pt2 && d0.pt2_emissive && d0.pt2_emissive_nee) ? jobs[0].scene->emit : EmitD{};
    gp.sampleOffset = 0;
    gp.halfE = nullptr;
    gp.rsv = nullptr;
    // ReSTIR rounds exclude adaptive spp (embree_renderer.cpp:626-636)
    const bool restir = pt2 && d0.pt2_rounds > 0;
    const bool adapt = pt2 && d0.pt2_adaptive && !restir && spp >= 2;
    const int extra = adapt ? spp * (std::max(2, d0.pt2_adaptive_mul) - 1) : 0;
    auto pow2 = [](uint32_t v) {
      uint32_t q = 1;
      while (q < v) q <<= 1;
      return q;
    };
    gp.sppPow2 = pow2(uint32_t(spp + extra));
    float4* Ef = scratchT<float4>(c, 116, npix, gs);
    if (gs != UBR_OK) return gs;
    // denoisePt1E on a w x h grid
    auto denoiseE = [&](int w, int h, float4* E, const float4* ne, const float4* pd) -> ubr_status {
      const uint32_t n = uint32_t(w) * uint32_t(h);
      ubr_status ds = UBR_OK;
      uint8_t* valid = scratchT<uint8_t>(c, 121, n, ds);
      float4* irrA = scratchT<float4>(c, 122, n, ds);
      float4* irrB = scratchT<float4>(c, 123, n, ds);
      float* var = scratchT<float>(c, 124, n, ds);
      float* pgrad = scratchT<float>(c, 125, n, ds);
      if (ds != UBR_OK) return ds;
      giDenoiseInit(s, n, E, ne, valid, irrA);
      ++kernels;
      const int iters = std::max(0, d0.denoise_iters);
      if (iters > 0) {
        giDenoiseAux(s, w, h, valid, irrA, pd, var, pgrad);
        float4* cur = irrA;
        float4* nxt = irrB;
        for (int it = 0; it < iters; ++it) {
          giDenoiseIter(s, w, h, 1 << it, valid, ne, pd, cur, var, pgrad, d0.denoise_sigma_n,
                        std::max(1.0e-4f, d0.denoise_sigma_z), std::max(1.0e-4f, d0.denoise_sigma_l), nxt);
          std::swap(cur, nxt);
        }
        giDenoiseWrite(s, n, valid, cur, E);
        kernels += 2u + uint32_t(iters);
      }
      UBR_CUDA(c, cudaGetLastError());
      return UBR_OK;
    };
    // the gather over a grid, with pt2's adaptive refinement (pt2_adaptive.hpp:
    // mask of noisy points, dilated twice, re-gathered continuing their
    // sequences, merged as a weighted mean)
    auto gatherGrid = [&](const GiGrid& gr, float4* E) -> ubr_status {
      const uint32_t n = uint32_t(gr.W) * uint32_t(gr.H);
      ubr_status as = UBR_OK;
      float* halfE = adapt ? scratchT<float>(c, 129, size_t(n) * 3, as) : nullptr;
      if (as != UBR_OK) return as;
      GiP g0 = gp;
      g0.halfE = halfE;
      float4* rsvA = restir ? scratchT<float4>(c, 144, size_t(n) * kRsvF4, as) : nullptr;
      float4* rsvB = restir ? scratchT<float4>(c, 145, size_t(n) * kRsvF4, as) : nullptr;
      if (as != UBR_OK) return as;
      g0.rsv = rsvA;
      giGather(km, s, g0, s1, lt, nL, gr, nullptr, nullptr, n, spp, E);
      ++kernels;
      if (restir) {
        // spatial rounds over the reservoirs, ping-pong; the last one writes E
        // (pt2_spatial.hpp:278-296)
        const GiSpatial sp{d0.pt2_rounds, d0.pt2_radius, d0.pt2_m_cap, d0.pt2_w_clamp, d0.pt2_unbiased ? 1 : 0,
                           gp.seedMix};
        float4* cur = rsvA;
        float4* nxt = rsvB;
        for (int r = 0; r < d0.pt2_rounds; ++r) {
          giSpatialRound(km, s, sp, s1, gr, cur, nxt, r, r == d0.pt2_rounds - 1 ? E : nullptr, gp.overflow);
          std::swap(cur, nxt);
          ++kernels;
        }
      }
      if (adapt) {
        uint8_t* m0 = scratchT<uint8_t>(c, 130, n, as);
        uint8_t* m1 = scratchT<uint8_t>(c, 131, n, as);
        uint32_t* list = scratchT<uint32_t>(c, 132, n, as);
        uint32_t* cnt = scratchT<uint32_t>(c, 133, 4, as);
        float4* Er = scratchT<float4>(c, 134, n, as);
        if (as != UBR_OK) return as;
        UBR_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(uint32_t), s));
        giAdaptiveMask(s, gr.W, gr.H, E, halfE, gr.ne, spp, d0.pt2_adaptive_thresh, m0);
        giDilate(s, gr.W, gr.H, m0, gr.ne, m1);
        giDilate(s, gr.W, gr.H, m1, gr.ne, m0);
        giMaskList(s, n, m0, list, cnt);
        GiP g1 = gp;
        g1.sampleOffset = spp;
        giGather(km, s, g1, s1, lt, nL, gr, list, cnt, n, extra, Er);
        giMerge(s, list, cnt, n, spp, extra, Er, E);
        kernels += 6;
      }
      UBR_CUDA(c, cudaGetLastError());
      return UBR_OK;
    };
    cudaEventRecord(c->giEv[0], s);
    if (giDiv > 1) {
      const int hw = (p1.W + giDiv - 1) / giDiv, hh = (p1.H + giDiv - 1) / giDiv;
      const uint32_t nlo = uint32_t(hw) * uint32_t(hh);
      float4* lpd = scratchT<float4>(c, 117, nlo, gs);
      float4* lne = scratchT<float4>(c, 118, nlo, gs);
      float4* lng = scratchT<float4>(c, 119, nlo, gs);
      float4* Elo = scratchT<float4>(c, 120, nlo, gs);
      uint32_t* patchList = scratchT<uint32_t>(c, 126, npix, gs);
      uint32_t* patchCount = scratchT<uint32_t>(c, 127, 4, gs);
      uint8_t* patchFlag = scratchT<uint8_t>(c, 147, npix, gs);
      const size_t listBytes = giPatchListBytes(npix);
      void* listTemp = scratchT<uint8_t>(c, 148, listBytes, gs);
      float4* Esnap = d0.pt1_edge_patch ? scratchT<float4>(c, 128, npix, gs) : nullptr;
      if (gs != UBR_OK) return gs;
      UBR_CUDA(c, cudaMemsetAsync(patchCount, 0, 2 * sizeof(uint32_t), s));
      giGBuffer(km, s, p1, s1, hw, hh, lpd, lne, lng, gp.stats, b.stats + 3);
      ++kernels;
      const GiGrid lo{hw, hh, lpd, lne, lng};
      cudaEventRecord(c->giEv[1], s);
      gs = gatherGrid(lo, Elo);
      if (gs != UBR_OK) return gs;
      cudaEventRecord(c->giEv[2], s);
      if (d0.pt1_denoise) {
        gs = denoiseE(hw, hh, Elo, lne, lpd);
        if (gs != UBR_OK) return gs;
      }
      cudaEventRecord(c->giEv[3], s);
      UBR_CUDA(c, giUpsample(s, p1.W, p1.H, b.giA, b.giB, lo, Elo, d0.pt1_upsample_normal_pow,
                             d0.pt1_upsample_depth_scale, giDiv <= 2 ? 0 : giDiv, d0.pt1_edge_patch ? 1 : 0,
                             d0.pt1_edge_patch_thresh, Ef, patchFlag, listTemp, listBytes, patchList, patchCount,
                             gp.stats + 3));
      ++kernels;
      cudaEventRecord(c->giEv[4], s);
      if (d0.pt1_edge_patch) {
        // re-gather the rim pixels at full resolution with spp x the patch
        // multiplier (their own sample layout), then blend them into the
        // field (radius 2)
        const int pspp = spp * std::max(1, d0.pt1_edge_patch_spp_mul);
        GiP gpat = gp;
        gpat.sppPow2 = pow2(uint32_t(pspp));
        giGather(km, s, gpat, s1, lt, nL, full, patchList, patchCount, npix, pspp, Ef);
        UBR_CUDA(c, cudaMemcpyAsync(Esnap, Ef, size_t(npix) * sizeof(float4), cudaMemcpyDeviceToDevice, s));
        giSmooth(s, p1.W, p1.H, patchList, patchCount, npix, b.giA, b.giB, d0.pt1_upsample_normal_pow,
                 d0.pt1_upsample_depth_scale, 2, Esnap, Ef);
        kernels += 2;
        UBR_CUDA(c, cudaMemcpyAsync(static_cast<char*>(c->pinned) + 256, patchCount, sizeof(uint32_t),
                                    cudaMemcpyDeviceToHost, s));
      }
      cudaEventRecord(c->giEv[5], s);
    } else {
      cudaEventRecord(c->giEv[1], s);
      gs = gatherGrid(full, Ef);
      if (gs != UBR_OK) return gs;
      cudaEventRecord(c->giEv[2], s);
      if (d0.pt1_denoise) {
        gs = denoiseE(p1.W, p1.H, Ef, b.giB, b.giA);
        if (gs != UBR_OK) return gs;
      }
      cudaEventRecord(c->giEv[3], s);
      cudaEventRecord(c->giEv[4], s);
      cudaEventRecord(c->giEv[5], s);
    }
    giComposite(s, npix, b.giB, b.giR, Ef, d0.gi_intensity, b.colorHi);
    ++kernels;
    // pt2 traced reflection (embree_renderer.cpp:935-1086): the mirror pass,
    // then the glossy GGX gather with its denoise, after the diffuse composite
    if (p1.pt2Refl && jobs[0].scene->reflective) {
      GiP gr = gp;
      gr.sppPow2 = 1;
      const GiCam cam{p1.camPos, p1.camDir, p1.ortho};
      giReflect(km, s, gr, s1, lt, nL, full, b.rfl, cam, npix, b.colorHi);
      ++kernels;
      if (p1.pt2Glossy && jobs[0].scene->glossy) {
        const int gspp = std::max(1, d0.pt2_glossy_spp);
        float4* Es = scratchT<float4>(c, 135, npix, gs);
        if (gs != UBR_OK) return gs;
        giGlossy(km, s, gr, s1, lt, nL, full, b.rfl, cam, npix, gspp, d0.pt1_seed, Es);
        ++kernels;
        if (d0.pt1_denoise && d0.pt2_glossy_denoise) {
          const int ssg = p1.ss;
          if (ssg <= 1 || p1.W % ssg != 0 || p1.H % ssg != 0) {
            gs = denoiseE(p1.W, p1.H, Es, b.giB, b.giA);  // render grid = output grid
            if (gs != UBR_OK) return gs;
          } else {
            // denoise at the output grid, then back up over the glossy pixels
            const int Wo = p1.W / ssg, Ho = p1.H / ssg;
            const uint32_t no = uint32_t(Wo) * uint32_t(Ho);
            float4* Eo = scratchT<float4>(c, 136, no, gs);
            float4* pdo = scratchT<float4>(c, 137, no, gs);
            float4* neo = scratchT<float4>(c, 138, no, gs);
            float4* gne = scratchT<float4>(c, 139, npix, gs);
            if (gs != UBR_OK) return gs;
            giGlossyDown(s, p1.W, p1.H, ssg, b.rfl, Es, b.giA, b.giB, Eo, pdo, neo);
            gs = denoiseE(Wo, Ho, Eo, neo, pdo);
            if (gs != UBR_OK) return gs;
            giGlossyElig(s, npix, b.rfl, b.giB, gne);
            const GiGrid go{Wo, Ho, pdo, neo, nullptr};
            UBR_CUDA(c, giUpsample(s, p1.W, p1.H, b.giA, gne, go, Eo, d0.pt1_upsample_normal_pow,
                                   d0.pt1_upsample_depth_scale, 0, 0, 0.0f, Es, nullptr, nullptr, 0, nullptr,
                                   nullptr, gp.stats + 3));
            kernels += 3;
          }
        }
        giGlossyComposite(s, npix, b.rfl, Es, b.colorHi);
        ++kernels;
      }
    }
    cudaEventRecord(c->giEv[6], s);
    UBR_CUDA(c, cudaGetLastError());
    return UBR_OK;
  };
  const bool useGraph = singleLayer && !prof && !count && c->useGraphs && !adaptive && !giOn;
  if (useGraph) {
    // key: everything the captured launches depend on
    std::vector<unsigned char> key(sizeof(Params) + sizeof(DScene) + sizeof(Batch) + sizeof(Bufs) + 64);
    size_t o = 0;
    auto put = [&](const void* src, size_t n) {
      std::memcpy(key.data() + o, src, n);
      o += n;
    };
    put(&p1, sizeof(Params));
    put(&s1, sizeof(DScene));
    put(&bt, sizeof(Batch));
    put(&b, sizeof(Bufs));
    const uint64_t misc[6] = {npix, nout, uint64_t(km), uint64_t(c->traceMode), uint64_t(outColor), R};
    put(misc, sizeof(misc));
    key.resize(o);
    if (!c->graphExec || key != c->graphKey) {
      UBR_CUDA(c, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      cudaMemsetAsync(b.stats, 0, 8 * sizeof(unsigned long long), s);
      k_init_pixels<<<(npix + 255) / 256, 256, 0, s>>>(npix, b.depth, b.viewZ, b.hitGeom, b.hitPrim, b.aovA,
                                                       b.aovB, b.aovC, nullptr, nullptr, b.aoPatch);
      gbInit();
      ubr_status rs = coarsePrepass();
      if (rs == UBR_OK) rs = round(p1, b, R, 0, npix, nullptr, q0);
      if (rs == UBR_OK) gbClip();
      if (rs == UBR_OK) rs = post();
      cudaGraph_t graph = nullptr;
      const cudaError_t ce = cudaStreamEndCapture(s, &graph);
      if (rs != UBR_OK) {
        if (graph) cudaGraphDestroy(graph);
        return rs;
      }
      if (ce != cudaSuccess) return cudaFail(c, ce, "cudaStreamEndCapture");
      bool updated = false;
      if (c->graphExec) {
        cudaGraphExecUpdateResultInfo info;
        updated = cudaGraphExecUpdate(c->graphExec, graph, &info) == cudaSuccess;
        if (!updated) {
          cudaGetLastError();
          cudaGraphExecDestroy(c->graphExec);
          c->graphExec = nullptr;
        }
      }
      if (!updated) {
        const cudaError_t ie = cudaGraphInstantiate(&c->graphExec, graph, 0);
        if (ie != cudaSuccess) {
          cudaGraphDestroy(graph);
          return cudaFail(c, ie, "cudaGraphInstantiate");
        }
      }
      cudaGraphDestroy(graph);
      c->graphKey = key;
    } else {
      kernels = (secondary ? 4u : 2u) + 1u + (aov ? 1u : 0u) + (coarseOn ? 3u : 0u) +
                (edgeGb ? (clipPlanes ? 2u : 1u) : 0u) +
                (denoise ? 3u + 2u * uint32_t(std::max(0, d0.denoise_iters)) +
                               (fabsf(p1.gamma - 1.0f) <= 1.0e-4f ? 0u : 1u)
                         : 0u);
    }
    cudaEventRecord(c->ev[2], s);
    UBR_CUDA(c, cudaGraphLaunch(c->graphExec, s));
    cudaEventRecord(c->ev[3], s);
    layer = 1;
    ++kernels;  // k_init_pixels
  } else {
    UBR_CUDA(c, cudaMemsetAsync(b.stats, 0, 8 * sizeof(unsigned long long), s));
    k_init_pixels<<<(npix + 255) / 256, 256, 0, s>>>(npix, b.depth, b.viewZ, b.hitGeom, b.hitPrim, b.aovA,
                                                       b.aovB, b.aovC, b.aaN, nullptr, b.aoPatch);
    ++kernels;
    gbInit();
    cudaEventRecord(c->ev[2], s);
    st = coarsePrepass();
    if (st != UBR_OK) return st;
    if (giOn) UBR_CUDA(c, cudaMemsetAsync(b.giB, 0, size_t(npix) * sizeof(float4), s));
    if (b.rfl.amt) UBR_CUDA(c, cudaMemsetAsync(b.rfl.amt, 0, size_t(npix) * sizeof(float4), s));
    st = adaptive ? runAdaptive() : runLayers(p1, b, R, nullptr, npix);
    if (st != UBR_OK) return st;
    if (giOn && !cancelled) {
      // the GI pass and [E] composite, before fog (embree_renderer.cpp:1708-1712)
      st = giPass();
      if (st != UBR_OK) return st;
    }
    if (!cancelled) gbClip();
    cudaEventRecord(c->ev[3], s);
    st = post();
    if (st != UBR_OK) return st;
  }
  // outputs
  for (size_t f = 0; f < nf; ++f) {
    ubr_frame& fr = *jobs[f].frame;
    const Params& p = fds[f].p;
    const size_t fpix = size_t(p.W) * p.H, fout = size_t(p.outW) * p.outH;
    const cudaMemcpyKind kind = fr.memory == UBR_MEMORY_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t po = fds[f].pixOff, oo = fds[f].outOff;
    if (fr.color) UBR_CUDA(c, cudaMemcpyAsync(fr.color, outColor + oo, fout * 16, kind, s));
    if (fr.depth) UBR_CUDA(c, cudaMemcpyAsync(fr.depth, b.depth + po, fpix * 4, kind, s));
    if (fr.view_z) UBR_CUDA(c, cudaMemcpyAsync(fr.view_z, b.viewZ + po, fpix * 4, kind, s));
    if (fr.hit_geom) UBR_CUDA(c, cudaMemcpyAsync(fr.hit_geom, b.hitGeom + po, fpix * 4, kind, s));
    if (fr.hit_prim) UBR_CUDA(c, cudaMemcpyAsync(fr.hit_prim, b.hitPrim + po, fpix * 4, kind, s));
    if (fr.aa_mask && aaMaskOut) UBR_CUDA(c, cudaMemcpyAsync(fr.aa_mask, aaMaskOut, fout * 4, kind, s));
    if (fr.ao_patch_mask && b.aoPatch)
      UBR_CUDA(c, cudaMemcpyAsync(fr.ao_patch_mask, b.aoPatch + po, fpix * 4, kind, s));
    if (edgeGb) {
      if (fr.gb_object_id) UBR_CUDA(c, cudaMemcpyAsync(fr.gb_object_id, b.gbObj, fpix * 4, kind, s));
      if (fr.gb_material_id) UBR_CUDA(c, cudaMemcpyAsync(fr.gb_material_id, b.gbMat, fpix * 4, kind, s));
      if (fr.gb_normal) UBR_CUDA(c, cudaMemcpyAsync(fr.gb_normal, b.gbNrm, fpix * 12, kind, s));
      if (fr.gb_surf_alpha) UBR_CUDA(c, cudaMemcpyAsync(fr.gb_surf_alpha, b.gbAlpha, fpix * 4, kind, s));
      if (b.gbClip) {
        if (fr.gb_clip_cut) UBR_CUDA(c, cudaMemcpyAsync(fr.gb_clip_cut, b.gbClip, fpix, kind, s));
        if (fr.gb_clip_near_vz) UBR_CUDA(c, cudaMemcpyAsync(fr.gb_clip_near_vz, b.gbNear, fpix * 4, kind, s));
        if (fr.gb_clip_far_vz) UBR_CUDA(c, cudaMemcpyAsync(fr.gb_clip_far_vz, b.gbFar, fpix * 4, kind, s));
      } else {
        // no clip planes: nothing is cut and nothing recorded
        if (fr.gb_clip_cut) {
          if (fr.memory == UBR_MEMORY_DEVICE) UBR_CUDA(c, cudaMemsetAsync(fr.gb_clip_cut, 0, fpix, s));
          else std::memset(fr.gb_clip_cut, 0, fpix);
        }
        float* zs[2] = {fr.gb_clip_near_vz, fr.gb_clip_far_vz};
        for (float* z : zs) {
          if (!z) continue;
          if (fr.memory == UBR_MEMORY_DEVICE) UBR_CUDA(c, cudaMemsetAsync(z, 0, fpix * 4, s));
          else std::memset(z, 0, fpix * 4);
        }
      }
    }
    if (p.aoWriteAov) {
      const float* o = outAov;
      const size_t n = nout;
      float* dst[6] = {fr.albedo, fr.normal, fr.bent_normal, fr.contact_ao, fr.shape_ao, fr.avg_hit_dist};
      const size_t base[6] = {0, 3 * n, 6 * n, 9 * n, 10 * n, 11 * n};
      const size_t width[6] = {3, 3, 3, 1, 1, 1};
      for (int k = 0; k < 6; ++k)
        if (dst[k])
          UBR_CUDA(c, cudaMemcpyAsync(dst[k], o + base[k] + width[k] * oo, width[k] * fout * 4, kind, s));
    }
  }
  unsigned long long* hs = reinterpret_cast<unsigned long long*>(static_cast<char*>(c->pinned) + 64);
  UBR_CUDA(c, cudaMemcpyAsync(hs, b.stats, 8 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  if (giOn && !cancelled)
    UBR_CUDA(c, cudaMemcpyAsync(hs + 8, gp.stats, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  cudaEventRecord(c->ev[1], s);
  UBR_CUDA(c, cudaStreamSynchronize(s));
  float msTotal = 0.0f, msLoop = 0.0f;
  cudaEventElapsedTime(&msTotal, c->ev[0], c->ev[1]);
  cudaEventElapsedTime(&msLoop, c->ev[2], c->ev[3]);
  if (total) {
    ubr_frame& fr = *total;
    fr.total_ms = msTotal;
    fr.render_ms = msLoop;
    fr.rays_primary = hs[0];
    fr.rays_occlusion = hs[1];
    fr.capped_rays = hs[2];
    fr.stack_overflows = hs[3];
    fr.layers = uint32_t(layer);
    fr.kernels = kernels;
    for (int k = 0; k < 5; ++k) fr.phase_ms[k] = 0.0;
    for (const auto& m : marks) {
      float ms = 0.0f;
      cudaEventElapsedTime(&ms, c->pev[size_t(m.second)], c->pev[size_t(m.second + 1)]);
      fr.phase_ms[m.first] += ms;
    }
    fr.nodes_visited[0] = hs[4];
    fr.nodes_visited[1] = hs[6];
    fr.node_bytes[0] = hs[4] * uint64_t(kWideF4 * 16);
    fr.node_bytes[1] = hs[6] * uint64_t(kWideF4 * 16);
    fr.prim_bytes[0] = hs[5];
    fr.prim_bytes[1] = hs[7];
    for (int k = 0; k < 6; ++k) fr.gi_ms[k] = 0.0;
    fr.gi_gather_rays = fr.gi_nee_rays = fr.gi_gbuffer_rays = fr.gi_patched_pixels = 0;
    if (giOn && !cancelled) {
      for (int k = 0; k < 6; ++k) {
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, c->giEv[k], c->giEv[k + 1]);
        fr.gi_ms[k] = ms;
      }
      const unsigned long long* gs = hs + 8;
      fr.gi_gather_rays = gs[0];
      fr.gi_nee_rays = gs[1];
      fr.gi_gbuffer_rays = gs[2];
      if (giDiv > 1 && d0.pt1_edge_patch)
        fr.gi_patched_pixels = *reinterpret_cast<const uint32_t*>(static_cast<const char*>(c->pinned) + 256);
    }
  }
  if (cancelled) return setError(c, UBR_CANCELLED, "render cancelled");
  if (hs[3] > 0) return setError(c, UBR_TRAVERSAL_LIMIT, "traversal stack overflow");
  return UBR_OK;
}

ubr_status renderFrame(Context* c, const Scene* sc, const ubr_render_desc& d, ubr_frame& fr,
                       const volatile int32_t* cancel, uint64_t* progress) {
  std::vector<Job> jobs{Job{sc, &d, &fr}};
  return runFrames(c, jobs, &fr, cancel, progress);
}

// Frames whose passes depend on per-frame host decisions (adaptive AA, the
// coarse AO grid, the edge G-buffer) each run as their own launch sequence
// after the batched rest; `total` then sums the statistics.
static bool needsOwnPass(const ubr_render_desc& d) {
  const int ss = d.supersample < 1 ? 1 : d.supersample;
  if (d.aa_mode == 1 && (ss > 1 || d.aa_depth > 1)) return true;
  if (d.edge_gbuffer) return true;
  if (d.denoiser != 0 && d.ao_write_aov) return true;
  return (d.ao_res_div < 0 ? ss : d.ao_res_div) > 1 && d.ao_samples > 0;
}

ubr_status renderBatch(Context* c, const std::vector<Job>& jobs, ubr_frame* total) {
  std::vector<Job> together, alone;
  for (const Job& j : jobs) (needsOwnPass(*j.desc) ? alone : together).push_back(j);
  // frames that share a scene are made contiguous in the launch (stable
  // order otherwise): their rays then walk one BVH at a time, which keeps
  // it resident in L2; every frame still writes its own buffers
  std::stable_sort(together.begin(), together.end(),
                   [](const Job& a, const Job& b) { return a.scene < b.scene; });
  if (alone.empty()) return runFrames(c, together, total, nullptr, nullptr);
  const uint32_t flags = total ? total->flags : 0u;
  ubr_frame sum{};
  auto add = [&](const ubr_frame& t) {
    sum.total_ms += t.total_ms;
    sum.render_ms += t.render_ms;
    sum.rays_primary += t.rays_primary;
    sum.rays_occlusion += t.rays_occlusion;
    sum.capped_rays += t.capped_rays;
    sum.stack_overflows += t.stack_overflows;
    sum.layers = std::max(sum.layers, t.layers);
    sum.kernels += t.kernels;
    for (int k = 0; k < 5; ++k) sum.phase_ms[k] += t.phase_ms[k];
    for (int k = 0; k < 2; ++k) {
      sum.node_bytes[k] += t.node_bytes[k];
      sum.prim_bytes[k] += t.prim_bytes[k];
      sum.nodes_visited[k] += t.nodes_visited[k];
    }
  };
  if (!together.empty()) {
    ubr_frame t{};
    t.flags = flags;
    const ubr_status st = runFrames(c, together, &t, nullptr, nullptr);
    if (st != UBR_OK) return st;
    add(t);
  }
  for (const Job& j : alone) {
    ubr_frame t{};
    t.flags = flags;
    const ubr_status st = runFrames(c, std::vector<Job>{j}, &t, nullptr, nullptr);
    if (st != UBR_OK) return st;
    add(t);
  }
  if (total) {
    // statistics only: the frames' own buffers were written per item
    total->total_ms = sum.total_ms;
    total->render_ms = sum.render_ms;
    total->rays_primary = sum.rays_primary;
    total->rays_occlusion = sum.rays_occlusion;
    total->capped_rays = sum.capped_rays;
    total->stack_overflows = sum.stack_overflows;
    total->layers = sum.layers;
    total->kernels = sum.kernels;
    for (int k = 0; k < 5; ++k) total->phase_ms[k] = sum.phase_ms[k];
    for (int k = 0; k < 2; ++k) {
      total->node_bytes[k] = sum.node_bytes[k];
      total->prim_bytes[k] = sum.prim_bytes[k];
      total->nodes_visited[k] = sum.nodes_visited[k];
    }
  }
  return UBR_OK;
}

// End of a segment query: wait for its answers and report a traversal that
// ran out of stack or steps (its answer may have missed an occluder) as
// UBR_TRAVERSAL_LIMIT; the answers are written either way.
ubr_status finishQuery(Context* c, const unsigned long long* stats) {
  unsigned long long ovf = 0;
  UBR_CUDA(c, cudaMemcpyAsync(&ovf, stats + 3, sizeof(ovf), cudaMemcpyDeviceToHost, c->stream));
  UBR_CUDA(c, cudaStreamSynchronize(c->stream));
  if (ovf) return setError(c, UBR_TRAVERSAL_LIMIT, "traversal stack overflow");
  return UBR_OK;
}

ubr_status occludedBatch(Context* c, const Scene* sc, const float* segs, uint64_t n, float eps, uint8_t* out,
                         int32_t memory) {
  if (n == 0) return UBR_OK;
  if (!segs || !out) return setError(c, UBR_INVALID_ARGUMENT, "occluded_batch: NULL buffer");
  ubr_status st = UBR_OK;
  const float* dsegs = segs;
  uint8_t* dout = out;
  cudaStream_t s = c->stream;
  if (memory != UBR_MEMORY_DEVICE) {
    float* ts = scratchT<float>(c, 40, size_t(n) * 6, st);
    dout = scratchT<uint8_t>(c, 41, size_t(n), st);
    if (st != UBR_OK) return st;
    UBR_CUDA(c, cudaMemcpyAsync(ts, segs, size_t(n) * 6 * sizeof(float), cudaMemcpyHostToDevice, s));
    dsegs = ts;
  }
  unsigned long long* stats = scratchT<unsigned long long>(c, 42, 8, st);
  if (st != UBR_OK) return st;
  UBR_CUDA(c, cudaMemsetAsync(stats, 0, 8 * sizeof(unsigned long long), s));
  k_occluded_segments<<<uint32_t((n + 127) / 128), 128, 0, s>>>(sc->view, dsegs, n, eps, dout, stats);
  UBR_CUDA(c, cudaGetLastError());
  if (memory != UBR_MEMORY_DEVICE) UBR_CUDA(c, cudaMemcpyAsync(out, dout, size_t(n), cudaMemcpyDeviceToHost, s));
  return finishQuery(c, stats);
}

ubr_status occludedFilteredBatch(Context* c, const Scene* sc, const float* segs, uint64_t n, float eps,
                                 float grazeCos, float coplanar, const uint32_t* offs, const int32_t* faces,
                                 uint8_t* out, int32_t memory) {
  if (n == 0) return UBR_OK;
  if (!segs || !out) return setError(c, UBR_INVALID_ARGUMENT, "occluded_filtered_batch: NULL buffer");
  if ((offs == nullptr) != (faces == nullptr))
    return setError(c, UBR_INVALID_ARGUMENT, "occluded_filtered_batch: exclude offsets and faces go together");
  ubr_status st = UBR_OK;
  const float* dsegs = segs;
  const uint32_t* doffs = offs;
  const int32_t* dfaces = faces;
  uint8_t* dout = out;
  cudaStream_t s = c->stream;
  if (memory != UBR_MEMORY_DEVICE) {
    uint64_t nf = 0;
    if (offs) {
      if (offs[0] != 0) return setError(c, UBR_INVALID_ARGUMENT, "occluded_filtered_batch: offsets[0] != 0");
      for (uint64_t i = 0; i < n; ++i)
        if (offs[i + 1] < offs[i])
          return setError(c, UBR_INVALID_ARGUMENT, "occluded_filtered_batch: offsets decrease");
      nf = offs[n];
    }
    float* ts = scratchT<float>(c, 40, size_t(n) * 6, st);
    dout = scratchT<uint8_t>(c, 41, size_t(n), st);
    uint32_t* to = offs ? scratchT<uint32_t>(c, 43, size_t(n) + 1, st) : nullptr;
    int32_t* tf = offs ? scratchT<int32_t>(c, 44, size_t(nf) + 1, st) : nullptr;
    if (st != UBR_OK) return st;
    UBR_CUDA(c, cudaMemcpyAsync(ts, segs, size_t(n) * 6 * sizeof(float), cudaMemcpyHostToDevice, s));
    if (offs) {
      UBR_CUDA(c, cudaMemcpyAsync(to, offs, (size_t(n) + 1) * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
      if (nf) UBR_CUDA(c, cudaMemcpyAsync(tf, faces, size_t(nf) * sizeof(int32_t), cudaMemcpyHostToDevice, s));
    }
    dsegs = ts;
    doffs = to;
    dfaces = tf;
  }
  unsigned long long* stats = scratchT<unsigned long long>(c, 42, 8, st);
  if (st != UBR_OK) return st;
  UBR_CUDA(c, cudaMemsetAsync(stats, 0, 8 * sizeof(unsigned long long), s));
  k_occluded_filtered<<<uint32_t((n + 127) / 128), 128, 0, s>>>(sc->view, dsegs, n, eps, grazeCos, coplanar, doffs,
                                                                dfaces, sc->primCount[kMesh] > 0 ? 1 : 0, dout,
                                                                stats);
  UBR_CUDA(c, cudaGetLastError());
  if (memory != UBR_MEMORY_DEVICE) UBR_CUDA(c, cudaMemcpyAsync(out, dout, size_t(n), cudaMemcpyDeviceToHost, s));
  return finishQuery(c, stats);
}

}  // namespace ubr

// ---------------------------------------------------------------------------
// Segment occlusion without allocation (ubr_occluded_batch_noalloc).
//
// Some callers of this library cannot allocate device memory at the time they
// need an answer: a host that runs the query from inside its own per-frame
// loop under a strict GPU memory budget, a plugin sandbox whose host owns all
// device allocations, or code that must not risk an allocation failure or the
// implicit synchronisation cudaMalloc/cudaFree can cause mid-frame.  For them
// the segments and the results are staged through one file-scope device array
// of fixed size instead of the context's growable scratch.  Every GPU that
// loads the library holds this array until the process exits.

constexpr uint64_t kNoAllocMaxSegments = 1ull << 19;  // 524,288 segments per call
constexpr size_t kNoAllocHeader = 256;                // counters (8 x u64), padded
constexpr size_t kNoAllocBytes = kNoAllocHeader + kNoAllocMaxSegments * 6 * sizeof(float) + kNoAllocMaxSegments;

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocBytes];

namespace ubr {

namespace {

// Device address of g_noallocScratch, resolved by the first allocation-free
// call made on a context (its device is current on the calling thread then:
// every entry point makes it so) and kept in the context.  A context never
// outlives its device's primary context, so the address stays valid for it.
ubr_status noallocScratch(Context* c, unsigned char** out) {
  if (!c->noallocArray) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
    if (e != cudaSuccess) return cudaFail(c, e, "cudaGetSymbolAddress(g_noallocScratch)");
    c->noallocArray = p;
  }
  *out = static_cast<unsigned char*>(c->noallocArray);
  return UBR_OK;
}

}  // namespace

ubr_status occludedBatchNoAlloc(Context* c, const Scene* sc, const float* segs, uint64_t n, float eps,
                                uint8_t* out) {
  if (n == 0) return UBR_OK;
  if (!segs || !out) return setError(c, UBR_INVALID_ARGUMENT, "occluded_batch_noalloc: NULL buffer");
  if (n > kNoAllocMaxSegments)
    return setError(c, UBR_INVALID_ARGUMENT,
                    "occluded_batch_noalloc: more than 524288 segments in one call (the fixed scratch limit)");
  unsigned char* base = nullptr;
  ubr_status st = noallocScratch(c, &base);
  if (st != UBR_OK) return st;
  unsigned long long* stats = reinterpret_cast<unsigned long long*>(base);
  float* dsegs = reinterpret_cast<float*>(base + kNoAllocHeader);
  uint8_t* dout = reinterpret_cast<uint8_t*>(base + kNoAllocHeader + kNoAllocMaxSegments * 6 * sizeof(float));
  cudaStream_t s = c->stream;
  // the array keeps the previous call's contents: the counters start at zero
  UBR_CUDA(c, cudaMemsetAsync(stats, 0, 8 * sizeof(unsigned long long), s));
  UBR_CUDA(c, cudaMemcpyAsync(dsegs, segs, size_t(n) * 6 * sizeof(float), cudaMemcpyHostToDevice, s));
  k_occluded_segments<<<uint32_t((n + 127) / 128), 128, 0, s>>>(sc->view, dsegs, n, eps, dout, stats);
  UBR_CUDA(c, cudaGetLastError());
  UBR_CUDA(c, cudaMemcpyAsync(out, dout, size_t(n), cudaMemcpyDeviceToHost, s));
  return finishQuery(c, stats);
}

}  // namespace ubr

// rtcore_shim.cpp -- TEST INFRASTRUCTURE: the Embree 4 API subset declared in
// shim/embree4/rtcore.h, implemented on the oracle's CPU substrate
// (oracle_geom.hpp), so the reference's own render path runs here as a
// parity check.  A scene holds at most one geometry per kind (triangles,
// point spheres, round linear curves, cone linear curves), which is how the
// reference builds its scenes (render/scene_build.cpp, render/curve_build.cpp,
// edges/edge_mesh_bvh.cpp); geomIDs are the attach order.
#include <embree4/rtcore.h>

#include <cstring>
#include <limits>
#include <memory>
#include <stdexcept>
#include <vector>

#include "oracle_geom.hpp"

struct RTCDeviceTy {
  RTCError err = RTC_ERROR_NONE;
};

struct RTCGeometryTy {
  int refs = 1;
  RTCGeometryType type;
  std::vector<unsigned char> buf[4][2];  // [buffer type][slot]
  size_t count[4][2] = {};
  size_t stride[4][2] = {};
  bool filterFromArgs = false;
};

struct RTCSceneTy {
  RTCDeviceTy* dev = nullptr;
  std::vector<RTCGeometryTy*> geoms;  // by geomID
  oracle::GeomSet set;
  oracle::Bvh bvh;
  int kindOf[8] = {-1, -1, -1, -1, -1, -1, -1, -1};  // geomID -> oracle kind
  bool committed = false;
  ~RTCSceneTy() {
    for (RTCGeometryTy* g : geoms)
      if (--g->refs == 0) delete g;
  }
};

RTCDevice rtcNewDevice(const char*) { return new RTCDeviceTy(); }
void rtcReleaseDevice(RTCDevice d) { delete d; }
RTCError rtcGetDeviceError(RTCDevice d) {
  if (!d) return RTC_ERROR_NONE;
  const RTCError e = d->err;
  d->err = RTC_ERROR_NONE;
  return e;
}
void rtcSetDeviceErrorFunction(RTCDevice, RTCErrorFunction, void*) {}

RTCScene rtcNewScene(RTCDevice d) {
  RTCScene s = new RTCSceneTy();
  s->dev = d;
  return s;
}
void rtcReleaseScene(RTCScene s) { delete s; }
void rtcSetSceneFlags(RTCScene, RTCSceneFlags) {}
void rtcSetSceneBuildQuality(RTCScene, RTCBuildQuality) {}

RTCGeometry rtcNewGeometry(RTCDevice, RTCGeometryType type) {
  RTCGeometry g = new RTCGeometryTy();
  g->type = type;
  return g;
}
void rtcReleaseGeometry(RTCGeometry g) {
  if (g && --g->refs == 0) delete g;
}
void rtcCommitGeometry(RTCGeometry) {}
void* rtcSetNewGeometryBuffer(RTCGeometry g, RTCBufferType type, unsigned int slot, RTCFormat, size_t byteStride,
                              size_t itemCount) {
  if (int(type) > 3 || slot > 1) throw std::runtime_error("rtcore shim: unsupported buffer");
  g->buf[type][slot].assign(byteStride * itemCount + 16, 0);
  g->count[type][slot] = itemCount;
  g->stride[type][slot] = byteStride;
  return g->buf[type][slot].data();
}
void rtcSetGeometryVertexAttributeCount(RTCGeometry, unsigned int) {}
void rtcSetGeometryEnableFilterFunctionFromArguments(RTCGeometry g, bool enable) { g->filterFromArgs = enable; }

unsigned int rtcAttachGeometry(RTCScene s, RTCGeometry g) {
  ++g->refs;
  s->geoms.push_back(g);
  return unsigned(s->geoms.size() - 1);
}

void rtcCommitScene(RTCScene s) {
  oracle::GeomSet& gs = s->set;
  gs = oracle::GeomSet();
  for (size_t id = 0; id < s->geoms.size(); ++id) {
    RTCGeometryTy* g = s->geoms[id];
    const int kind = g->type == RTC_GEOMETRY_TYPE_TRIANGLE ? oracle::kMesh
                     : g->type == RTC_GEOMETRY_TYPE_SPHERE_POINT ? oracle::kSphere
                     : g->type == RTC_GEOMETRY_TYPE_ROUND_LINEAR_CURVE ? oracle::kRound
                                                                      : oracle::kCone;
    if (gs.geomID[kind] != oracle::kInvalid) {
      if (s->dev) s->dev->err = RTC_ERROR_INVALID_OPERATION;
      throw std::runtime_error("rtcore shim: one geometry per kind");
    }
    gs.geomID[kind] = unsigned(id);
    if (id < 8) s->kindOf[id] = kind;
    const auto& vb = g->buf[RTC_BUFFER_TYPE_VERTEX][0];
    const size_t nv = g->count[RTC_BUFFER_TYPE_VERTEX][0];
    const auto* vf = reinterpret_cast<const float*>(vb.data());
    const auto* ib = reinterpret_cast<const uint32_t*>(g->buf[RTC_BUFFER_TYPE_INDEX][0].data());
    const size_t ni = g->count[RTC_BUFFER_TYPE_INDEX][0];
    switch (kind) {
      case oracle::kMesh:
        gs.triPos.assign(vf, vf + 3 * nv);
        gs.triIdx.assign(ib, ib + 3 * ni);
        break;
      case oracle::kSphere:
        gs.sph.assign(vf, vf + 4 * nv);
        break;
      case oracle::kRound: {
        gs.rcV.assign(vf, vf + 4 * nv);
        gs.rcIdx.assign(ib, ib + ni);
        const auto& fb = g->buf[RTC_BUFFER_TYPE_FLAGS][0];
        gs.rcFlags.assign(fb.begin(), fb.begin() + ni);
        break;
      }
      default:
        gs.ccV.assign(vf, vf + 4 * nv);
        gs.ccIdx.assign(ib, ib + ni);
    }
  }
  s->bvh.build(&gs);
  s->committed = true;
}

void rtcInitRayQueryContext(RTCRayQueryContext* c) { c->instID[0] = RTC_INVALID_GEOMETRY_ID; }
void rtcInitIntersectArguments(RTCIntersectArguments* a) {
  a->flags = RTC_RAY_QUERY_FLAG_INCOHERENT;
  a->context = nullptr;
  a->filter = nullptr;
}
void rtcInitOccludedArguments(RTCOccludedArguments* a) {
  a->flags = RTC_RAY_QUERY_FLAG_INCOHERENT;
  a->context = nullptr;
  a->filter = nullptr;
}

namespace {
oracle::Ray toRay(const RTCRay& r) {
  oracle::Ray o;
  o.org = oracle::V3(r.org_x, r.org_y, r.org_z);
  o.dir = oracle::V3(r.dir_x, r.dir_y, r.dir_z);
  o.tnear = r.tnear;
  o.tfar = r.tfar;
  return o;
}
}  // namespace

void rtcIntersect1(RTCScene s, RTCRayHit* rh, RTCIntersectArguments*) {
  if (!s || !s->committed || !(rh->ray.tnear <= rh->ray.tfar)) return;
  oracle::Hit h;
  if (!s->bvh.closest(toRay(rh->ray), h)) return;
  rh->ray.tfar = h.t;
  rh->hit.geomID = h.geomID;
  rh->hit.primID = h.primID;
  rh->hit.u = h.u;
  rh->hit.v = h.v;
  rh->hit.Ng_x = h.Ng.x;
  rh->hit.Ng_y = h.Ng.y;
  rh->hit.Ng_z = h.Ng.z;
  rh->hit.instID[0] = RTC_INVALID_GEOMETRY_ID;
}

void rtcOccluded1(RTCScene s, RTCRay* ray, RTCOccludedArguments* args) {
  if (!s || !s->committed || !(ray->tnear <= ray->tfar)) return;
  const oracle::Ray r = toRay(*ray);
  bool hit;
  if (args && args->filter && (args->flags & RTC_RAY_QUERY_FLAG_INVOKE_ARGUMENT_FILTER)) {
    // the argument filter sees each candidate (geometries that enabled it)
    hit = s->bvh.occludedIf(r, [&](int kind, uint32_t prim, const oracle::Hit& h) {
      const uint32_t gid = s->set.geomID[kind];
      if (!s->geoms[gid]->filterFromArgs) return true;
      RTCRay rr = *ray;
      rr.tfar = h.t;
      RTCHit hh;
      hh.Ng_x = h.Ng.x;
      hh.Ng_y = h.Ng.y;
      hh.Ng_z = h.Ng.z;
      hh.u = h.u;
      hh.v = h.v;
      hh.primID = prim;
      hh.geomID = gid;
      hh.instID[0] = RTC_INVALID_GEOMETRY_ID;
      int valid = -1;
      RTCFilterFunctionNArguments fa;
      fa.valid = &valid;
      fa.geometryUserPtr = nullptr;
      fa.context = args->context;
      fa.ray = reinterpret_cast<RTCRayN*>(&rr);
      fa.hit = reinterpret_cast<RTCHitN*>(&hh);
      fa.N = 1;
      args->filter(&fa);
      return valid != 0;
    });
  } else {
    hit = s->bvh.occluded(r);
  }
  if (hit) ray->tfar = -std::numeric_limits<float>::infinity();
}

void rtcInterpolate0(RTCGeometry g, unsigned int primID, float u, float v, RTCBufferType bufferType,
                     unsigned int slot, float* P, unsigned int valueCount) {
  const auto* ib = reinterpret_cast<const uint32_t*>(g->buf[RTC_BUFFER_TYPE_INDEX][0].data());
  const auto& ab = g->buf[bufferType][slot];
  const size_t stride = g->stride[bufferType][slot] / sizeof(float);
  const auto* a = reinterpret_cast<const float*>(ab.data());
  const uint32_t i0 = ib[3 * primID], i1 = ib[3 * primID + 1], i2 = ib[3 * primID + 2];
  const float w0 = 1.0f - u - v;
  for (unsigned int k = 0; k < valueCount; ++k)
    P[k] = w0 * a[stride * i0 + k] + u * a[stride * i1 + k] + v * a[stride * i2 + k];
}

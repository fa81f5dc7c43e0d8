// A stand-in for the subset of the Embree 4 ray-tracing API that CueMol/
// umbreon's renderer calls, declared from those call sites so the
// reference's own sources compile unmodified against it.  TEST
// INFRASTRUCTURE ONLY: it exists to run the reference's render path on the
// CPU as a parity check.  Its BVH and intersectors are the oracle's own
// (oracle_geom.hpp: a binned-SAH BVH, the watertight triangle test, spheres,
// round and capped-cone linear curves); nothing here comes from Embree.
#pragma once

#include <cstddef>
#include <cstdint>

#define RTC_INVALID_GEOMETRY_ID (~0u)
#define RTC_MAX_INSTANCE_LEVEL_COUNT 1

typedef struct RTCDeviceTy* RTCDevice;
typedef struct RTCSceneTy* RTCScene;
typedef struct RTCGeometryTy* RTCGeometry;

enum RTCError {
  RTC_ERROR_NONE = 0,
  RTC_ERROR_UNKNOWN = 1,
  RTC_ERROR_INVALID_ARGUMENT = 2,
  RTC_ERROR_INVALID_OPERATION = 3,
  RTC_ERROR_OUT_OF_MEMORY = 4,
  RTC_ERROR_UNSUPPORTED_CPU = 5,
  RTC_ERROR_CANCELLED = 6
};

enum RTCGeometryType {
  RTC_GEOMETRY_TYPE_TRIANGLE = 0,
  RTC_GEOMETRY_TYPE_SPHERE_POINT = 1,
  RTC_GEOMETRY_TYPE_ROUND_LINEAR_CURVE = 2,
  RTC_GEOMETRY_TYPE_CONE_LINEAR_CURVE = 3
};

enum RTCBufferType {
  RTC_BUFFER_TYPE_INDEX = 0,
  RTC_BUFFER_TYPE_VERTEX = 1,
  RTC_BUFFER_TYPE_VERTEX_ATTRIBUTE = 2,
  RTC_BUFFER_TYPE_FLAGS = 3
};

enum RTCFormat {
  RTC_FORMAT_UNDEFINED = 0,
  RTC_FORMAT_UCHAR = 1,
  RTC_FORMAT_UINT = 2,
  RTC_FORMAT_UINT3 = 3,
  RTC_FORMAT_FLOAT3 = 4,
  RTC_FORMAT_FLOAT4 = 5
};
#define RTC_INVALID RTC_FORMAT_UNDEFINED

enum RTCSceneFlags { RTC_SCENE_FLAG_NONE = 0, RTC_SCENE_FLAG_ROBUST = 4 };
enum RTCBuildQuality { RTC_BUILD_QUALITY_LOW = 0, RTC_BUILD_QUALITY_MEDIUM = 1, RTC_BUILD_QUALITY_HIGH = 2 };
enum RTCRayQueryFlags {
  RTC_RAY_QUERY_FLAG_NONE = 0,
  RTC_RAY_QUERY_FLAG_INVOKE_ARGUMENT_FILTER = 2,
  RTC_RAY_QUERY_FLAG_INCOHERENT = 0,
  RTC_RAY_QUERY_FLAG_COHERENT = 1
};
inline RTCRayQueryFlags operator|(RTCRayQueryFlags a, RTCRayQueryFlags b) {
  return RTCRayQueryFlags(int(a) | int(b));
}
enum RTCCurveFlags { RTC_CURVE_FLAG_NEIGHBOR_LEFT = 1, RTC_CURVE_FLAG_NEIGHBOR_RIGHT = 2 };

struct RTCRay {
  float org_x, org_y, org_z;
  float tnear;
  float dir_x, dir_y, dir_z;
  float time;
  float tfar;
  unsigned int mask, id, flags;
};

struct RTCHit {
  float Ng_x, Ng_y, Ng_z;
  float u, v;
  unsigned int primID, geomID;
  unsigned int instID[RTC_MAX_INSTANCE_LEVEL_COUNT];
};

struct RTCRayHit {
  RTCRay ray;
  RTCHit hit;
};

struct RTCRayQueryContext {
  unsigned int instID[RTC_MAX_INSTANCE_LEVEL_COUNT];
};

// a single ray / hit seen through the N-wide accessors (N = 1 here)
struct RTCRayN;
struct RTCHitN;

struct RTCFilterFunctionNArguments {
  int* valid;
  void* geometryUserPtr;
  RTCRayQueryContext* context;
  RTCRayN* ray;
  RTCHitN* hit;
  unsigned int N;
};
typedef void (*RTCFilterFunctionN)(const RTCFilterFunctionNArguments* args);

struct RTCIntersectArguments {
  RTCRayQueryFlags flags;
  RTCRayQueryContext* context;
  RTCFilterFunctionN filter;
};
struct RTCOccludedArguments {
  RTCRayQueryFlags flags;
  RTCRayQueryContext* context;
  RTCFilterFunctionN filter;
};

inline unsigned int RTCHitN_geomID(RTCHitN* h, unsigned int, unsigned int) {
  return reinterpret_cast<RTCHit*>(h)->geomID;
}
inline unsigned int RTCHitN_primID(RTCHitN* h, unsigned int, unsigned int) {
  return reinterpret_cast<RTCHit*>(h)->primID;
}
inline float RTCHitN_Ng_x(RTCHitN* h, unsigned int, unsigned int) { return reinterpret_cast<RTCHit*>(h)->Ng_x; }
inline float RTCHitN_Ng_y(RTCHitN* h, unsigned int, unsigned int) { return reinterpret_cast<RTCHit*>(h)->Ng_y; }
inline float RTCHitN_Ng_z(RTCHitN* h, unsigned int, unsigned int) { return reinterpret_cast<RTCHit*>(h)->Ng_z; }
inline float RTCHitN_u(RTCHitN* h, unsigned int, unsigned int) { return reinterpret_cast<RTCHit*>(h)->u; }
inline float RTCHitN_v(RTCHitN* h, unsigned int, unsigned int) { return reinterpret_cast<RTCHit*>(h)->v; }
inline float RTCRayN_dir_x(RTCRayN* r, unsigned int, unsigned int) { return reinterpret_cast<RTCRay*>(r)->dir_x; }
inline float RTCRayN_dir_y(RTCRayN* r, unsigned int, unsigned int) { return reinterpret_cast<RTCRay*>(r)->dir_y; }
inline float RTCRayN_dir_z(RTCRayN* r, unsigned int, unsigned int) { return reinterpret_cast<RTCRay*>(r)->dir_z; }
inline float RTCRayN_org_x(RTCRayN* r, unsigned int, unsigned int) { return reinterpret_cast<RTCRay*>(r)->org_x; }
inline float RTCRayN_org_y(RTCRayN* r, unsigned int, unsigned int) { return reinterpret_cast<RTCRay*>(r)->org_y; }
inline float RTCRayN_org_z(RTCRayN* r, unsigned int, unsigned int) { return reinterpret_cast<RTCRay*>(r)->org_z; }
inline float RTCRayN_tfar(RTCRayN* r, unsigned int, unsigned int) { return reinterpret_cast<RTCRay*>(r)->tfar; }
inline float RTCRayN_tnear(RTCRayN* r, unsigned int, unsigned int) { return reinterpret_cast<RTCRay*>(r)->tnear; }

typedef void (*RTCErrorFunction)(void* userPtr, RTCError code, const char* str);

RTCDevice rtcNewDevice(const char* config);
void rtcReleaseDevice(RTCDevice device);
RTCError rtcGetDeviceError(RTCDevice device);
void rtcSetDeviceErrorFunction(RTCDevice device, RTCErrorFunction fn, void* userPtr);

RTCScene rtcNewScene(RTCDevice device);
void rtcReleaseScene(RTCScene scene);
void rtcSetSceneFlags(RTCScene scene, RTCSceneFlags flags);
void rtcSetSceneBuildQuality(RTCScene scene, RTCBuildQuality quality);
unsigned int rtcAttachGeometry(RTCScene scene, RTCGeometry geometry);
void rtcCommitScene(RTCScene scene);

RTCGeometry rtcNewGeometry(RTCDevice device, RTCGeometryType type);
void rtcReleaseGeometry(RTCGeometry geometry);
void rtcCommitGeometry(RTCGeometry geometry);
void* rtcSetNewGeometryBuffer(RTCGeometry geometry, RTCBufferType type, unsigned int slot, RTCFormat format,
                              size_t byteStride, size_t itemCount);
void rtcSetGeometryVertexAttributeCount(RTCGeometry geometry, unsigned int count);
void rtcSetGeometryEnableFilterFunctionFromArguments(RTCGeometry geometry, bool enable);

void rtcInitRayQueryContext(RTCRayQueryContext* context);
void rtcInitIntersectArguments(RTCIntersectArguments* args);
void rtcInitOccludedArguments(RTCOccludedArguments* args);
void rtcIntersect1(RTCScene scene, RTCRayHit* rayhit, RTCIntersectArguments* args = nullptr);
void rtcOccluded1(RTCScene scene, RTCRay* ray, RTCOccludedArguments* args = nullptr);

// barycentric interpolation of a triangle's vertex attribute slot at (u, v):
// (1 - u - v) a0 + u a1 + v a2, valueCount floats
void rtcInterpolate0(RTCGeometry geometry, unsigned int primID, float u, float v, RTCBufferType bufferType,
                     unsigned int bufferSlot, float* P, unsigned int valueCount);

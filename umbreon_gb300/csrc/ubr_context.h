// ubr_context.h -- context, device buffers and scene object of libubr.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "gi.cuh"
#include "ubr_internal.h"

namespace ubr {

// A device allocation owned by the context or a scene.  Grows on demand;
// contents are not preserved across growth.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

struct Context {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool ownStream = false;
  uint64_t arenaCap = 0;     // 0 = unlimited
  int leafMax = 1;           // wide-BVH leaf size (1..kWideLeafMax); 1 measured fastest
  int builder = 1;           // binary tree before the 8-wide collapse: 1 Karras radix tree, 2 PLOC
  int collapse = 1;          // 8-wide collapse: 1 greedy (fixed leaf size), 2 SAH-optimal (leaves 1..3)
  float sahPrimScale = 1.0f; // SAH collapse: weight of primitive tests against node visits
  int traceMode = 1;         // occlusion kernel: 1 one thread per ray (measured faster), 2 persistent
  uint64_t arenaUsed = 0;
  std::string lastError;
  // frame scratch, reused across frames
  std::vector<DevBuf> scratch;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<cudaEvent_t> pev;  // profiling events, created on first use
  void* pinned = nullptr;    // small pinned host block for counters
  bool useGraphs = true;     // replay single-layer frames from a CUDA graph
  cudaGraphExec_t graphExec = nullptr;
  std::vector<unsigned char> graphKey;  // launch parameters the graph was captured with
  std::vector<void*> sceneHandles;      // live ubr_scene handles built on this context
  cudaMemPool_t pool = nullptr;         // stream-ordered device allocations (scenes, scratch)
  void* noallocArray = nullptr;         // device address of the allocation-free query's fixed array
  cudaEvent_t giEv[7] = {};             // GI pass stage boundaries, created on first use
};

struct Scene {
  Context* ctx = nullptr;
  DScene view;
  std::vector<DevBuf> bufs;  // owned allocations
  uint64_t primCount[4] = {0, 0, 0, 0};
  uint64_t nodes = 0;
  bool opaque = true;        // every primitive fully opaque: frames are one layer deep
  bool aoReceivers = false;  // a mesh or a non-outline primitive exists (coarse AO grid eligible)
  bool principled = false;   // some material uses the principled model
  // pt2 GI: a first hit can own a traced reflection (POV reflection > 0, or a
  // principled specular lobe); some can be glossy (a highlight-bearing POV
  // finish, or principled roughness^2 >= 0.015); an anisotropic principled
  // sphere / cylinder exists; the emissive primitives sampled as lights
  bool reflective = false, glossy = false, anisoPrincipled = false;
  EmitD emit;
  uint64_t deviceBytes = 0;
  double buildMs = 0.0;
  double flattenMs = 0.0;    // host: validation, primID ordering, chaining, material table
  double uploadMs = 0.0;     // host: allocations and copies queued
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
};

// error helpers
ubr_status setError(Context* c, ubr_status s, const std::string& msg);
ubr_status cudaFail(Context* c, cudaError_t e, const char* what);
// allocate `bytes` on the context's device, honouring the arena cap
ubr_status devAlloc(Context* c, DevBuf& b, size_t bytes);
void devFree(Context* c, DevBuf& b);
// scratch slot `i` of at least `bytes`
ubr_status scratchGet(Context* c, int i, size_t bytes, void** out);

// typed view of scratch slot `slot` (count elements); a no-op once st != OK
template <class T>
T* scratchT(Context* c, int slot, size_t count, ubr_status& st) {
  void* ptr = nullptr;
  if (st == UBR_OK) st = scratchGet(c, slot, count * sizeof(T) + 16, &ptr);
  return static_cast<T*>(ptr);
}

// Frame parameters and light table of a render description (camera basis,
// lights, AO / fog / gamma settings), validated.
ubr_status makeParams(Context* c, const ubr_render_desc& d, Params& p, std::vector<LightD>& lights);

#define UBR_CUDA(ctx, call)                                  \
  do {                                                       \
    cudaError_t e_ = (call);                                 \
    if (e_ != cudaSuccess) return cudaFail((ctx), e_, #call); \
  } while (0)

}  // namespace ubr

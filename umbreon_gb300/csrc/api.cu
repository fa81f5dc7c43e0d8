// api.cu -- the extern "C" entry points of libubr (declared in include/ubr.h).
// The C-ABI never throws: every failure is a ubr_status plus a message kept
// on the context (ubr_context_last_error).
#include <cstdio>
#include <algorithm>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "ubr_context.h"

namespace ubr {

ubr_status buildScene(Context* c, const ubr_scene_desc& d, Scene** out);
void releaseScene(Scene* sc);
ubr_status renderFrame(Context* c, const Scene* sc, const ubr_render_desc& d, ubr_frame& fr,
                       const volatile int32_t* cancel, uint64_t* progress);
ubr_status occludedBatch(Context* c, const Scene* sc, const float* segs, uint64_t n, float eps, uint8_t* out,
                         int32_t memory);
struct Job {
  const Scene* scene;
  const ubr_render_desc* desc;
  ubr_frame* frame;
};
ubr_status renderBatch(Context* c, const std::vector<Job>& jobs, ubr_frame* total);
ubr_status adjoint(Context* c, const Scene* sc, const ubr_render_desc& d, const float* dColor, ubr_grads& g);
ubr_status occludedFilteredBatch(Context* c, const Scene* sc, const float* segs, uint64_t n, float eps,
                                 float grazeCos, float coplanar, const uint32_t* offs, const int32_t* faces,
                                 uint8_t* out, int32_t memory);
ubr_status occludedBatchNoAlloc(Context* c, const Scene* sc, const float* segs, uint64_t n, float eps,
                                uint8_t* out);

ubr_status setError(Context* c, ubr_status s, const std::string& msg) {
  if (c) c->lastError = msg;
  return s;
}

ubr_status cudaFail(Context* c, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear a non-sticky error so the context stays usable
  return setError(c, e == cudaErrorMemoryAllocation ? UBR_OUT_OF_MEMORY : UBR_CUDA_ERROR, m);
}

ubr_status devAlloc(Context* c, DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (c->arenaCap && c->arenaUsed + bytes > c->arenaCap)
    return setError(c, UBR_OUT_OF_MEMORY, "device arena cap exceeded");
  void* p = nullptr;
  // stream-ordered from the context's pool: after the first frames a scene
  // build or a scratch growth reuses pooled memory instead of cudaMalloc
  cudaError_t e = c->pool ? cudaMallocFromPoolAsync(&p, bytes, c->pool, c->stream) : cudaMalloc(&p, bytes);
  if (e != cudaSuccess) return cudaFail(c, e, "device allocation");
  b.ptr = p;
  b.bytes = bytes;
  c->arenaUsed += bytes;
  return UBR_OK;
}

void devFree(Context* c, DevBuf& b) {
  if (b.ptr) {
    if (c->pool) cudaFreeAsync(b.ptr, c->stream);
    else cudaFree(b.ptr);
    c->arenaUsed -= b.bytes;
  }
  b.ptr = nullptr;
  b.bytes = 0;
}

ubr_status scratchGet(Context* c, int i, size_t bytes, void** out) {
  if (size_t(i) >= c->scratch.size()) c->scratch.resize(size_t(i) + 1);
  DevBuf& b = c->scratch[size_t(i)];
  if (b.bytes < bytes) {
    // grow geometrically; wait for in-flight users of the old block first
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cudaFail(c, e, "cudaStreamSynchronize");
    devFree(c, b);
    ubr_status st = devAlloc(c, b, bytes + bytes / 4);
    if (st != UBR_OK) return st;
  }
  *out = b.ptr;
  return UBR_OK;
}

}  // namespace ubr

using namespace ubr;

struct ubr_context {
  Context impl;
};
struct ubr_scene {
  Scene* impl;
};

extern "C" {

const char* ubr_status_string(ubr_status s) {
  switch (s) {
    case UBR_OK: return "ok";
    case UBR_INVALID_ARGUMENT: return "invalid argument";
    case UBR_OUT_OF_MEMORY: return "out of memory";
    case UBR_CUDA_ERROR: return "CUDA error";
    case UBR_CANCELLED: return "cancelled";
    case UBR_TRAVERSAL_LIMIT: return "traversal stack limit reached";
    case UBR_NO_DEVICE: return "no CUDA device";
    case UBR_INTERNAL: return "internal error";
  }
  return "unrecognized status";
}

uint32_t ubr_abi_version(void) { return UBR_ABI_VERSION; }

ubr_status ubr_context_create(ubr_context** out, const ubr_context_desc* desc) {
  if (!out) return UBR_INVALID_ARGUMENT;
  *out = nullptr;
  if (desc && desc->abi_version != UBR_ABI_VERSION) return UBR_INVALID_ARGUMENT;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return UBR_NO_DEVICE;
  }
  const int dev = desc ? desc->device : 0;
  if (dev < 0 || dev >= ndev) return UBR_INVALID_ARGUMENT;
  ubr_context* c = new (std::nothrow) ubr_context();
  if (!c) return UBR_OUT_OF_MEMORY;
  Context& x = c->impl;
  x.device = dev;
  x.arenaCap = desc ? desc->arena_bytes : 0;
  if (desc && desc->bvh_leaf_max) {
    if (desc->bvh_leaf_max > uint32_t(kWideLeafMax)) {
      delete c;
      return UBR_INVALID_ARGUMENT;
    }
    x.leafMax = int(desc->bvh_leaf_max);
  }
  if (desc && desc->trace_mode) {
    if (desc->trace_mode > 4) {
      delete c;
      return UBR_INVALID_ARGUMENT;
    }
    x.traceMode = int(desc->trace_mode);
  }
  if (desc && desc->disable_graphs) x.useGraphs = false;
  if (desc && desc->bvh_builder) {
    if (desc->bvh_builder > 2) {
      delete c;
      return UBR_INVALID_ARGUMENT;
    }
    x.builder = int(desc->bvh_builder);
  }
  if (desc && desc->bvh_collapse) {
    if (desc->bvh_collapse > 2) {
      delete c;
      return UBR_INVALID_ARGUMENT;
    }
    x.collapse = int(desc->bvh_collapse);
  }
  if (desc && desc->bvh_sah_prim_scale != 0.0f) {
    if (!(desc->bvh_sah_prim_scale > 0.0f && desc->bvh_sah_prim_scale < 1000.0f)) {
      delete c;
      return UBR_INVALID_ARGUMENT;
    }
    x.sahPrimScale = desc->bvh_sah_prim_scale;
  }
  if (cudaSetDevice(dev) != cudaSuccess) {
    delete c;
    return UBR_CUDA_ERROR;
  }
  if (desc && desc->stream) {
    x.stream = static_cast<cudaStream_t>(desc->stream);
  } else {
    if (cudaStreamCreateWithFlags(&x.stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return UBR_CUDA_ERROR;
    }
    x.ownStream = true;
  }
  for (cudaEvent_t& e : x.ev) cudaEventCreate(&e);
  {
    // the context's device memory pool; freed blocks stay in the pool
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    if (cudaMemPoolCreate(&x.pool, &props) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(x.pool, cudaMemPoolAttrReleaseThreshold, &keep);
    } else {
      cudaGetLastError();
      x.pool = nullptr;  // plain cudaMalloc
    }
  }
  if (cudaMallocHost(&x.pinned, 4096) != cudaSuccess) {
    cudaGetLastError();
    x.pinned = nullptr;
    ubr_context_destroy(c);
    return UBR_OUT_OF_MEMORY;
  }
  *out = c;
  return UBR_OK;
}

ubr_status ubr_context_destroy(ubr_context* c) {
  if (!c) return UBR_OK;
  Context& x = c->impl;
  cudaSetDevice(x.device);
  if (x.stream) cudaStreamSynchronize(x.stream);
  // scenes still alive lose their device memory now; their handles stay
  // valid for ubr_scene_release only
  for (void* h : x.sceneHandles) {
    ubr_scene* s = static_cast<ubr_scene*>(h);
    if (s->impl) releaseScene(s->impl);
    s->impl = nullptr;
  }
  x.sceneHandles.clear();
  for (DevBuf& b : x.scratch) devFree(&x, b);
  if (x.pool) {
    cudaStreamSynchronize(x.stream);
    cudaMemPoolDestroy(x.pool);
    x.pool = nullptr;
  }
  for (cudaEvent_t& e : x.ev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t& e : x.pev)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t& e : x.giEv)
    if (e) cudaEventDestroy(e);
  if (x.graphExec) cudaGraphExecDestroy(x.graphExec);
  if (x.pinned) cudaFreeHost(x.pinned);
  if (x.ownStream && x.stream) cudaStreamDestroy(x.stream);
  delete c;
  return UBR_OK;
}

const char* ubr_context_last_error(const ubr_context* c) {
  if (!c) return "null context";
  return c->impl.lastError.c_str();
}

ubr_status ubr_scene_build(ubr_context* c, const ubr_scene_desc* desc, ubr_scene** out) {
  if (!c || !desc || !out) return c ? setError(&c->impl, UBR_INVALID_ARGUMENT, "scene_build: NULL argument")
                                    : UBR_INVALID_ARGUMENT;
  *out = nullptr;
  cudaSetDevice(c->impl.device);
  Scene* sc = nullptr;
  ubr_status st;
  try {
    st = buildScene(&c->impl, *desc, &sc);
  } catch (const std::bad_alloc&) {
    return setError(&c->impl, UBR_OUT_OF_MEMORY, "host allocation failed");
  } catch (...) {
    return setError(&c->impl, UBR_INTERNAL, "scene build failed");
  }
  if (st != UBR_OK) return st;
  ubr_scene* s = new (std::nothrow) ubr_scene{sc};
  if (!s) {
    releaseScene(sc);
    return setError(&c->impl, UBR_OUT_OF_MEMORY, "host allocation failed");
  }
  c->impl.sceneHandles.push_back(s);
  *out = s;
  return UBR_OK;
}

ubr_status ubr_scene_release(ubr_scene* s) {
  if (!s) return UBR_OK;
  if (s->impl) {
    Context* x = s->impl->ctx;
    cudaSetDevice(x->device);
    cudaStreamSynchronize(x->stream);
    releaseScene(s->impl);
    auto& v = x->sceneHandles;
    v.erase(std::remove(v.begin(), v.end(), static_cast<void*>(s)), v.end());
  }
  delete s;
  return UBR_OK;
}

ubr_status ubr_scene_get_info(const ubr_scene* s, ubr_scene_info* info) {
  if (!s || !info || !s->impl) return UBR_INVALID_ARGUMENT;
  const Scene& sc = *s->impl;
  std::memset(info, 0, sizeof(*info));
  for (int k = 0; k < 4; ++k) {
    info->prim_count[k] = sc.primCount[k];
    info->geom_id[k] = sc.view.geomID[k];
  }
  info->bvh_nodes = sc.nodes;
  info->device_bytes = sc.deviceBytes;
  info->build_ms = sc.buildMs;
  info->flatten_ms = sc.flattenMs;
  info->upload_ms = sc.uploadMs;
  for (int k = 0; k < 3; ++k) {
    info->bounds_lo[k] = sc.lo[k];
    info->bounds_hi[k] = sc.hi[k];
  }
  return UBR_OK;
}

ubr_status ubr_render(ubr_context* c, const ubr_scene* s, const ubr_render_desc* desc, ubr_frame* frame,
                      const volatile int32_t* cancel_flag, uint64_t* progress_units) {
  if (!c) return UBR_INVALID_ARGUMENT;
  if (!s || !s->impl || !desc || !frame)
    return setError(&c->impl, UBR_INVALID_ARGUMENT, "render: NULL argument");
  if (s->impl->ctx != &c->impl) return setError(&c->impl, UBR_INVALID_ARGUMENT, "render: scene from another context");
  cudaSetDevice(c->impl.device);
  if (cancel_flag && *cancel_flag) return setError(&c->impl, UBR_CANCELLED, "render cancelled before launch");
  try {
    return renderFrame(&c->impl, s->impl, *desc, *frame, cancel_flag, progress_units);
  } catch (const std::bad_alloc&) {
    return setError(&c->impl, UBR_OUT_OF_MEMORY, "host allocation failed");
  } catch (...) {
    return setError(&c->impl, UBR_INTERNAL, "render failed");
  }
}

ubr_status ubr_render_batch(ubr_context* c, uint32_t n, const ubr_batch_item* items, ubr_frame* total) {
  if (!c) return UBR_INVALID_ARGUMENT;
  if (n == 0) return UBR_OK;
  if (!items) return setError(&c->impl, UBR_INVALID_ARGUMENT, "render_batch: NULL items");
  std::vector<Job> jobs;
  jobs.reserve(n);
  for (uint32_t i = 0; i < n; ++i) {
    const ubr_batch_item& it = items[i];
    if (!it.scene || !it.scene->impl || !it.desc || !it.frame)
      return setError(&c->impl, UBR_INVALID_ARGUMENT, "render_batch: NULL scene, desc or frame in an item");
    if (it.scene->impl->ctx != &c->impl)
      return setError(&c->impl, UBR_INVALID_ARGUMENT, "render_batch: scene from another context");
    jobs.push_back(Job{it.scene->impl, it.desc, it.frame});
  }
  cudaSetDevice(c->impl.device);
  try {
    return renderBatch(&c->impl, jobs, total);
  } catch (const std::bad_alloc&) {
    return setError(&c->impl, UBR_OUT_OF_MEMORY, "host allocation failed");
  } catch (...) {
    return setError(&c->impl, UBR_INTERNAL, "render failed");
  }
}

ubr_status ubr_adjoint(ubr_context* c, const ubr_scene* s, const ubr_render_desc* desc, const float* d_color,
                       ubr_grads* grads) {
  if (!c) return UBR_INVALID_ARGUMENT;
  if (!s || !s->impl) return setError(&c->impl, UBR_INVALID_ARGUMENT, "adjoint: NULL scene");
  if (!desc || !grads) return setError(&c->impl, UBR_INVALID_ARGUMENT, "adjoint: NULL desc or grads");
  if (s->impl->ctx != &c->impl) return setError(&c->impl, UBR_INVALID_ARGUMENT, "adjoint: scene from another context");
  cudaSetDevice(c->impl.device);
  return adjoint(&c->impl, s->impl, *desc, d_color, *grads);
}

ubr_status ubr_occluded_batch(ubr_context* c, const ubr_scene* s, const float* segs, uint64_t n, float eps,
                              uint8_t* out, int32_t memory) {
  if (!c) return UBR_INVALID_ARGUMENT;
  if (!s || !s->impl) return setError(&c->impl, UBR_INVALID_ARGUMENT, "occluded_batch: NULL scene");
  cudaSetDevice(c->impl.device);
  return occludedBatch(&c->impl, s->impl, segs, n, eps, out, memory);
}

ubr_status ubr_occluded_filtered_batch(ubr_context* c, const ubr_scene* s, const float* segs, uint64_t n,
                                       float eps, float graze_cos_eps, float coplanar_eps,
                                       const uint32_t* exclude_offsets, const int32_t* exclude_faces, uint8_t* out,
                                       int32_t memory) {
  if (!c) return UBR_INVALID_ARGUMENT;
  if (!s || !s->impl) return setError(&c->impl, UBR_INVALID_ARGUMENT, "occluded_filtered_batch: NULL scene");
  if (s->impl->ctx != &c->impl)
    return setError(&c->impl, UBR_INVALID_ARGUMENT, "occluded_filtered_batch: scene from another context");
  cudaSetDevice(c->impl.device);
  return occludedFilteredBatch(&c->impl, s->impl, segs, n, eps, graze_cos_eps, coplanar_eps, exclude_offsets,
                               exclude_faces, out, memory);
}

ubr_status ubr_occluded_batch_noalloc(ubr_context* c, const ubr_scene* s, const float* segs, uint64_t n, float eps,
                                      uint8_t* out) {
  if (!c) return UBR_INVALID_ARGUMENT;
  if (!s || !s->impl) return setError(&c->impl, UBR_INVALID_ARGUMENT, "occluded_batch_noalloc: NULL scene");
  if (s->impl->ctx != &c->impl)
    return setError(&c->impl, UBR_INVALID_ARGUMENT, "occluded_batch_noalloc: scene from another context");
  cudaSetDevice(c->impl.device);
  return occludedBatchNoAlloc(&c->impl, s->impl, segs, n, eps, out);
}

}  // extern "C"

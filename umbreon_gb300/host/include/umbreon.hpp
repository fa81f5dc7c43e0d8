// umbreon public API, GB300 edition.
//
// render() runs the ray-cast + shade frame on the GPU through the C-ABI in
// ubr.h: scene upload and BVH build, primary rays through the transparency
// walk, POV and Principled (direct) shading with AO and shadow rays, fog,
// supersample resolve or adaptive AA, coarse-grid AO, the a-trous denoiser
// and assumed gamma.  Group-alpha blending (Scene::groupBlend) runs one GPU
// pass per group on the host side exactly as the reference composes them.
// Requests outside this library throw std::runtime_error: GI (gi), stroke or
// object-space edges.  An OIDN denoiser request runs the a-trous with a
// logged warning, as the reference does when built without OIDN.
#pragma once

#include <chrono>
#include <memory>

#include "render/render_types.hpp"
#include "scene.hpp"

#define UMBREON_VERSION_MAJOR 0
#define UMBREON_VERSION_MINOR 1
#define UMBREON_VERSION_PATCH 0

namespace umbreon {

FrameResult render(const Scene& scene, const RenderOptions& opt);
FrameResult render(const Scene& scene, const RenderOptions& opt, RenderProgress& progress);

class RenderTask {
 public:
  RenderTask(RenderTask&&) noexcept;
  RenderTask& operator=(RenderTask&&) noexcept;
  ~RenderTask();
  RenderTask(const RenderTask&) = delete;
  RenderTask& operator=(const RenderTask&) = delete;

  float progress() const noexcept;
  RenderPhase phase() const noexcept;
  bool done() const noexcept;
  void cancel() noexcept;
  bool wait_for(std::chrono::milliseconds timeout) const;
  void wait() const;
  FrameResult get();

 private:
  struct Impl;
  explicit RenderTask(std::unique_ptr<Impl> impl) noexcept;
  friend RenderTask renderAsync(Scene scene, RenderOptions opt);
  std::unique_ptr<Impl> p_;
};

RenderTask renderAsync(Scene scene, RenderOptions opt);

}  // namespace umbreon

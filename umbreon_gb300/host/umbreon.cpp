// umbreon.cpp -- the C++ drop-in layer of the GB300 path.
//
// Implements the umbreon public API (umbreon.hpp) on top of the C-ABI in
// ubr.h: a Scene is flattened into the ABI's structure-of-arrays description,
// built and rendered on the GPU, and the result is returned as a FrameResult
// laid out the way renderFrame leaves it (src/umbreon/render/pipeline.cpp:
// colour at the final size, depth/viewZ on the supersampled grid).
// Group-alpha blending (src/umbreon/umbreon.cpp:141-253) is composed here, on
// the host, from one GPU render per pass.
#include "umbreon.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <mutex>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "log.hpp"
#include "postprocess/image_ops.hpp"
#include "ubr.h"

namespace umbreon {

// ---------------------------------------------------------------------------
// logging (process-wide sink, stderr default)

namespace {
std::mutex& logMutex() {
  static std::mutex m;
  return m;
}
LogSink& logSink() {
  static LogSink s;
  return s;
}
}  // namespace

void setLogSink(LogSink sink) {
  std::lock_guard<std::mutex> lk(logMutex());
  logSink() = std::move(sink);
}

void logMessage(LogLevel level, const char* fmt, ...) {
  char buf[2048];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  std::lock_guard<std::mutex> lk(logMutex());
  if (logSink()) logSink()(level, buf);
  else std::fprintf(stderr, "umbreon %s: %s\n", level == LogLevel::Warning ? "warning" : "info", buf);
}

// ---------------------------------------------------------------------------
// progress

void RenderProgress::setPhasePlan(const RenderPhasePlan& plan) noexcept {
  const float share[kPlanSlots] = {plan.setup, plan.coarseAo, plan.primary, plan.globalIllum, plan.edges,
                                   plan.postprocess};
  double sum = 0.0;
  for (float f : share)
    if (std::isfinite(f) && f > 0.0f) sum += f;
  if (!(sum > 0.0)) {
    plan_.store(kDefaultPlanPacked, std::memory_order_relaxed);
    return;
  }
  std::uint64_t packed = 0;
  for (int i = 0; i < kPlanSlots; ++i) {
    const double f = (std::isfinite(share[i]) && share[i] > 0.0f) ? share[i] : 0.0;
    const std::uint64_t q = static_cast<std::uint64_t>(f / sum * double(kPlanPermille) + 0.5);
    packed |= std::min(q, kPlanMask) << (i * kPlanBits);
  }
  plan_.store(packed ? packed : kDefaultPlanPacked, std::memory_order_relaxed);
}

RenderPhasePlan RenderProgress::phasePlan() const noexcept {
  const std::uint64_t packed = plan_.load(std::memory_order_relaxed);
  float w[kPlanSlots];
  float total = 0.0f;
  for (int i = 0; i < kPlanSlots; ++i) {
    w[i] = float((packed >> (i * kPlanBits)) & kPlanMask);
    total += w[i];
  }
  RenderPhasePlan out;
  if (total <= 0.0f) return out;
  out.setup = w[0] / total;
  out.coarseAo = w[1] / total;
  out.primary = w[2] / total;
  out.globalIllum = w[3] / total;
  out.edges = w[4] / total;
  out.postprocess = w[5] / total;
  return out;
}

float RenderProgress::fraction() const noexcept {
  const RenderPhasePlan pl = phasePlan();
  const float shares[kPlanSlots] = {pl.setup, pl.coarseAo, pl.primary, pl.globalIllum, pl.edges, pl.postprocess};
  const int slot = static_cast<int>(phase()) - 1;  // Idle -> -1, Done -> 6
  float before = 0.0f;
  for (int i = 0; i < slot && i < kPlanSlots; ++i) before += shares[i];
  float within = 0.0f;
  const std::uint64_t total = unitsTotal(), done = unitsDone();
  if (total > 0) within = std::min(1.0f, std::max(0.0f, float(done) / float(total)));
  const float span = (slot >= 0 && slot < kPlanSlots) ? shares[slot] : 0.0f;
  const float inPass = before + span * within;
  const std::uint64_t count = std::max<std::uint64_t>(1, passCount_.load(std::memory_order_relaxed));
  const std::uint64_t index = std::min<std::uint64_t>(count - 1, passIndex_.load(std::memory_order_relaxed));
  return std::min(1.0f, std::max(0.0f, (float(index) + inPass) / float(count)));
}

const char* toString(RenderPhase p) noexcept {
  switch (p) {
    case RenderPhase::Idle: return "Idle";
    case RenderPhase::Setup: return "Setup";
    case RenderPhase::CoarseAo: return "CoarseAO";
    case RenderPhase::Primary: return "Primary";
    case RenderPhase::GlobalIllum: return "GI";
    case RenderPhase::Edges: return "Edges";
    case RenderPhase::Postprocess: return "Postprocess";
    case RenderPhase::Done: return "Done";
  }
  return "Unknown";
}

// ---------------------------------------------------------------------------
// image helpers (host side)

std::vector<float> boxDownsample(const std::vector<float>& src, int w, int h, int channels, int ss) {
  const int ow = w / ss, oh = h / ss;
  std::vector<float> out(static_cast<std::size_t>(ow) * oh * channels, 0.0f);
  const float inv = 1.0f / static_cast<float>(ss * ss);
  for (int y = 0; y < oh; ++y)
    for (int x = 0; x < ow; ++x)
      for (int c = 0; c < channels; ++c) {
        float acc = 0.0f;
        for (int dy = 0; dy < ss; ++dy)
          for (int dx = 0; dx < ss; ++dx) {
            const float v = src[(static_cast<std::size_t>(y * ss + dy) * w + (x * ss + dx)) * channels + c];
            acc += std::isfinite(v) ? v : 0.0f;  // a non-finite sample counts as 0
          }
        out[(static_cast<std::size_t>(y) * ow + x) * channels + c] = acc * inv;
      }
  return out;
}

void applyAssumedGamma(FrameResult& frame, float g) {
  if (std::fabs(g - 1.0f) <= 1.0e-4f) return;
  const std::size_t n = static_cast<std::size_t>(frame.width) * frame.height;
  for (std::size_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) {
      float& v = frame.color[i * 4 + c];
      v = v > 0.0f ? std::pow(v, g) : 0.0f;
    }
}

float srgbEncodeF(float v) {
  v = std::min(1.0f, std::max(0.0f, v));
  return v <= 0.0031308f ? 12.92f * v : 1.055f * std::pow(v, 1.0f / 2.4f) - 0.055f;
}

float srgbDecodeF(float s) {
  s = std::min(1.0f, std::max(0.0f, s));
  return s <= 0.04045f ? s / 12.92f : std::pow((s + 0.055f) / 1.055f, 2.4f);
}

std::vector<std::uint8_t> srgbEncode8(const FrameResult& frame, int channels) {
  const std::size_t n = static_cast<std::size_t>(frame.width) * frame.height;
  std::vector<std::uint8_t> out(n * channels);
  auto q = [](float v) {
    const int i = static_cast<int>(v * 255.0f + 0.5f);
    return static_cast<std::uint8_t>(std::min(255, std::max(0, i)));
  };
  for (std::size_t i = 0; i < n; ++i) {
    for (int c = 0; c < 3 && c < channels; ++c) out[i * channels + c] = q(srgbEncodeF(frame.color[i * 4 + c]));
    if (channels == 4) out[i * 4 + 3] = q(std::min(1.0f, std::max(0.0f, frame.color[i * 4 + 3])));
  }
  return out;
}

// ---------------------------------------------------------------------------
// GPU frame

namespace {

// One process-wide context; render() is synchronous and, like the reference,
// not meant to be called concurrently -- the mutex serialises callers.
std::mutex& gpuMutex() {
  static std::mutex m;
  return m;
}

ubr_context* gpuContext() {
  static ubr_context* ctx = nullptr;
  if (!ctx) {
    ubr_context_desc d{};
    d.abi_version = UBR_ABI_VERSION;
    const char* dev = std::getenv("UMBREON_GB300_DEVICE");
    d.device = dev ? std::atoi(dev) : 0;
    const ubr_status st = ubr_context_create(&ctx, &d);
    if (st != UBR_OK)
      throw std::runtime_error(std::string("umbreon: GPU context creation failed: ") + ubr_status_string(st));
  }
  return ctx;
}

void check(ubr_context* ctx, ubr_status st, const char* what) {
  if (st == UBR_OK || st == UBR_CANCELLED) return;
  throw std::runtime_error(std::string("umbreon: ") + what + " failed: " + ubr_status_string(st) + ": " +
                           ubr_context_last_error(ctx));
}

ubr_material toAbi(const Material& m) {
  ubr_material a{};
  a.ambient = m.ambient;
  a.diffuse = m.diffuse;
  a.specular = m.specular;
  a.roughness = m.roughness;
  a.brilliance = m.brilliance;
  a.phong = m.phong;
  a.phong_size = m.phongSize;
  a.metallic = m.metallic ? 1u : 0u;
  a.reflection = m.reflection;
  a.emission = m.emission;
  a.model = static_cast<uint32_t>(m.model);
  a.pbr_metallic = m.pbr.metallic;
  a.pbr_roughness = m.pbr.roughness;
  a.pbr_specular = m.pbr.specular;
  a.pbr_anisotropy = m.pbr.anisotropy;
  a.pbr_anisotropy_rotation = m.pbr.anisotropyRotation;
  return a;
}

// Structure-of-arrays copy of a Scene that owns the arrays the desc points at.
struct FlatScene {
  std::vector<float> pos, nrm, col;
  std::vector<ubr_material> meshMats;
  std::vector<float> sph, sphCol, cylP0, cylP1, cylR, cylCol, cylOp1, offs;
  std::vector<ubr_material> sphMat, cylMat;
  std::vector<uint16_t> sphGrp, cylGrp;
  std::vector<uint8_t> sphEdge, cylOpen, cylEdge;
  ubr_scene_desc desc{};

  explicit FlatScene(const Scene& s) {
    ubr_scene_desc& d = desc;
    d.abi_version = UBR_ABI_VERSION;
    const Mesh& m = s.mesh;
    for (const Vec3& p : m.positions) pos.insert(pos.end(), {p.x, p.y, p.z});
    for (std::size_t i = 0; i < m.positions.size(); ++i) {
      const Vec3 n = i < m.normals.size() ? m.normals[i] : Vec3{};
      const Vec4 c = i < m.colors.size() ? m.colors[i] : Vec4{};
      nrm.insert(nrm.end(), {n.x, n.y, n.z});
      col.insert(col.end(), {c.x, c.y, c.z, c.w});
    }
    d.mesh_vertex_count = m.positions.size();
    d.mesh_positions = pos.data();
    d.mesh_normals = nrm.data();
    d.mesh_colors = col.data();
    d.mesh_triangle_count = m.triangleCount();
    d.mesh_index = m.index.empty() ? nullptr : m.index.data();
    d.mesh_material = toAbi(m.material);
    for (const Material& mm : m.materials) meshMats.push_back(toAbi(mm));
    d.mesh_materials = meshMats.empty() ? nullptr : meshMats.data();
    d.mesh_material_count = static_cast<uint32_t>(meshMats.size());
    d.mesh_tri_material = m.triMaterialId.empty() ? nullptr : m.triMaterialId.data();
    d.mesh_tri_group = m.triGroupId.empty() ? nullptr : m.triGroupId.data();
    for (const Sphere& sp : s.spheres) {
      sph.insert(sph.end(), {sp.center.x, sp.center.y, sp.center.z, sp.radius});
      sphCol.insert(sphCol.end(), {sp.color.x, sp.color.y, sp.color.z, sp.color.w});
      sphMat.push_back(toAbi(sp.material));
      sphGrp.push_back(sp.group);
      sphEdge.push_back(sp.fromEdgeMacro ? 1 : 0);
    }
    d.sphere_count = s.spheres.size();
    d.sphere_center_radius = sph.data();
    d.sphere_color = sphCol.data();
    d.sphere_material = sphMat.data();
    d.sphere_group = sphGrp.data();
    d.sphere_from_edge = sphEdge.data();
    for (const Cylinder& c : s.cylinders) {
      cylP0.insert(cylP0.end(), {c.p0.x, c.p0.y, c.p0.z});
      cylP1.insert(cylP1.end(), {c.p1.x, c.p1.y, c.p1.z});
      cylR.push_back(c.radius);
      cylCol.insert(cylCol.end(), {c.color.x, c.color.y, c.color.z, c.color.w});
      cylOp1.push_back(c.opacity1);
      cylMat.push_back(toAbi(c.material));
      cylGrp.push_back(c.group);
      cylOpen.push_back(c.open ? 1 : 0);
      cylEdge.push_back(c.fromEdgeMacro ? 1 : 0);
    }
    d.cylinder_count = s.cylinders.size();
    d.cyl_p0 = cylP0.data();
    d.cyl_p1 = cylP1.data();
    d.cyl_radius = cylR.data();
    d.cyl_color = cylCol.data();
    d.cyl_opacity1 = cylOp1.data();
    d.cyl_material = cylMat.data();
    d.cyl_group = cylGrp.data();
    d.cyl_open = cylOpen.data();
    d.cyl_from_edge = cylEdge.data();
    for (const Vec3& o : s.instanceOffsets) offs.insert(offs.end(), {o.x, o.y, o.z});
    d.instance_count = s.instanceOffsets.size();
    d.instance_offsets = offs.empty() ? nullptr : offs.data();
  }
};

ubr_render_desc toRenderDesc(const Scene& s, const RenderOptions& o, std::vector<ubr_light>& lights) {
  ubr_render_desc d{};
  d.abi_version = UBR_ABI_VERSION;
  d.width = o.width;
  d.height = o.height;
  d.supersample = o.supersample;
  const Camera& c = s.camera;
  const float cp[3] = {c.position.x, c.position.y, c.position.z};
  const float cd[3] = {c.direction.x, c.direction.y, c.direction.z};
  const float cu[3] = {c.up.x, c.up.y, c.up.z};
  for (int k = 0; k < 3; ++k) {
    d.cam_position[k] = cp[k];
    d.cam_direction[k] = cd[k];
    d.cam_up[k] = cu[k];
  }
  d.cam_fovy = c.fovy;
  d.cam_orthographic = c.orthographic ? 1u : 0u;
  d.cam_height = c.height;
  lights.clear();
  for (const DistantLight& l : s.lights) {
    ubr_light a{};
    a.direction[0] = l.direction.x;
    a.direction[1] = l.direction.y;
    a.direction[2] = l.direction.z;
    a.color[0] = l.color.x;
    a.color[1] = l.color.y;
    a.color[2] = l.color.z;
    a.intensity = l.intensity;
    a.casts_highlight = l.castsHighlight ? 1u : 0u;
    a.angular_radius = l.angularRadius;
    lights.push_back(a);
  }
  d.lights = lights.empty() ? nullptr : lights.data();
  d.light_count = static_cast<uint32_t>(lights.size());
  const float amb[3] = {s.ambientColor.x, s.ambientColor.y, s.ambientColor.z};
  const float bg[3] = {s.background.x, s.background.y, s.background.z};
  const float fc[3] = {s.fog.color.x, s.fog.color.y, s.fog.color.z};
  for (int k = 0; k < 3; ++k) {
    d.ambient_color[k] = amb[k];
    d.background[k] = bg[k];
    d.fog_color[k] = fc[k];
    d.ao_sky_color[k] = o.aoSkyColor[k];
    d.ao_ground_color[k] = o.aoGroundColor[k];
    d.ao_up[k] = o.aoUp[k];
  }
  d.fog_enabled = s.fog.enabled ? 1u : 0u;
  d.fog_start = s.fog.start;
  d.fog_end = s.fog.end;
  d.clip_near = s.clipNear;
  d.clip_far = s.clipFar;
  d.assumed_gamma = s.assumedGamma;
  d.ao_samples = o.aoSamples;
  d.ao_distance = o.aoDistance;
  d.ao_intensity = o.aoIntensity;
  d.ao_falloff_power = o.aoFalloffPower;
  d.ao_multiscale = o.aoMultiScale;
  d.ao_bent_normal = o.aoBentNormal;
  d.ao_use_camera_up = o.aoUseCameraUp;
  d.ao_multibounce = o.aoMultibounce;
  d.ao_low_discrepancy = o.aoLowDiscrepancy;
  d.ao_diffuse_factor = o.aoDiffuseFactor;
  d.shadows = o.shadows;
  d.shadow_samples = o.shadowSamples;
  d.light_radius_deg = o.lightRadius;
  d.env_lights = o.envLights;
  d.env_intensity = o.envIntensity;
  d.env_key_scale = o.envKeyScale;
  d.env_angle = o.envAngle;
  d.specular_scale = o.specularScale;
  d.transparency = o.transparency;
  d.transparent_background = o.transparentBackground;
  d.max_transparent_layers = o.maxTransparentLayers;
  d.gi_integrator = o.giIntegrator;
  d.ao_write_aov = o.aoWriteAov ? 1u : 0u;
  d.aa_mode = o.aaMode;
  d.aa_threshold = o.aaThreshold;
  d.aa_depth = o.aaDepth;
  d.ao_res_div = o.aoResDiv;
  d.denoiser = o.denoiser;
  d.denoise_iters = o.denoiseIters;
  d.denoise_sigma_z = o.denoiseSigmaZ;
  d.denoise_sigma_n = o.denoiseSigmaN;
  d.denoise_sigma_l = o.denoiseSigmaL;
  d.denoise_demodulate_albedo = o.denoiseDemodulateAlbedo ? 1u : 0u;
  if (o.gi) {
    // pipeline.cpp:60-78: adaptive AA and coarse-grid AO fall back under GI
    if (d.aa_mode == 1) d.aa_mode = 0;
    if ((o.aoResDiv < 0 ? std::max(1, o.supersample) : o.aoResDiv) > 1) d.ao_res_div = 0;
    d.gi = 1u;
    d.pt1_spp = o.pt1Spp;
    d.gi_bounces = o.giBounces;
    d.gi_max_distance = o.giMaxDistance;
    d.gi_intensity = o.giIntensity;
    d.gi_env_intensity = o.giEnvIntensity;
    d.pt1_seed = o.pt1Seed;
    d.pt1_sky_mode = o.pt1SkyMode;
    for (int k = 0; k < 3; ++k) d.pt1_sky_radiance[k] = o.pt1SkyRadiance[k];
    d.pt1_ld = o.pt1Ld ? 1u : 0u;
    d.pt1_clamp = o.pt1Clamp;
    d.pt1_gather_div = o.pt1GatherDiv;  // -1 (the supersample factor) resolved by the library
    d.pt1_half_res = o.pt1HalfRes ? 1u : 0u;
    d.pt1_denoise = o.pt1Denoise ? 1u : 0u;
    d.pt1_upsample_normal_pow = o.pt1UpsampleNormalPow;
    d.pt1_upsample_depth_scale = o.pt1UpsampleDepthScale;
    d.pt1_edge_patch = o.pt1EdgePatch ? 1u : 0u;
    d.pt1_edge_patch_spp_mul = o.pt1EdgePatchSppMul;
    d.pt1_edge_patch_thresh = o.pt1EdgePatchThresh;
    d.pt2_pattern = o.pt2Pattern;
    d.pt2_emissive = o.pt2Emissive ? 1u : 0u;
    d.pt2_rounds = o.pt2Rounds;
    d.pt2_radius = o.pt2Radius;
    d.pt2_unbiased = o.pt2Unbiased ? 1u : 0u;
    d.pt2_m_cap = o.pt2MCap;
    d.pt2_w_clamp = o.pt2WClamp;
    d.pt2_adaptive = o.pt2Adaptive ? 1u : 0u;
    d.pt2_adaptive_thresh = o.pt2AdaptiveThresh;
    d.pt2_adaptive_mul = o.pt2AdaptiveMul;
    d.pt2_emissive_nee = o.pt2EmissiveNee ? 1u : 0u;
    d.pt2_reflect = o.pt2Reflect ? 1u : 0u;
    d.pt2_glossy = o.pt2Glossy ? 1u : 0u;
    d.pt2_glossy_spp = o.pt2GlossySpp;
    d.pt2_glossy_denoise = o.pt2GlossyDenoise ? 1u : 0u;
  }
  return d;
}

void rejectUnsupported(const RenderOptions& opt) {
  if (opt.strokeEdges.enable && opt.objectSpaceEdges.enable)
    throw std::runtime_error(
        "umbreon::render: strokeEdges and objectSpaceEdges are mutually exclusive; enable at most one");
  if (opt.gi && opt.giIntegrator != 1 && opt.giIntegrator != 2)
    throw std::runtime_error(
        "umbreon::render: the irradiance-cache GI integrator (giIntegrator = 0) is not part of this library");
  if (opt.strokeEdges.enable || opt.objectSpaceEdges.enable)
    throw std::runtime_error("umbreon::render: edge passes are not part of the GB300 ray-cast + shade library");
}

// One GPU pass: the work of renderFrame (pipeline.cpp:20-256) minus the
// edge passes and GI.
FrameResult renderFrameGpu(const Scene& scene, const RenderOptions& opt, RenderProgress* progress) {
  if (opt.denoiser == 2)
    logMessage(LogLevel::Warning,
               "OIDN denoiser backend not built; falling back to the built-in a-trous denoiser");
  const int ss = std::max(1, opt.supersample);
  FrameResult f;
  f.width = opt.width;
  f.height = opt.height;
  const std::size_t nout = static_cast<std::size_t>(opt.width) * opt.height;
  const std::size_t nhi = nout * ss * ss;
  f.color.assign(nout * 4, 0.0f);
  f.depth.assign(nhi, 0.0f);
  if (scene.fog.enabled) f.viewZ.assign(nhi, 0.0f);
  f.effectiveTriangles = scene.effectiveTriangles();
  if (progress) progress->beginPhase(RenderPhase::Setup);
  std::lock_guard<std::mutex> lk(gpuMutex());
  ubr_context* ctx = gpuContext();
  FlatScene flat(scene);
  ubr_scene* built = nullptr;
  check(ctx, ubr_scene_build(ctx, &flat.desc, &built), "scene build");
  ubr_scene_info info{};
  ubr_scene_get_info(built, &info);
  std::vector<ubr_light> lights;
  const ubr_render_desc rd = toRenderDesc(scene, opt, lights);
  ubr_frame fr{};
  fr.memory = UBR_MEMORY_HOST;
  fr.color = f.color.data();
  fr.depth = f.depth.data();
  fr.view_z = f.viewZ.empty() ? nullptr : f.viewZ.data();
  const int aoDiv = opt.aoResDiv < 0 ? ss : opt.aoResDiv;
  if (opt.aoResDebug && aoDiv > 1 && opt.aoSamples > 0) {
    // coarse-AO fallback mask at the render resolution (embree_renderer.cpp:549-550)
    f.aoPatchMask.assign(nhi, 0.0f);
    fr.ao_patch_mask = f.aoPatchMask.data();
  }
  if (opt.aaMode == 1 && opt.aaDebug) {
    // refinement mask at the output resolution (embree_renderer.cpp:1539)
    f.aaMask.assign(nout, 0.0f);
    fr.aa_mask = f.aaMask.data();
  }
  if (opt.aoWriteAov) {
    // AO AOVs at the output resolution (allocateFrameBuffers neutral values;
    // renderFrame box-averages them with the colour)
    f.albedo.assign(nout * 3, 0.0f);
    f.normal.assign(nout * 3, 0.0f);
    f.bentNormal.assign(nout * 3, 0.0f);
    f.contactAo.assign(nout, 1.0f);
    f.shapeAo.assign(nout, 1.0f);
    f.avgHitDist.assign(nout, 0.0f);
    fr.albedo = f.albedo.data();
    fr.normal = f.normal.data();
    fr.bent_normal = f.bentNormal.data();
    fr.contact_ao = f.contactAo.data();
    fr.shape_ao = f.shapeAo.data();
    fr.avg_hit_dist = f.avgHitDist.data();
  }
  // The C-ABI polls a plain int between rounds; mirror the progress cancel
  // flag into it while the render runs.
  volatile int32_t cancelFlag = 0;
  std::atomic<bool> running{true};
  std::thread watcher;
  if (progress) {
    progress->beginPhase(RenderPhase::Primary, 1);
    if (progress->cancelRequested()) cancelFlag = 1;
    watcher = std::thread([&] {
      while (running.load(std::memory_order_relaxed)) {
        if (progress->cancelRequested()) cancelFlag = 1;
        std::this_thread::sleep_for(std::chrono::milliseconds(1));
      }
    });
  }
  const ubr_status st = ubr_render(ctx, built, &rd, &fr, progress ? &cancelFlag : nullptr, nullptr);
  running = false;
  if (watcher.joinable()) watcher.join();
  ubr_scene_release(built);
  check(ctx, st, "render");
  f.renderSeconds = fr.render_ms / 1e3;
  f.pt1Timing.bvhBuild = info.build_ms / 1e3;
  f.pt1Timing.primary = f.renderSeconds;
  if (opt.gi) {
    // embree_renderer.cpp:859-1123: the GI pass's split and ray counts
    f.pt1Timing.gather = (fr.gi_ms[0] + fr.gi_ms[1] + fr.gi_ms[4] + fr.gi_ms[5]) / 1e3;
    f.pt1Timing.denoise = fr.gi_ms[2] / 1e3;
    f.pt1Timing.upsample = fr.gi_ms[3] / 1e3;
    f.pt1Rays.gatherRays = fr.gi_gather_rays;
    f.pt1Rays.neeRays = fr.gi_nee_rays;
    f.pt1Rays.gbufferRays = fr.gi_gbuffer_rays;
    if (opt.pt1Denoise) f.pt1DenoiserUsed = 1;  // the a-trous (OIDN absent)
  }
  f.cancelled = st == UBR_CANCELLED;
  // pipeline.cpp:231-251: which backend ran (the a-trous, also for OIDN requests)
  if (opt.denoiser != 0) f.denoiserUsed = 1;
  if (fr.capped_rays > 0)
    logMessage(LogLevel::Warning,
               "%llu ray(s) reached the transparent-layer cap (%d); transmission past that depth was dropped",
               static_cast<unsigned long long>(fr.capped_rays), opt.maxTransparentLayers);
  if (progress && !f.cancelled) {
    progress->advance(1);
    progress->beginPhase(RenderPhase::Postprocess);
  }
  return f;
}

// Scene minus the primitives of hidden groups (umbreon.cpp:53-116 semantics).
Scene hideGroups(const Scene& s, const std::vector<uint8_t>& hide) {
  auto hidden = [&](uint16_t g) { return g < hide.size() && hide[g] != 0; };
  Scene out = s;
  out.groupBlend.clear();
  const std::size_t nt = s.mesh.triangleCount();
  std::vector<uint32_t> idx;
  std::vector<uint8_t> mat;
  std::vector<uint16_t> grp;
  for (std::size_t t = 0; t < nt; ++t) {
    if (hidden(s.mesh.groupForTri(t))) continue;
    for (int k = 0; k < 3; ++k) idx.push_back(s.mesh.cornerVertex(t * 3 + k));
    if (!s.mesh.triMaterialId.empty()) mat.push_back(s.mesh.triMaterialId[t]);
    if (!s.mesh.triGroupId.empty()) grp.push_back(s.mesh.triGroupId[t]);
  }
  if (idx.empty()) {
    out.mesh = Mesh{};
  } else {
    out.mesh.index = std::move(idx);
    out.mesh.triMaterialId = std::move(mat);
    out.mesh.triGroupId = std::move(grp);
  }
  out.spheres.clear();
  for (const Sphere& sp : s.spheres)
    if (!hidden(sp.group)) out.spheres.push_back(sp);
  out.cylinders.clear();
  for (const Cylinder& c : s.cylinders)
    if (!hidden(c.group)) out.cylinders.push_back(c);
  return out;
}

FrameResult renderImpl(const Scene& scene, const RenderOptions& opt, RenderProgress* progress) {
  rejectUnsupported(opt);
  if (scene.groupBlend.empty()) {
    FrameResult f = renderFrameGpu(scene, opt, progress);
    if (progress && !f.cancelled) progress->markDone();
    return f;
  }
  // Group-alpha: out = (1 - sum a_i) * pass(all groups hidden)
  //                  + sum a_i * pass(group i kept), blended in sRGB space.
  float sumA = 0.0f;
  uint16_t maxGroup = 0;
  for (const GroupBlend& gb : scene.groupBlend) {
    sumA += gb.alpha;
    maxGroup = std::max(maxGroup, gb.group);
  }
  std::vector<uint8_t> hideAll(static_cast<std::size_t>(maxGroup) + 1, 0);
  for (const GroupBlend& gb : scene.groupBlend) hideAll[gb.group] = 1;
  const std::uint64_t passCount = 1 + scene.groupBlend.size();
  std::uint64_t passIndex = 0;
  FrameResult carrier;
  std::vector<float> acc;
  double seconds = 0.0, bvh = 0.0;
  bool cancelled = false;
  auto pass = [&](const std::vector<uint8_t>& hide, float w) {
    if (cancelled) return;
    if (progress) progress->beginPass(passIndex, passCount);
    ++passIndex;
    FrameResult f = renderFrameGpu(hideGroups(scene, hide), opt, progress);
    cancelled = f.cancelled;
    seconds += f.renderSeconds;
    bvh += f.pt1Timing.bvhBuild;
    if (acc.empty()) acc.assign(f.color.size(), 0.0f);
    for (std::size_t p = 0; p < acc.size() / 4; ++p) {
      for (int c = 0; c < 3; ++c) acc[p * 4 + c] += w * srgbEncodeF(f.color[p * 4 + c]);
      acc[p * 4 + 3] += w * f.color[p * 4 + 3];
    }
    carrier = std::move(f);
  };
  pass(hideAll, 1.0f - sumA);
  for (const GroupBlend& gb : scene.groupBlend) {
    std::vector<uint8_t> hide = hideAll;
    hide[gb.group] = 0;
    pass(hide, gb.alpha);
  }
  for (std::size_t p = 0; p < acc.size() / 4; ++p) {
    for (int c = 0; c < 3; ++c) acc[p * 4 + c] = srgbDecodeF(std::fmax(0.0f, acc[p * 4 + c]));
    acc[p * 4 + 3] = std::fmin(1.0f, std::fmax(0.0f, acc[p * 4 + 3]));
  }
  carrier.color = std::move(acc);
  carrier.renderSeconds = seconds;
  carrier.pt1Timing.bvhBuild = bvh;
  carrier.pt1Timing.primary = seconds;
  carrier.cancelled = cancelled;
  if (progress && !cancelled) progress->markDone();
  return carrier;
}

}  // namespace

FrameResult render(const Scene& scene, const RenderOptions& opt) { return renderImpl(scene, opt, nullptr); }

FrameResult render(const Scene& scene, const RenderOptions& opt, RenderProgress& progress) {
  return renderImpl(scene, opt, &progress);
}

// ---------------------------------------------------------------------------
// async handle

struct RenderTask::Impl {
  RenderProgress progress;
  Scene scene;
  RenderOptions opt;
  FrameResult result;
  std::exception_ptr err;
  std::atomic<bool> finished{false};
  std::mutex m;
  std::condition_variable cv;
  std::thread worker;
  ~Impl() {
    if (worker.joinable()) {
      progress.requestCancel();
      worker.join();
    }
  }
};

RenderTask::RenderTask(std::unique_ptr<Impl> impl) noexcept : p_(std::move(impl)) {}
RenderTask::RenderTask(RenderTask&&) noexcept = default;
RenderTask& RenderTask::operator=(RenderTask&&) noexcept = default;
RenderTask::~RenderTask() = default;

float RenderTask::progress() const noexcept { return p_->progress.fraction(); }
RenderPhase RenderTask::phase() const noexcept { return p_->progress.phase(); }
bool RenderTask::done() const noexcept { return p_->finished.load(std::memory_order_acquire); }
void RenderTask::cancel() noexcept { p_->progress.requestCancel(); }

bool RenderTask::wait_for(std::chrono::milliseconds timeout) const {
  std::unique_lock<std::mutex> lk(p_->m);
  return p_->cv.wait_for(lk, timeout, [this] { return p_->finished.load(std::memory_order_acquire); });
}

void RenderTask::wait() const {
  std::unique_lock<std::mutex> lk(p_->m);
  p_->cv.wait(lk, [this] { return p_->finished.load(std::memory_order_acquire); });
}

FrameResult RenderTask::get() {
  if (p_->worker.joinable()) p_->worker.join();
  if (p_->err) std::rethrow_exception(p_->err);
  return std::move(p_->result);
}

RenderTask renderAsync(Scene scene, RenderOptions opt) {
  auto impl = std::make_unique<RenderTask::Impl>();
  impl->scene = std::move(scene);
  impl->opt = std::move(opt);
  RenderTask::Impl* raw = impl.get();
  impl->worker = std::thread([raw] {
    try {
      raw->result = render(raw->scene, raw->opt, raw->progress);
    } catch (...) {
      raw->err = std::current_exception();
    }
    {
      std::lock_guard<std::mutex> lk(raw->m);
      raw->finished.store(true, std::memory_order_release);
    }
    raw->cv.notify_all();
  });
  return RenderTask(std::move(impl));
}

}  // namespace umbreon

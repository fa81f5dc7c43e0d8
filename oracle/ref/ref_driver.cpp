// ref_driver.cpp -- TEST INFRASTRUCTURE: runs the REFERENCE's own
// umbreon::render (CueMol/umbreon src/umbreon, compiled unmodified against the
// Embree / oneTBB stand-ins in oracle/shim) on a scene and options given as
// this library's C-ABI descriptors, so a test can hold the oracle's
// restatement to the reference's code on the same inputs.  Built by
// oracle/build_ref.py into oracle/_ref (never shipped, never on the product
// path).
#include <cstring>
#include <vector>

#include "ubr.h"
#include "umbreon.hpp"

namespace {

umbreon::Material toMat(const ubr_material& m) {
  umbreon::Material r;
  r.ambient = m.ambient;
  r.diffuse = m.diffuse;
  r.specular = m.specular;
  r.roughness = m.roughness;
  r.brilliance = m.brilliance;
  r.phong = m.phong;
  r.phongSize = m.phong_size;
  r.metallic = m.metallic != 0;
  r.reflection = m.reflection;
  r.emission = m.emission;
  r.model = m.model == 1 ? umbreon::ShadingModel::Principled
            : m.model == 2 ? umbreon::ShadingModel::Toon
                           : umbreon::ShadingModel::Pov;
  r.pbr.metallic = m.pbr_metallic;
  r.pbr.roughness = m.pbr_roughness;
  r.pbr.specular = m.pbr_specular;
  r.pbr.anisotropy = m.pbr_anisotropy;
  r.pbr.anisotropyRotation = m.pbr_anisotropy_rotation;
  return r;
}

umbreon::Vec3 v3(const float* p) { return umbreon::Vec3{p[0], p[1], p[2]}; }

void toScene(const ubr_scene_desc& d, const ubr_render_desc& r, umbreon::Scene& s) {
  for (uint64_t v = 0; v < d.mesh_vertex_count; ++v) {
    s.mesh.positions.push_back(v3(d.mesh_positions + 3 * v));
    s.mesh.normals.push_back(d.mesh_normals ? v3(d.mesh_normals + 3 * v) : umbreon::Vec3{0, 0, 0});
    const float* c = d.mesh_colors ? d.mesh_colors + 4 * v : nullptr;
    s.mesh.colors.push_back(c ? umbreon::Vec4{c[0], c[1], c[2], c[3]} : umbreon::Vec4{0, 0, 0, 1});
  }
  if (d.mesh_index) s.mesh.index.assign(d.mesh_index, d.mesh_index + 3 * d.mesh_triangle_count);
  s.mesh.material = toMat(d.mesh_material);
  for (uint32_t i = 0; i < d.mesh_material_count && d.mesh_materials; ++i)
    s.mesh.materials.push_back(toMat(d.mesh_materials[i]));
  if (d.mesh_tri_material) s.mesh.triMaterialId.assign(d.mesh_tri_material, d.mesh_tri_material + d.mesh_triangle_count);
  if (d.mesh_tri_group) s.mesh.triGroupId.assign(d.mesh_tri_group, d.mesh_tri_group + d.mesh_triangle_count);
  for (uint64_t i = 0; i < d.sphere_count; ++i) {
    umbreon::Sphere sp;
    sp.center = v3(d.sphere_center_radius + 4 * i);
    sp.radius = d.sphere_center_radius[4 * i + 3];
    const float* c = d.sphere_color + 4 * i;
    sp.color = umbreon::Vec4{c[0], c[1], c[2], c[3]};
    sp.material = toMat(d.sphere_material[i]);
    sp.group = d.sphere_group ? d.sphere_group[i] : 0;
    sp.fromEdgeMacro = d.sphere_from_edge && d.sphere_from_edge[i];
    s.spheres.push_back(sp);
  }
  for (uint64_t i = 0; i < d.cylinder_count; ++i) {
    umbreon::Cylinder cy;
    cy.p0 = v3(d.cyl_p0 + 3 * i);
    cy.p1 = v3(d.cyl_p1 + 3 * i);
    cy.radius = d.cyl_radius[i];
    const float* c = d.cyl_color + 4 * i;
    cy.color = umbreon::Vec4{c[0], c[1], c[2], c[3]};
    cy.material = toMat(d.cyl_material[i]);
    cy.group = d.cyl_group ? d.cyl_group[i] : 0;
    cy.opacity1 = d.cyl_opacity1 ? d.cyl_opacity1[i] : -1.0f;
    cy.open = d.cyl_open && d.cyl_open[i];
    cy.fromEdgeMacro = d.cyl_from_edge && d.cyl_from_edge[i];
    s.cylinders.push_back(cy);
  }
  for (uint64_t i = 0; i < d.instance_count; ++i) s.instanceOffsets.push_back(v3(d.instance_offsets + 3 * i));
  s.camera.position = v3(r.cam_position);
  s.camera.direction = v3(r.cam_direction);
  s.camera.up = v3(r.cam_up);
  s.camera.fovy = r.cam_fovy;
  s.camera.orthographic = r.cam_orthographic != 0;
  s.camera.height = r.cam_height;
  for (uint32_t i = 0; i < r.light_count; ++i) {
    umbreon::DistantLight l;
    l.direction = v3(r.lights[i].direction);
    l.color = v3(r.lights[i].color);
    l.intensity = r.lights[i].intensity;
    l.castsHighlight = r.lights[i].casts_highlight != 0;
    l.angularRadius = r.lights[i].angular_radius;
    s.lights.push_back(l);
  }
  s.ambientColor = v3(r.ambient_color);
  s.background = v3(r.background);
  s.fog.enabled = r.fog_enabled != 0;
  s.fog.color = v3(r.fog_color);
  s.fog.start = r.fog_start;
  s.fog.end = r.fog_end;
  s.clipNear = r.clip_near;
  s.clipFar = r.clip_far;
  s.assumedGamma = r.assumed_gamma;
}

void toOptions(const ubr_render_desc& d, umbreon::RenderOptions& o) {
  o.width = d.width;
  o.height = d.height;
  o.supersample = d.supersample;
  o.aoSamples = d.ao_samples;
  o.aoDistance = d.ao_distance;
  o.aoIntensity = d.ao_intensity;
  o.aoFalloffPower = d.ao_falloff_power;
  o.aoMultiScale = d.ao_multiscale != 0;
  o.aoBentNormal = d.ao_bent_normal != 0;
  for (int k = 0; k < 3; ++k) {
    o.aoSkyColor[k] = d.ao_sky_color[k];
    o.aoGroundColor[k] = d.ao_ground_color[k];
    o.aoUp[k] = d.ao_up[k];
  }
  o.aoUseCameraUp = d.ao_use_camera_up != 0;
  o.aoMultibounce = d.ao_multibounce != 0;
  o.aoLowDiscrepancy = d.ao_low_discrepancy != 0;
  o.aoDiffuseFactor = d.ao_diffuse_factor;
  o.shadows = d.shadows != 0;
  o.shadowSamples = d.shadow_samples;
  o.lightRadius = d.light_radius_deg;
  o.envLights = d.env_lights;
  o.envIntensity = d.env_intensity;
  o.envKeyScale = d.env_key_scale;
  o.envAngle = d.env_angle;
  o.specularScale = d.specular_scale;
  o.transparency = d.transparency != 0;
  o.transparentBackground = d.transparent_background != 0;
  o.maxTransparentLayers = d.max_transparent_layers;
  o.giIntegrator = d.gi_integrator;
  o.aoWriteAov = d.ao_write_aov != 0;
  o.aaMode = d.aa_mode;
  o.aaThreshold = d.aa_threshold;
  o.aaDepth = d.aa_depth;
  o.aoResDiv = d.ao_res_div;
  o.denoiser = d.denoiser;
  o.denoiseIters = d.denoise_iters;
  o.denoiseSigmaZ = d.denoise_sigma_z;
  o.denoiseSigmaN = d.denoise_sigma_n;
  o.denoiseSigmaL = d.denoise_sigma_l;
  o.denoiseDemodulateAlbedo = d.denoise_demodulate_albedo != 0;
  o.gi = d.gi != 0;
  if (o.gi) {
    o.pt1Spp = d.pt1_spp;
    o.giBounces = d.gi_bounces;
    o.giMaxDistance = d.gi_max_distance;
    o.giIntensity = d.gi_intensity;
    o.giEnvIntensity = d.gi_env_intensity;
    o.pt1Seed = d.pt1_seed;
    o.pt1SkyMode = d.pt1_sky_mode;
    for (int k = 0; k < 3; ++k) o.pt1SkyRadiance[k] = d.pt1_sky_radiance[k];
    o.pt1Ld = d.pt1_ld != 0;
    o.pt1Clamp = d.pt1_clamp;
    o.pt1GatherDiv = d.pt1_gather_div;
    o.pt1HalfRes = d.pt1_half_res != 0;
    o.pt1Denoise = d.pt1_denoise != 0;
    o.pt1UpsampleNormalPow = d.pt1_upsample_normal_pow;
    o.pt1UpsampleDepthScale = d.pt1_upsample_depth_scale;
    o.pt1EdgePatch = d.pt1_edge_patch != 0;
    o.pt1EdgePatchSppMul = d.pt1_edge_patch_spp_mul;
    o.pt1EdgePatchThresh = d.pt1_edge_patch_thresh;
    o.pt2Pattern = d.pt2_pattern;
    o.pt2Emissive = d.pt2_emissive != 0;
    o.pt2Rounds = d.pt2_rounds;
    o.pt2Radius = d.pt2_radius;
    o.pt2Unbiased = d.pt2_unbiased != 0;
    o.pt2MCap = d.pt2_m_cap;
    o.pt2WClamp = d.pt2_w_clamp;
    o.pt2Adaptive = d.pt2_adaptive != 0;
    o.pt2AdaptiveThresh = d.pt2_adaptive_thresh;
    o.pt2AdaptiveMul = d.pt2_adaptive_mul;
    o.pt2EmissiveNee = d.pt2_emissive_nee != 0;
    o.pt2Reflect = d.pt2_reflect != 0;
    o.pt2Glossy = d.pt2_glossy != 0;
    o.pt2GlossySpp = d.pt2_glossy_spp;
    o.pt2GlossyDenoise = d.pt2_glossy_denoise != 0;
  }
}

}  // namespace

extern "C" {

// umbreon::render of the reference on the given scene and options; writes
// the frame's colour (W*H*4) and, when non-null, depth and view z (hi-res
// planes as renderFrame leaves them).  0 = ok, 1 = the reference threw.
int ref_render(const ubr_scene_desc* sd, const ubr_render_desc* rd, float* color, float* depth, float* viewZ,
               double* renderSeconds) {
  try {
    umbreon::Scene s;
    toScene(*sd, *rd, s);
    umbreon::RenderOptions o;
    toOptions(*rd, o);
    const umbreon::FrameResult f = umbreon::render(s, o);
    if (color) std::memcpy(color, f.color.data(), f.color.size() * sizeof(float));
    if (depth && !f.depth.empty()) std::memcpy(depth, f.depth.data(), f.depth.size() * sizeof(float));
    if (viewZ && !f.viewZ.empty()) std::memcpy(viewZ, f.viewZ.data(), f.viewZ.size() * sizeof(float));
    if (renderSeconds) *renderSeconds = f.renderSeconds;
    return 0;
  } catch (...) {
    return 1;
  }
}

}  // extern "C"

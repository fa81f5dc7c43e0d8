// oracle_render.cpp -- TEST INFRASTRUCTURE (the oracle), never shipped.
//
// Plain C++ restatement, on the CPU, of umbreon's ray-cast + shade path, used
// only by tests/, by __graft_entry__.smoke() and by bench.py's CPU baseline as
// the checker.  Every function names the reference lines it follows (paths
// inside the CueMol/umbreon project).  Float expressions keep the reference's
// operation order so that, built with -ffp-contract=off, results match the
// reference's own code on the same intersections bit for bit.
//
// Scope: the POV and Principled (direct pass) shading models, adaptive AA and
// coarse-grid AO; the GI and edge branches are outside the path and rejected
// or ignored as documented at each site.
#include <atomic>
#include <chrono>
#include <cmath>
#include <functional>
#include <cstdint>
#include <cstring>
#include <map>
#include <array>
#include <thread>
#include <vector>

#include "oracle_geom.hpp"
#include "ubr.h"

namespace oracle {
namespace {

constexpr float kInf = std::numeric_limits<float>::infinity();

// scene.hpp:44-49 safeNormalize(a)
inline V3 safeNormalize(V3 a) {
  float s = 1.0f / std::sqrt(std::fmax(dot(a, a), 0x1.0p-126f));
  return a * s;
}
// scene.hpp:53-57 safeNormalize(a, fallback)
inline V3 safeNormalize(V3 a, V3 fb) {
  float d = dot(a, a);
  if (d < 1.0e-18f) return fb;
  return a * (1.0f / std::sqrt(d));
}
struct Frame { V3 t, b, n; };
// scene.hpp:69-76 frameFromNormal
inline Frame frameFromNormal(V3 n) {
  const V3 seed0{0.0f, n.z, -n.y};
  const V3 seed1{-n.z, 0.0f, n.x};
  const V3 t = safeNormalize(std::fabs(n.x) < std::fabs(n.y) ? seed0 : seed1, V3{1.0f, 0.0f, 0.0f});
  const V3 b = cross(n, t);
  return {t, b, n};
}
inline float radians(float deg) { return deg * 0.01745329252f; }  // scene.hpp:78

struct Mat {  // umbreon::Material (scene.hpp:130-175) as the shaders read it
  float ambient, diffuse, specular, roughness, brilliance, phong, phongSize;
  bool metallic;
  float reflection, emission;
  uint32_t model;  // 0 Pov, 1 Principled, 2 Toon (shaded as Pov)
  float pbrMetallic, pbrRoughness, pbrSpecular, pbrAnisotropy, pbrAnisotropyRotation;
};
Mat fromAbi(const ubr_material& m) {
  return {m.ambient, m.diffuse, m.specular, m.roughness, m.brilliance, m.phong,
          m.phong_size, m.metallic != 0, m.reflection, m.emission, m.model,
          m.pbr_metallic, m.pbr_roughness, m.pbr_specular, m.pbr_anisotropy, m.pbr_anisotropy_rotation};
}

struct Light {  // secondary_rays.hpp:26-31
  V3 L, color;
  bool highlight = true;
  float radius = 0.0f;
};

// Scene tables in primID order (scene_build.hpp:63-118).
struct Scene {
  GeomSet geo;
  Bvh bvh;
  // mesh (scene_build.cpp:16-88): attributes per baked vertex
  std::vector<float> nrm, col;
  size_t baseTri = 0;
  uint32_t baseSpheres = 0;      // Scene::spheres.size() (edge materialId block)
  std::vector<Mat> meshMats;     // Mesh::materials
  Mat meshMat{};
  std::vector<uint8_t> triMat;   // per base triangle
  std::vector<uint16_t> triGroup;
  // per kind side tables, index = kind (1..3), element = primID
  std::vector<float> color[4];   // 4 per prim
  std::vector<Mat> mat[4];
  std::vector<uint16_t> group[4];
  std::vector<uint8_t> fromEdge[4];
  std::vector<float> opacity1[4];
  // per-segment unit axis of cylinders (curve_build.cpp:163-167, 243-245),
  // built only when an anisotropic principled cylinder exists
  std::vector<V3> axis[4];
  // pt2 emissive primitives sampled as lights (pt2_emissive.hpp:37-97):
  // triangles first, then CSG records (sphere, cylinder side, cylinder cap)
  struct EmitTri { V3 p0, p1, p2, e0, e1, e2, ng; float area; };
  struct EmitCsg { int kind; V3 p0, axis, Le; float len, radius, area; };  // kind 1 sphere 2 side 3 cap
  std::vector<EmitTri> emTris;
  std::vector<EmitCsg> emCsg;
  std::vector<float> emCdf, emPdf;
  std::vector<uint32_t> emTriIndex, emSphereIndex;
  std::vector<std::array<uint32_t, 3>> emCylIndex;  // side, cap0, cap1 per capped-cylinder primID
  bool emEmpty() const { return emTris.empty() && emCsg.empty(); }
};

// pt2_emissive.hpp:104-277 pt2BuildEmissiveLights: the base mesh triangles
// whose material emits (un-offset corners), then the real emissive spheres
// and capped cylinders in primID order (instance offsets outer), one
// power-weighted CDF (area x luminance) accumulated in double.
void buildEmitters(const ubr_scene_desc& d, const std::vector<V3>& offs, Scene& s) {
  const float kPi = 3.14159265358979323846f;
  auto lum = [](const V3& c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; };
  const size_t nt = d.mesh_vertex_count >= 3 ? d.mesh_triangle_count : 0;
  bool meshEm = d.mesh_material.emission > 0.0f;
  for (uint32_t i = 0; i < d.mesh_material_count && d.mesh_materials; ++i)
    meshEm = meshEm || d.mesh_materials[i].emission > 0.0f;
  bool csgEm = false;
  for (size_t i = 0; i < d.sphere_count; ++i)
    csgEm = csgEm || (!(d.sphere_from_edge && d.sphere_from_edge[i]) && d.sphere_material[i].emission > 0.0f &&
                      d.sphere_center_radius[4 * i + 3] > 0.0f);
  for (size_t i = 0; i < d.cylinder_count; ++i)
    csgEm = csgEm || (!(d.cyl_from_edge && d.cyl_from_edge[i]) && !(d.cyl_open && d.cyl_open[i]) &&
                      d.cyl_material[i].emission > 0.0f && d.cyl_radius[i] > 0.0f);
  if (!(meshEm && nt > 0) && !csgEm) return;
  std::vector<float> power;
  if (meshEm && nt > 0) {
    s.emTriIndex.assign(nt, 0xFFFFFFFFu);
    for (size_t t = 0; t < nt; ++t) {
      const ubr_material& mm = d.mesh_tri_material ? d.mesh_materials[d.mesh_tri_material[t]] : d.mesh_material;
      if (mm.emission <= 0.0f) continue;
      Scene::EmitTri et;
      V3* P[3] = {&et.p0, &et.p1, &et.p2};
      V3* E[3] = {&et.e0, &et.e1, &et.e2};
      for (int k = 0; k < 3; ++k) {
        const uint32_t v = d.mesh_index ? d.mesh_index[3 * t + k] : static_cast<uint32_t>(3 * t + k);
        *P[k] = V3{d.mesh_positions[3 * v], d.mesh_positions[3 * v + 1], d.mesh_positions[3 * v + 2]};
        const float* cc = d.mesh_colors ? d.mesh_colors + 4 * size_t(v) : nullptr;
        *E[k] = cc ? V3{mm.emission * cc[0], mm.emission * cc[1], mm.emission * cc[2]} : V3{0.0f, 0.0f, 0.0f};
      }
      const V3 a{et.p1.x - et.p0.x, et.p1.y - et.p0.y, et.p1.z - et.p0.z};
      const V3 b{et.p2.x - et.p0.x, et.p2.y - et.p0.y, et.p2.z - et.p0.z};
      const V3 cr{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
      const float len = std::sqrt(dot(cr, cr));
      if (len <= 0.0f) continue;
      et.area = 0.5f * len;
      et.ng = V3{cr.x / len, cr.y / len, cr.z / len};
      const V3 avg{(et.e0.x + et.e1.x + et.e2.x) / 3.0f, (et.e0.y + et.e1.y + et.e2.y) / 3.0f,
                   (et.e0.z + et.e1.z + et.e2.z) / 3.0f};
      const float pw = et.area * lum(avg);
      if (pw <= 0.0f) continue;
      s.emTriIndex[t] = static_cast<uint32_t>(s.emTris.size());
      s.emTris.push_back(et);
      power.push_back(pw);
    }
    if (s.emTris.empty()) s.emTriIndex.clear();
  }
  if (csgEm) {
    s.emSphereIndex.assign(d.sphere_count * offs.size(), 0xFFFFFFFFu);
    uint32_t prim = 0;
    for (const V3& off : offs)
      for (size_t i = 0; i < d.sphere_count; ++i, ++prim) {
        const ubr_material& m = d.sphere_material[i];
        const float r = d.sphere_center_radius[4 * i + 3];
        if ((d.sphere_from_edge && d.sphere_from_edge[i]) || !(m.emission > 0.0f) || !(r > 0.0f)) continue;
        Scene::EmitCsg ec{};
        ec.kind = 1;
        ec.p0 = V3{d.sphere_center_radius[4 * i] + off.x, d.sphere_center_radius[4 * i + 1] + off.y,
                   d.sphere_center_radius[4 * i + 2] + off.z};
        ec.axis = V3{0.0f, 0.0f, 1.0f};
        ec.radius = r;
        ec.area = 4.0f * kPi * r * r;
        ec.Le = V3{m.emission * d.sphere_color[4 * i], m.emission * d.sphere_color[4 * i + 1],
                   m.emission * d.sphere_color[4 * i + 2]};
        const float pw = ec.area * lum(ec.Le);
        if (!(pw > 0.0f)) continue;
        s.emSphereIndex[prim] = static_cast<uint32_t>(s.emCsg.size());
        s.emCsg.push_back(ec);
        power.push_back(pw);
      }
    std::vector<size_t> capIdx;
    for (size_t i = 0; i < d.cylinder_count; ++i)
      if (!(d.cyl_open && d.cyl_open[i])) capIdx.push_back(i);
    s.emCylIndex.assign(capIdx.size() * offs.size(), {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu});
    prim = 0;
    for (const V3& off : offs)
      for (size_t i : capIdx) {
        const uint32_t me = prim++;
        const ubr_material& m = d.cyl_material[i];
        const float r = d.cyl_radius[i];
        if ((d.cyl_from_edge && d.cyl_from_edge[i]) || !(m.emission > 0.0f) || !(r > 0.0f)) continue;
        const V3 p0{d.cyl_p0[3 * i] + off.x, d.cyl_p0[3 * i + 1] + off.y, d.cyl_p0[3 * i + 2] + off.z};
        const V3 p1{d.cyl_p1[3 * i] + off.x, d.cyl_p1[3 * i + 1] + off.y, d.cyl_p1[3 * i + 2] + off.z};
        const V3 dd{p1.x - p0.x, p1.y - p0.y, p1.z - p0.z};
        const float len = std::sqrt(dot(dd, dd));
        if (!(len > 0.0f)) continue;
        Scene::EmitCsg ec{};
        ec.axis = V3{dd.x / len, dd.y / len, dd.z / len};
        ec.radius = r;
        ec.Le = V3{m.emission * d.cyl_color[4 * i], m.emission * d.cyl_color[4 * i + 1],
                   m.emission * d.cyl_color[4 * i + 2]};
        const float l = lum(ec.Le);
        auto& ref = s.emCylIndex[me];
        ec.kind = 2;
        ec.p0 = p0;
        ec.len = len;
        ec.area = 2.0f * kPi * r * len;
        if (ec.area * l > 0.0f) {
          ref[0] = static_cast<uint32_t>(s.emCsg.size());
          s.emCsg.push_back(ec);
          power.push_back(ec.area * l);
        }
        ec.kind = 3;
        ec.len = 0.0f;
        ec.area = kPi * r * r;
        if (ec.area * l > 0.0f) {
          ec.p0 = p0;
          ref[1] = static_cast<uint32_t>(s.emCsg.size());
          s.emCsg.push_back(ec);
          power.push_back(ec.area * l);
          ec.p0 = p1;
          ref[2] = static_cast<uint32_t>(s.emCsg.size());
          s.emCsg.push_back(ec);
          power.push_back(ec.area * l);
        }
      }
    if (s.emCsg.empty()) {
      s.emSphereIndex.clear();
      s.emCylIndex.clear();
    }
  }
  if (s.emEmpty()) {
    s.emTriIndex.clear();
    return;
  }
  double total = 0.0;
  for (float pw : power) total += pw;
  double acc = 0.0;
  for (float pw : power) {
    acc += pw;
    s.emCdf.push_back(static_cast<float>(acc / total));
    s.emPdf.push_back(static_cast<float>(pw / total));
  }
  s.emCdf.back() = 1.0f;
}

// render/curve_build.cpp:41-267 buildCylinderGeometry (open chains + capped)
void buildCylinders(const ubr_scene_desc& d, const std::vector<V3>& offs, Scene& s) {
  const size_t n = d.cylinder_count;
  if (n == 0) return;
  std::vector<int> openIdx, capIdx;
  for (size_t i = 0; i < n; ++i) {
    if (d.cyl_open && d.cyl_open[i]) openIdx.push_back(static_cast<int>(i));
    else capIdx.push_back(static_cast<int>(i));
  }
  auto P0 = [&](int i) { return V3(d.cyl_p0[3 * i], d.cyl_p0[3 * i + 1], d.cyl_p0[3 * i + 2]); };
  auto P1 = [&](int i) { return V3(d.cyl_p1[3 * i], d.cyl_p1[3 * i + 1], d.cyl_p1[3 * i + 2]); };
  auto op1 = [&](int i) { return d.cyl_opacity1 ? d.cyl_opacity1[i] : -1.0f; };
  auto grp = [&](int i) { return d.cyl_group ? d.cyl_group[i] : uint16_t(0); };
  bool axisTables = false;
  for (size_t i = 0; i < n && !axisTables; ++i)
    axisTables = d.cyl_material[i].model == 1 && d.cyl_material[i].pbr_anisotropy != 0.0f;
  auto pushSide = [&](int kind, int i) {
    for (int k = 0; k < 4; ++k) s.color[kind].push_back(d.cyl_color[4 * i + k]);
    s.mat[kind].push_back(fromAbi(d.cyl_material[i]));
    s.group[kind].push_back(grp(i));
    s.opacity1[kind].push_back(op1(i));
    s.fromEdge[kind].push_back(d.cyl_from_edge && d.cyl_from_edge[i] ? 1 : 0);
  };
  if (!openIdx.empty()) {
    const size_t no = openIdx.size();
    const float eps = 1.0e-4f;  // curve_build.cpp:88
    auto keyOf = [&](const V3& p) {
      return std::array<long long, 3>{std::llround(p.x / eps), std::llround(p.y / eps),
                                      std::llround(p.z / eps)};
    };
    for (const V3& off : offs) {
      std::vector<V3> a0(no), a1(no);
      for (size_t i = 0; i < no; ++i) {
        a0[i] = P0(openIdx[i]) + off;
        a1[i] = P1(openIdx[i]) + off;
      }
      std::map<std::array<long long, 3>, std::vector<std::pair<int, int>>> inc;
      for (int i = 0; i < static_cast<int>(no); ++i) {
        inc[keyOf(a0[i])].push_back({i, 0});
        inc[keyOf(a1[i])].push_back({i, 1});
      }
      auto compatible = [&](int a, int b) {
        return grp(openIdx[a]) == grp(openIdx[b]) &&
               (op1(openIdx[a]) < 0.0f) == (op1(openIdx[b]) < 0.0f);
      };
      std::vector<int> next(no, -1), prev(no, -1);
      for (int sg = 0; sg < static_cast<int>(no); ++sg) {
        const auto& ends = inc[keyOf(a1[sg])];
        if (ends.size() != 2) continue;
        int t = -1;
        for (const auto& e : ends)
          if (e.first != sg) t = (e.second == 0) ? e.first : -1;
        if (t >= 0 && t != sg && compatible(sg, t)) next[sg] = t;
      }
      for (int sg = 0; sg < static_cast<int>(no); ++sg)
        if (next[sg] >= 0) prev[next[sg]] = sg;
      std::vector<char> visited(no, 0);
      auto emitChain = [&](int start) {
        std::vector<int> chain;
        for (int sg = start; sg >= 0 && !visited[sg]; sg = next[sg]) {
          visited[sg] = 1;
          chain.push_back(sg);
        }
        const uint32_t base = static_cast<uint32_t>(s.geo.rcV.size() / 4);
        auto pushV = [&](const V3& p, float r) {
          s.geo.rcV.push_back(p.x); s.geo.rcV.push_back(p.y);
          s.geo.rcV.push_back(p.z); s.geo.rcV.push_back(r);
        };
        pushV(a0[chain[0]], d.cyl_radius[openIdx[chain[0]]]);
        for (int cs : chain) pushV(a1[cs], d.cyl_radius[openIdx[cs]]);
        const int nc = static_cast<int>(chain.size());
        for (int j = 0; j < nc; ++j) {
          s.geo.rcIdx.push_back(base + static_cast<uint32_t>(j));
          uint8_t fl = 0;
          if (j > 0) fl |= 1u;
          if (j < nc - 1) fl |= 2u;
          s.geo.rcFlags.push_back(fl);
          pushSide(kRound, openIdx[chain[j]]);
          if (axisTables) s.axis[kRound].push_back(safeNormalize(a1[chain[j]] - a0[chain[j]]));
        }
      };
      for (int sg = 0; sg < static_cast<int>(no); ++sg)
        if (prev[sg] < 0 && !visited[sg]) emitChain(sg);
      for (int sg = 0; sg < static_cast<int>(no); ++sg)
        if (!visited[sg]) emitChain(sg);
    }
  }
  if (!capIdx.empty()) {
    for (const V3& off : offs) {
      for (int idx : capIdx) {
        const uint32_t base = static_cast<uint32_t>(s.geo.ccV.size() / 4);
        const V3 a = P0(idx) + off, b = P1(idx) + off;
        const float r = d.cyl_radius[idx];
        for (float f : {a.x, a.y, a.z, r, b.x, b.y, b.z, r}) s.geo.ccV.push_back(f);
        s.geo.ccIdx.push_back(base);
        pushSide(kCone, idx);
        if (axisTables) s.axis[kCone].push_back(safeNormalize(P1(idx) - P0(idx)));
      }
    }
  }
}

// render/scene_build.cpp:133-170 buildEmbreeScene (+ :16-129)
Scene* buildScene(const ubr_scene_desc& d) {
  Scene* s = new Scene();
  std::vector<V3> offs;
  for (size_t i = 0; i < d.instance_count; ++i)
    offs.push_back({d.instance_offsets[3 * i], d.instance_offsets[3 * i + 1], d.instance_offsets[3 * i + 2]});
  if (offs.empty()) offs.push_back(V3());
  // mesh
  const size_t baseV = d.mesh_vertex_count;
  const size_t baseT = d.mesh_triangle_count;
  uint32_t nextGeom = 0;
  if (baseV >= 3 && baseT > 0) {
    s->geo.geomID[kMesh] = nextGeom++;
    for (size_t c = 0; c < offs.size(); ++c) {
      for (size_t v = 0; v < baseV; ++v) {
        const V3 p = V3(d.mesh_positions[3 * v], d.mesh_positions[3 * v + 1], d.mesh_positions[3 * v + 2]) + offs[c];
        s->geo.triPos.push_back(p.x); s->geo.triPos.push_back(p.y); s->geo.triPos.push_back(p.z);
        for (int k = 0; k < 3; ++k) s->nrm.push_back(d.mesh_normals ? d.mesh_normals[3 * v + k] : 0.0f);
        for (int k = 0; k < 4; ++k) s->col.push_back(d.mesh_colors ? d.mesh_colors[4 * v + k] : (k == 3 ? 1.0f : 0.0f));
      }
    }
    for (size_t c = 0; c < offs.size(); ++c)
      for (size_t t = 0; t < baseT; ++t)
        for (int k = 0; k < 3; ++k) {
          const size_t corner = t * 3 + k;
          const uint32_t cv = d.mesh_index ? d.mesh_index[corner] : static_cast<uint32_t>(corner);
          s->geo.triIdx.push_back(static_cast<uint32_t>(c * baseV + cv));
        }
    s->baseTri = baseT;
    s->meshMat = fromAbi(d.mesh_material);
    for (uint32_t i = 0; i < d.mesh_material_count; ++i) {
      s->meshMats.push_back(fromAbi(d.mesh_materials[i]));
    }
    if (d.mesh_tri_material) s->triMat.assign(d.mesh_tri_material, d.mesh_tri_material + baseT);
    if (d.mesh_tri_group) s->triGroup.assign(d.mesh_tri_group, d.mesh_tri_group + baseT);
  }
  // spheres (scene_build.cpp:91-129)
  s->baseSpheres = static_cast<uint32_t>(d.sphere_count);
  if (d.sphere_count > 0) {
    s->geo.geomID[kSphere] = nextGeom++;
    for (const V3& off : offs)
      for (size_t i = 0; i < d.sphere_count; ++i) {
        const float* c = d.sphere_center_radius + 4 * i;
        s->geo.sph.push_back(c[0] + off.x); s->geo.sph.push_back(c[1] + off.y);
        s->geo.sph.push_back(c[2] + off.z); s->geo.sph.push_back(c[3]);
        for (int k = 0; k < 4; ++k) s->color[kSphere].push_back(d.sphere_color[4 * i + k]);
        s->mat[kSphere].push_back(fromAbi(d.sphere_material[i]));
        s->group[kSphere].push_back(d.sphere_group ? d.sphere_group[i] : 0);
        s->fromEdge[kSphere].push_back(d.sphere_from_edge && d.sphere_from_edge[i] ? 1 : 0);
      }
  }
  buildCylinders(d, offs, *s);
  buildEmitters(d, offs, *s);
  if (!s->geo.rcIdx.empty()) s->geo.geomID[kRound] = nextGeom++;
  if (!s->geo.ccIdx.empty()) s->geo.geomID[kCone] = nextGeom++;
  s->bvh.build(&s->geo);
  return s;
}

int kindOfGeom(const Scene& s, uint32_t geomID) {
  for (int k = 0; k < 4; ++k) if (s.geo.geomID[k] == geomID) return k;
  return -1;
}

// ---------------------------------------------------------------------------
// shading math

// shading.hpp:27-30 faceForward
inline V3 faceForward(V3 n, V3 rayDir) { return (dot(n, rayDir) > 0.0f) ? V3{-n.x, -n.y, -n.z} : n; }
// shading.hpp:34-41 blinnExp
inline float blinnExp(float roughness) {
  float r = roughness;
  if (r < 1e-6f) r = 1e-6f;
  float e = 1.0f / r;
  if (e < 1.0f) e = 1.0f;
  if (e > 1.0e6f) e = 1.0e6f;
  return e;
}
// secondary_rays.hpp:38-46 selfIntersectEps
inline float selfIntersectEps(const V3& P, const V3& dir, float t) {
  const float dirMax = std::fmax(std::fabs(dir.x), std::fmax(std::fabs(dir.y), std::fabs(dir.z)));
  const float epsScale = std::fmax(std::fmax(std::fabs(P.x), std::fabs(P.y)), std::fmax(std::fabs(P.z), dirMax * t));
  return epsScale * 0x1.0fp-21f;
}
// secondary_rays.hpp:51-58 tea2
inline void tea2(uint32_t& v0, uint32_t& v1) {
  uint32_t sum = 0;
  for (int i = 0; i < 8; ++i) {
    sum += 0x9E3779B9u;
    v0 += ((v1 << 4) + 0xA341316Cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xC8013EA4u);
    v1 += ((v0 << 4) + 0xAD90777Du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7E95761Eu);
  }
}
inline float u32ToUnorm(uint32_t u) { return (u >> 8) * 0x1.0p-24f; }  // :61
// secondary_rays.hpp:66-73
inline V3 cosineSampleHemisphere(float u1, float u2, const Frame& f) {
  const float phi = 6.2831853072f * u1;
  const float r = std::sqrt(u2);
  const float z = std::sqrt(std::fmax(0.0f, 1.0f - u2));
  const float x = std::cos(phi) * r;
  const float y = std::sin(phi) * r;
  return f.t * x + f.b * y + f.n * z;
}
// Occlusion-type rays (AO, shadow, AO nearest-hit) traced by this thread:
// every call below is one traced ray, the same unit the GPU's occlusion
// kernel counts (rays it hands to a traversal).
thread_local uint64_t tOccRays = 0;

// secondary_rays.hpp:79-97 occluded
inline bool occludedQ(const Scene& s, const V3& P, const V3& dir, float tnear, float tfar) {
  ++tOccRays;
  Ray r;
  r.org = P; r.dir = dir; r.tnear = tnear; r.tfar = tfar;
  return s.bvh.occluded(r);
}
// secondary_rays.hpp:102-109
inline V3 sampleLightDir(const Light& l, float u1, float u2) {
  if (l.radius <= 0.0f) return l.L;
  const Frame f = frameFromNormal(l.L);
  const float phi = 6.2831853072f * u1;
  const float rr = std::tan(l.radius) * std::sqrt(u2);
  const V3 d = f.n + f.t * (rr * std::cos(phi)) + f.b * (rr * std::sin(phi));
  return safeNormalize(d, l.L);
}
// secondary_rays.hpp:118-134
inline float computeShadow(const Scene& s, const V3& P, const V3& Ng, const V3& N, float eps,
                           const Light& l, int shadowSamples, uint32_t& s0, uint32_t& s1) {
  V3 ng = (dot(Ng, N) < 0.0f) ? V3{-Ng.x, -Ng.y, -Ng.z} : Ng;
  ng = safeNormalize(ng, N);
  const V3 O = P + ng * eps;
  if (shadowSamples <= 1 || l.radius <= 0.0f) return occludedQ(s, O, l.L, eps, kInf) ? 0.0f : 1.0f;
  int hits = 0;
  for (int i = 0; i < shadowSamples; ++i) {
    tea2(s0, s1);
    const V3 dir = sampleLightDir(l, u32ToUnorm(s0), u32ToUnorm(s1));
    if (occludedQ(s, O, dir, eps, kInf)) ++hits;
  }
  return 1.0f - static_cast<float>(hits) / static_cast<float>(shadowSamples);
}
// ambient_occlusion.hpp:33-57 computeAO (legacy binary)
inline float computeAO(const Scene& s, const V3& P, const V3& Ng, const V3& Ns, float eps, int nSamples,
                       float aoRadius, uint32_t px, uint32_t py, int wHi) {
  if (nSamples <= 0) return 1.0f;
  const Frame f = frameFromNormal(Ns);
  V3 ng = (dot(Ng, Ns) < 0.0f) ? V3{-Ng.x, -Ng.y, -Ng.z} : Ng;
  ng = safeNormalize(ng, Ns);
  const V3 O = P + ng * eps;
  const uint32_t base = px + py * static_cast<uint32_t>(wHi);
  int hits = 0;
  for (int i = 0; i < nSamples; ++i) {
    uint32_t s0 = base, s1 = static_cast<uint32_t>(i);
    tea2(s0, s1);
    const V3 dir = cosineSampleHemisphere(u32ToUnorm(s0), u32ToUnorm(s1), f);
    if (dot(dir, Ns) < 0.01f) { ++hits; continue; }
    if (occludedQ(s, O, dir, eps, aoRadius)) ++hits;
  }
  return 1.0f - static_cast<float>(hits) / static_cast<float>(nSamples);
}
// ambient_occlusion.hpp:72-94 intersectNearest
inline float intersectNearest(const Scene& s, const V3& O, const V3& dir, float tnear, float tfar) {
  ++tOccRays;
  Ray r;
  r.org = O; r.dir = dir; r.tnear = tnear; r.tfar = tfar;
  Hit h;
  return s.bvh.closest(r, h) ? h.t : kInf;
}
// ambient_occlusion.hpp:98-105
inline float radicalInverse2(uint32_t bits) {
  bits = (bits << 16) | (bits >> 16);
  bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
  bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
  bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
  bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
  return static_cast<float>(bits) * 0x1.0p-32f;
}
// ambient_occlusion.hpp:112-127
inline void aoSample2d(bool ld, uint32_t base, int i, int n, float cpx, float cpy, float& u1, float& u2) {
  if (ld) {
    u1 = static_cast<float>(i) / static_cast<float>(n) + cpx;
    u2 = radicalInverse2(static_cast<uint32_t>(i)) + cpy;
    if (u1 >= 1.0f) u1 -= 1.0f;
    if (u2 >= 1.0f) u2 -= 1.0f;
  } else {
    uint32_t s0 = base, s1 = static_cast<uint32_t>(i);
    tea2(s0, s1);
    u1 = u32ToUnorm(s0);
    u2 = u32ToUnorm(s1);
  }
}
// ambient_occlusion.hpp:134-139
inline float aoMultibounce(float ao, float albedo) {
  const float a = 2.0404f * albedo - 0.3324f;
  const float b = -4.7951f * albedo + 0.6417f;
  const float c = 2.7552f * albedo + 0.6903f;
  return std::fmax(ao, ((ao * a + b) * ao + c) * ao);
}
struct AOResult { float contact = 1.0f, shape = 1.0f, openness = 1.0f; V3 bent; float avgHitDist = 0.0f; };
// ambient_occlusion.hpp:171-267 computeAOQuality
inline AOResult computeAOQuality(const Scene& s, const V3& P, const V3& Ng, const V3& Ns, float eps,
                                 int nSamples, float R, float power, bool multiScale, bool ld,
                                 uint32_t px, uint32_t py, int wHi) {
  AOResult r;
  if (nSamples <= 0) { r.bent = Ns; return r; }
  const Frame f = frameFromNormal(Ns);
  V3 ng = (dot(Ng, Ns) < 0.0f) ? V3{-Ng.x, -Ng.y, -Ng.z} : Ng;
  ng = safeNormalize(ng, Ns);
  const V3 O = P + ng * eps;
  const uint32_t base = px + py * static_cast<uint32_t>(wHi);
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
  uint32_t c0 = px + 1u, c1 = py + 1u;
  tea2(c0, c1);
  const float cpx = u32ToUnorm(c0), cpy = u32ToUnorm(c1);
  float obsScale[3] = {0.0f, 0.0f, 0.0f};
  float weightedObs = 0.0f;
  V3 bentAccum{0.0f, 0.0f, 0.0f};
  float hitDistSum = 0.0f;
  int nHit = 0;
  for (int i = 0; i < nSamples; ++i) {
    float u1, u2;
    aoSample2d(ld, base, i, nSamples, cpx, cpy, u1, u2);
    const V3 dir = cosineSampleHemisphere(u1, u2, f);
    if (dot(dir, Ns) < 0.01f) {
      obsScale[0] += 1.0f; obsScale[1] += 1.0f; obsScale[2] += 1.0f;
      weightedObs += 1.0f;
      continue;
    }
    const float t = intersectNearest(s, O, dir, eps, R);
    float perSample = 0.0f;
    for (int k = 0; k < K; ++k) {
      if (t < radius[k]) {
        float fk = 1.0f;
        if (power > 0.0f) {
          float a = 1.0f - t / radius[k];
          if (a < 0.0f) a = 0.0f;
          fk = std::pow(a, power);
        }
        obsScale[k] += fk;
        perSample += weight[k] * fk;
      }
    }
    weightedObs += perSample;
    bentAccum = bentAccum + dir * (1.0f - perSample);
    if (t < R) { hitDistSum += t; ++nHit; }
  }
  const float invN = 1.0f / static_cast<float>(nSamples);
  r.openness = 1.0f - weightedObs * invN;
  r.contact = 1.0f - obsScale[0] * invN;
  if (multiScale) {
    const float wMid = weight[1] + weight[2];
    r.shape = 1.0f - (weight[1] * obsScale[1] + weight[2] * obsScale[2]) / (wMid * static_cast<float>(nSamples));
  } else {
    r.shape = r.openness;
  }
  r.bent = safeNormalize(bentAccum, Ns);
  r.avgHitDist = (nHit > 0) ? hitDistSum / static_cast<float>(nHit) : R;
  return r;
}

struct Opt {  // the RenderOptions fields this path reads
  int aoSamples; float aoDistance, aoIntensity, aoFalloffPower;
  bool aoMultiScale, aoBentNormal, aoMultibounce, aoLowDiscrepancy;
  float aoSky[3], aoGround[3], aoDiffuseFactor;
  bool shadows; int shadowSamples; int envLights;
  float specularScale; bool transparency, transparentBackground; int maxTransparentLayers;
  bool aoWriteAov = false;
  int aaMode = 0;
  bool edgeGbuffer = false;  // capture the stroke-edge pass's first-hit G-buffer
  // pt1 GI gather (render_options.hpp:85-151; the gather at every hi-res
  // pixel, no denoise of E)
  bool gi = false;
  int pt1Spp = 8, giBounces = 1, pt1SkyMode = 0;
  float giMaxDistance = 0.0f, giIntensity = 1.0f, giEnvIntensity = 1.0f, pt1Clamp = 0.0f;
  uint32_t pt1Seed = 0;
  float pt1SkyRadiance[3] = {1.0f, 1.0f, 1.0f};
  bool pt1Ld = true;
  // the gather grid and what follows it (render_options.hpp:130-176)
  int pt1GatherDiv = 1;  // resolved divisor
  bool pt1Denoise = false, pt1EdgePatch = false;
  float pt1UpNormalPow = 32.0f, pt1UpDepthScale = 0.02f, pt1EdgePatchThresh = 0.3f;
  int pt1EdgePatchSppMul = 4;
  int denoiseIters = 5;
  float denoiseSigmaN = 128.0f, denoiseSigmaZ = 1.0f, denoiseSigmaL = 4.0f;
  // pt2 (render_options.hpp:178-252)
  int giIntegrator = 1, pt2Pattern = 1, pt2AdaptiveMul = 4, pt2GlossySpp = 8;
  bool pt2Emissive = true, pt2EmissiveNee = true, pt2Reflect = true, pt2Glossy = true, pt2GlossyDenoise = true;
  bool pt2Adaptive = false;
  float pt2AdaptiveThresh = 0.15f;
  int pt2Rounds = 0;
  float pt2Radius = 16.0f, pt2MCap = 100.0f, pt2WClamp = 0.0f;
  bool pt2Unbiased = false;
  bool pt2() const { return gi && giIntegrator == 2; }
  bool traceRefl() const { return pt2() && pt2Reflect; }
  bool aoEnhanced() const {  // render_options.hpp:79-82
    return aoFalloffPower > 0.0f || aoMultiScale || aoBentNormal || aoMultibounce || aoLowDiscrepancy ||
           aoDiffuseFactor > 0.0f;
  }
};

struct AoShade { V3 aoFactor{1.0f, 1.0f, 1.0f}; V3 ambLight; float diffuseAo = 1.0f; };

// ao_shade.hpp:80-117 aoApplyFactors
inline AoShade aoApplyFactors(const Opt& o, const V3& ambLight, const V3& aoUp, float openness,
                              const AOResult& aov, const V3& C) {
  AoShade r;
  r.ambLight = ambLight;
  if (o.aoEnhanced() && o.aoBentNormal) {
    const float w = 0.5f * (dot(aov.bent, aoUp) + 1.0f);
    const float gx = o.aoGround[0], sx = o.aoSky[0];
    const float gy = o.aoGround[1], sy = o.aoSky[1];
    const float gz = o.aoGround[2], sz = o.aoSky[2];
    r.ambLight = V3{ambLight.x * (gx + (sx - gx) * w), ambLight.y * (gy + (sy - gy) * w),
                    ambLight.z * (gz + (sz - gz) * w)};
  }
  if (o.aoMultibounce) {
    const float ox = aoMultibounce(openness, C.x);
    const float oy = aoMultibounce(openness, C.y);
    const float oz = aoMultibounce(openness, C.z);
    r.aoFactor = V3{1.0f - o.aoIntensity * (1.0f - ox), 1.0f - o.aoIntensity * (1.0f - oy),
                    1.0f - o.aoIntensity * (1.0f - oz)};
  } else {
    const float sv = 1.0f - o.aoIntensity * (1.0f - openness);
    r.aoFactor = V3{sv, sv, sv};
  }
  if (o.aoDiffuseFactor > 0.0f) r.diffuseAo = 1.0f - o.aoDiffuseFactor * (1.0f - openness);
  return r;
}

// ao_shade.hpp:44-72 aoGather + :128-141 computeAoShade (sampleMul 1, wSeed = hi-res width)
// (ao_shade.hpp:43-72 aoGather: legacy colour + one single-scale quality pass
// for the AOVs when aoWriteAov asks for them)
inline AoShade computeAoShade(const Scene& s, const Opt& o, const V3& ambLight, const V3& aoUp,
                              const V3& P, const V3& Ng, const V3& N, const V3& C, float secEps,
                              uint32_t px, uint32_t py, int wSeed, AOResult* aovOut = nullptr) {
  if (o.aoSamples <= 0) { AoShade r; r.ambLight = ambLight; return r; }
  AOResult aov;
  float openness;
  if (o.aoEnhanced()) {
    aov = computeAOQuality(s, P, Ng, N, secEps, o.aoSamples, o.aoDistance, o.aoFalloffPower,
                           o.aoMultiScale, o.aoLowDiscrepancy, px, py, wSeed);
    openness = aov.openness;
  } else {
    openness = computeAO(s, P, Ng, N, secEps, o.aoSamples, o.aoDistance, px, py, wSeed);
    if (o.aoWriteAov)
      aov = computeAOQuality(s, P, Ng, N, secEps, o.aoSamples, o.aoDistance, 0.0f, false, false, px, py, wSeed);
  }
  if (aovOut) *aovOut = aov;
  return aoApplyFactors(o, ambLight, aoUp, openness, aov, C);
}

// shading.hpp:76-192 shadeLocal, POV branch
inline V3 shadeLocal(const Scene& s, const Mat& mat, const V3& C, const V3& N, const V3& V,
                     const std::vector<Light>& lights, const V3& ambLight, const V3& bg,
                     float specularScale, const V3& aoFactor, float diffuseAo, const V3& P,
                     const V3& Ng, float eps, bool shadowsOn, int shadowSamples, uint32_t px,
                     uint32_t py, bool traceRefl = false) {
  V3 out{mat.emission * C.x + aoFactor.x * mat.ambient * C.x * ambLight.x,
         mat.emission * C.y + aoFactor.y * mat.ambient * C.y * ambLight.y,
         mat.emission * C.z + aoFactor.z * mat.ambient * C.z * ambLight.z};
  const float ex = blinnExp(mat.roughness);
  uint32_t s0 = px, s1 = py;
  for (const Light& l : lights) {
    const float ndl = dot(N, l.L);
    if (ndl <= 0.0f) continue;
    const float shadowFactor = shadowsOn ? computeShadow(s, P, Ng, N, eps, l, shadowSamples, s0, s1) : 1.0f;
    const V3 Lc{l.color.x * shadowFactor, l.color.y * shadowFactor, l.color.z * shadowFactor};
    float d;
    if (mat.brilliance == 1.0f) d = ndl;
    else if (mat.brilliance == 0.0f) d = 1.0f;
    else d = std::pow(ndl, mat.brilliance);
    const float dk = mat.diffuse * d * diffuseAo;
    out.x += dk * C.x * Lc.x;
    out.y += dk * C.y * Lc.y;
    out.z += dk * C.z * Lc.z;
    if (!l.highlight) continue;
    V3 hl;
    if (mat.metallic) {
      float c = ndl;
      if (c > 1.0f) c = 1.0f;
      const float x = std::acos(c) * 0.63661977f;
      float f = 0.014567225f / ((x - 1.12f) * (x - 1.12f)) - 0.011612903f;
      if (f < 0.0f) f = 0.0f;
      if (f > 1.0f) f = 1.0f;
      hl = V3{Lc.x * (f + (1.0f - f) * C.x), Lc.y * (f + (1.0f - f) * C.y), Lc.z * (f + (1.0f - f) * C.z)};
    } else {
      hl = Lc;
    }
    float specW = 0.0f;
    if (mat.specular > 0.0f) {
      const V3 H = normalize(V3{l.L.x + V.x, l.L.y + V.y, l.L.z + V.z});
      float nh = dot(N, H);
      if (nh > 0.0f) specW += mat.specular * std::pow(nh, ex);
    }
    if (mat.phong > 0.0f) {
      const V3 Rr = 2.0f * ndl * N - l.L;
      float rv = dot(Rr, V);
      if (rv > 0.0f && (mat.phongSize < 60.0f || rv > 0.0008f)) specW += mat.phong * std::pow(rv, mat.phongSize);
    }
    if (specW > 0.0f) {
      const float sc = specW * specularScale;
      out.x += sc * hl.x;
      out.y += sc * hl.y;
      out.z += sc * hl.z;
    }
  }
  // the fake reflection x background; pt2's traced pass owns it instead (:181-190)
  if (mat.reflection > 0.0f && !traceRefl) {
    out.x += mat.reflection * bg.x;
    out.y += mat.reflection * bg.y;
    out.z += mat.reflection * bg.z;
  }
  return out;
}

// shading/principled.hpp:35-126: the GGX helpers of the principled model.
constexpr float kGgxDirectAlphaMin = 1.0e-3f;
inline V3 principledF0(const Mat& m, const V3& C) {
  const float dd = 0.08f * m.pbrSpecular;
  const float t = m.pbrMetallic;
  return V3{dd + (C.x - dd) * t, dd + (C.y - dd) * t, dd + (C.z - dd) * t};
}
inline V3 schlickF(const V3& F0, float u) {
  float c = 1.0f - u;
  if (c < 0.0f) c = 0.0f;
  if (c > 1.0f) c = 1.0f;
  const float c5 = c * c * c * c * c;
  return V3{F0.x + (1.0f - F0.x) * c5, F0.y + (1.0f - F0.y) * c5, F0.z + (1.0f - F0.z) * c5};
}
inline float ggxD(float a2, float ndh) {
  if (ndh <= 0.0f) return 0.0f;
  const float t = ndh * ndh * (a2 - 1.0f) + 1.0f;
  return a2 / (3.14159265358979323846f * t * t);
}
inline float ggxLambda(float a2, float cosT) {
  const float c2 = std::fmax(cosT * cosT, 1.0e-12f);
  const float t2 = (1.0f - c2) / c2;
  return 0.5f * (std::sqrt(1.0f + a2 * t2) - 1.0f);
}
inline float principledAspect(float anisotropy) {
  float a = std::fabs(anisotropy);
  if (a > 1.0f) a = 1.0f;
  return std::sqrt(1.0f - 0.9f * a);
}
inline float ggxDAniso(float ax, float ay, float hx, float hy, float hz) {
  if (hz <= 0.0f) return 0.0f;
  const float sx = hx / ax, sy = hy / ay;
  const float t = sx * sx + sy * sy + hz * hz;
  return 1.0f / (3.14159265358979323846f * ax * ay * t * t);
}
inline float ggxLambdaAniso(float ax, float ay, float vx, float vy, float vz) {
  const float z2 = std::fmax(vz * vz, 1.0e-12f);
  const float t2 = (ax * ax * vx * vx + ay * ay * vy * vy) / z2;
  return 0.5f * (std::sqrt(1.0f + t2) - 1.0f);
}

// shading/principled.hpp:139-302 shadePrincipled (direct pass, no traced
// reflection): one GGX lobe with Schlick Fresnel; an area light (shadows on,
// samples > 1, radius > 0) evaluates visibility and BRDF per cone sample on
// its own ('PBRD'-tagged) per-pixel stream.  `tangent` (anisotropy frame,
// sphere / cylinder hits) or null.
inline V3 shadePrincipled(const Scene& s, const Mat& mat, const V3& C, const V3& N, const V3& V,
                          const std::vector<Light>& lights, const V3& ambLight, const V3& bg, const V3& aoFactor,
                          float diffuseAo, const V3& P, const V3& Ng, float eps, bool shadowsOn, int shadowSamples,
                          uint32_t px, uint32_t py, const V3* tangent, bool traceRefl = false) {
  V3 out{mat.emission * C.x + aoFactor.x * mat.ambient * C.x * ambLight.x,
         mat.emission * C.y + aoFactor.y * mat.ambient * C.y * ambLight.y,
         mat.emission * C.z + aoFactor.z * mat.ambient * C.z * ambLight.z};
  const float kd = mat.diffuse * (1.0f - mat.pbrMetallic);
  const V3 F0 = principledF0(mat, C);
  const float f0max = std::fmax(F0.x, std::fmax(F0.y, F0.z));
  float alpha = mat.pbrRoughness * mat.pbrRoughness;
  if (alpha < kGgxDirectAlphaMin) alpha = kGgxDirectAlphaMin;
  const float a2 = alpha * alpha;
  const float ndv = std::fmax(dot(N, V), 1.0e-4f);
  const float lamV = ggxLambda(a2, ndv);
  constexpr float kPi = 3.14159265358979323846f;
  // principledAnisoCtx (:110-126)
  bool anActive = false;
  V3 at1, at2;
  float ax = 0.0f, ay = 0.0f;
  if (tangent != nullptr && mat.pbrAnisotropy != 0.0f) {
    anActive = true;
    at1 = *tangent;
    at2 = cross(N, at1);
    const float aspect = principledAspect(mat.pbrAnisotropy);
    ax = alpha / aspect;
    if (ax > 1.0f) ax = 1.0f;
    ay = alpha * aspect;
    if (ax < kGgxDirectAlphaMin) ax = kGgxDirectAlphaMin;
    if (ay < kGgxDirectAlphaMin) ay = kGgxDirectAlphaMin;
  }
  const float lamVA = anActive ? ggxLambdaAniso(ax, ay, dot(V, at1), dot(V, at2), ndv) : 0.0f;
  auto specWeight = [&](const V3& H, float ndh, const V3& w, float ndlw) {
    if (!anActive) {
      const float G2 = 1.0f / (1.0f + lamV + ggxLambda(a2, ndlw));
      return kPi * ggxD(a2, ndh) * G2 / (4.0f * ndv);
    }
    const float G2 = 1.0f / (1.0f + lamVA + ggxLambdaAniso(ax, ay, dot(w, at1), dot(w, at2), ndlw));
    return kPi * ggxDAniso(ax, ay, dot(H, at1), dot(H, at2), ndh) * G2 / (4.0f * ndv);
  };
  uint32_t s0 = px, s1 = py;
  uint32_t t0 = px ^ 0x50425244u, t1 = py;
  for (const Light& l : lights) {
    const float ndl = dot(N, l.L);
    if (ndl <= 0.0f) continue;
    const bool areaPath = shadowsOn && shadowSamples > 1 && l.radius > 0.0f;
    if (!areaPath) {
      const float shadowFactor = shadowsOn ? computeShadow(s, P, Ng, N, eps, l, shadowSamples, s0, s1) : 1.0f;
      const V3 Lc{l.color.x * shadowFactor, l.color.y * shadowFactor, l.color.z * shadowFactor};
      const float dk = kd * ndl * diffuseAo;
      out.x += dk * C.x * Lc.x;
      out.y += dk * C.y * Lc.y;
      out.z += dk * C.z * Lc.z;
      if (!l.highlight) continue;
      if (f0max > 0.0f) {
        const V3 H = normalize(V3{l.L.x + V.x, l.L.y + V.y, l.L.z + V.z});
        const float ndh = dot(N, H);
        if (ndh > 0.0f) {
          const float sW = specWeight(H, ndh, l.L, ndl);
          const V3 F = schlickF(F0, dot(V, H));
          out.x += sW * F.x * Lc.x;
          out.y += sW * F.y * Lc.y;
          out.z += sW * F.z * Lc.z;
        }
      }
    } else {
      V3 ng = (dot(Ng, N) < 0.0f) ? V3{-Ng.x, -Ng.y, -Ng.z} : Ng;
      ng = safeNormalize(ng, N);
      const V3 O = P + ng * eps;
      float accD = 0.0f;
      V3 accS{0.0f, 0.0f, 0.0f};
      for (int k = 0; k < shadowSamples; ++k) {
        tea2(t0, t1);
        const V3 w = sampleLightDir(l, u32ToUnorm(t0), u32ToUnorm(t1));
        const float ndlS = dot(N, w);
        if (ndlS <= 0.0f) continue;
        if (occludedQ(s, O, w, eps, kInf)) continue;
        accD += ndlS;
        if (l.highlight && f0max > 0.0f) {
          const V3 H = normalize(V3{w.x + V.x, w.y + V.y, w.z + V.z});
          const float ndh = dot(N, H);
          if (ndh > 0.0f) {
            const float sW = specWeight(H, ndh, w, ndlS);
            const V3 F = schlickF(F0, dot(V, H));
            accS.x += sW * F.x;
            accS.y += sW * F.y;
            accS.z += sW * F.z;
          }
        }
      }
      const float inv = 1.0f / static_cast<float>(shadowSamples);
      const float dk = kd * diffuseAo * inv * accD;
      out.x += dk * C.x * l.color.x;
      out.y += dk * C.y * l.color.y;
      out.z += dk * C.z * l.color.z;
      out.x += inv * accS.x * l.color.x;
      out.y += inv * accS.y * l.color.y;
      out.z += inv * accS.z * l.color.z;
    }
  }
  // principled.hpp:277-302: the environment term, owned by pt2's traced pass
  if (!traceRefl) {
    if (mat.reflection > 0.0f) {
      out.x += mat.reflection * bg.x;
      out.y += mat.reflection * bg.y;
      out.z += mat.reflection * bg.z;
    } else if (f0max > 0.0f) {
      out.x += F0.x * bg.x;
      out.y += F0.y * bg.y;
      out.z += F0.z * bg.z;
    }
  }
  return out;
}

// shading.hpp:48-60 pt2GgxAlphaFromRoughness: sqrt(2 / (blinnExp + 2)),
// a mirror (0) below 0.015, at most 1
inline float ggxAlphaFromRoughness(float roughness) {
  const float e = blinnExp(roughness);
  const float a = std::sqrt(2.0f / (e + 2.0f));
  if (a < 0.015f) return 0.0f;
  return a < 1.0f ? a : 1.0f;
}

// ao/ao_coarse.hpp:55-66 CoarseAoGrid: AO gathered once per coarse cell plus
// the lookup guides (shading normal, primary hit distance, eligibility).
struct CoarseAo {
  int w = 0, h = 0;
  bool quality = false;  // bent / contact / shape / avgHitDist gathered
  std::vector<float> openness, bent, contact, shape, avgHitDist, normal, depth;
  std::vector<uint8_t> hit;
};

struct Ctx {
  const Scene* s;
  std::vector<Light> lights;
  V3 ambLight, bg, aoUp;
  Opt o;
  int wHi;  // seed lattice width (hi-res width; W k on a fine lattice)
  float clipNear, clipFar;
  const CoarseAo* coarse = nullptr;  // coarse-grid AO when active
  int frameW = 0, frameH = 0;        // hi-res frame size (lookup lattice height)
};

// ao/ao_coarse.hpp:152-203 sampleCoarseAo: bilinear x normal^32 x depth
// weights over the 2x2 surrounding cells, rejected below a weight sum of 0.3.
inline bool sampleCoarseAo(const CoarseAo& g, int latW, int latH, uint32_t px, uint32_t py, const V3& N, float z,
                           float& openness, AOResult& aov) {
  if (g.w <= 0 || g.h <= 0) return false;
  const float sx = (static_cast<float>(px) + 0.5f) * static_cast<float>(g.w) / static_cast<float>(latW) - 0.5f;
  const float sy = (static_cast<float>(py) + 0.5f) * static_cast<float>(g.h) / static_cast<float>(latH) - 0.5f;
  const int bx = static_cast<int>(std::floor(sx));
  const int by = static_cast<int>(std::floor(sy));
  const float fx = sx - static_cast<float>(bx);
  const float fy = sy - static_cast<float>(by);
  float wSum = 0.0f, opSum = 0.0f, contactSum = 0.0f, shapeSum = 0.0f, ahdSum = 0.0f;
  V3 bentSum{0.0f, 0.0f, 0.0f};
  for (int dy = 0; dy < 2; ++dy) {
    const int cy = by + dy;
    if (cy < 0 || cy >= g.h) continue;
    for (int dx = 0; dx < 2; ++dx) {
      const int cx = bx + dx;
      if (cx < 0 || cx >= g.w) continue;
      const size_t cp = static_cast<size_t>(cy) * g.w + cx;
      if (!g.hit[cp]) continue;
      const float wb = (dx ? fx : 1.0f - fx) * (dy ? fy : 1.0f - fy);
      const V3 Nc{g.normal[cp * 3], g.normal[cp * 3 + 1], g.normal[cp * 3 + 2]};
      const float nd = dot(N, Nc);
      if (nd <= 0.0f) continue;
      const float wn = std::pow(nd, 32.0f);
      const float zc = g.depth[cp];
      const float wz = std::exp(-std::fabs(z - zc) / (0.02f * z + 1e-6f));
      const float wgt = wb * wn * wz;
      if (wgt <= 0.0f) continue;
      wSum += wgt;
      opSum += wgt * g.openness[cp];
      if (g.quality) {
        bentSum.x += wgt * g.bent[cp * 3];
        bentSum.y += wgt * g.bent[cp * 3 + 1];
        bentSum.z += wgt * g.bent[cp * 3 + 2];
        contactSum += wgt * g.contact[cp];
        shapeSum += wgt * g.shape[cp];
        ahdSum += wgt * g.avgHitDist[cp];
      }
    }
  }
  if (wSum < 0.3f) return false;
  const float inv = 1.0f / wSum;
  openness = opSum * inv;
  aov = AOResult{};
  aov.openness = openness;
  if (g.quality) {
    aov.bent = safeNormalize(V3{bentSum.x * inv, bentSum.y * inv, bentSum.z * inv}, N);
    aov.contact = contactSum * inv;
    aov.shape = shapeSum * inv;
    aov.avgHitDist = ahdSum * inv;
  }
  return true;
}

// hit_shader.hpp:129-145 aoShadeForHit: the coarse-grid lookup first (the hit
// is its own guide: N and its primary-ray distance), else the exact inline
// gather with the unchanged seeds, marking the hit as patched.
inline AoShade aoShadeForHit(const Ctx& c, const V3& P, const V3& Ng, const V3& N, const V3& C, float secEps,
                             float hitT, uint32_t px, uint32_t py, uint8_t* patched, AOResult* aovOut = nullptr) {
  if (c.coarse != nullptr && c.o.aoSamples > 0) {
    const int latW = c.wHi;
    const int latH = static_cast<int>(static_cast<int64_t>(latW) * c.frameH / c.frameW);
    float openness;
    AOResult aov;
    if (sampleCoarseAo(*c.coarse, latW, latH, px, py, N, hitT, openness, aov)) {
      if (aovOut) *aovOut = aov;
      return aoApplyFactors(c.o, c.ambLight, c.aoUp, openness, aov, C);
    }
    if (patched) *patched = 1;
  }
  return computeAoShade(*c.s, c.o, c.ambLight, c.aoUp, P, Ng, N, C, secEps, px, py, c.wHi, aovOut);
}

struct HitShade {
  V3 color;
  float opacity = 1.0f;
  V3 giRefl{0.0f, 0.0f, 0.0f};  // kd * pigment of a GI-eligible hit (hit_shader.hpp:48-54)
  uint8_t giElig = 0;
  // AO AOVs (hit_shader.hpp:41-55): set on mesh hits when aoWriteAov is on
  V3 albedo{0.0f, 0.0f, 0.0f}, normal{0.0f, 0.0f, 0.0f}, bent{0.0f, 0.0f, 0.0f};
  float contact = 1.0f, shape = 1.0f, avgHit = 0.0f;
  int group = 0;  // CueMol section of the hit (hit_shader.hpp:277, 457)
  uint8_t aoPatched = 0;  // coarse-grid AO fell back to the inline gather (hit_shader.hpp:60)
  // edge G-buffer (hit_shader.hpp:278-300, 460-478): (section << 2) | kind and
  // the global material index; background sentinels
  uint32_t objectId = 0xFFFFFFFFu, materialId = 0xFFFFFFFFu;
  // pt2 traced reflection of this hit (hit_shader.hpp:61-80)
  float reflAmt = 0.0f, reflAlpha = 0.0f, reflAspect = 1.0f;
  V3 reflF0{1.0f, 1.0f, 1.0f}, reflTan{0.0f, 0.0f, 0.0f};
};

// hit_shader.hpp:147-496 shadeHit (POV and principled direct; GI / edge branches off)
// Material::diffuseWeight / toonLike (scene.hpp:171-196)
inline float matDiffuseWeight(const Mat& m) { return m.model == 1 ? m.diffuse * (1.0f - m.pbrMetallic) : m.diffuse; }
inline bool matToonLike(const Mat& m) {
  if (m.model == 2) return true;
  if (m.model != 0) return false;
  if (m.specular > 1.0f || m.phong > 1.0f || m.brilliance == 0.0f) return true;
  return m.diffuse <= 0.0f && m.specular <= 0.0f && m.phong <= 0.0f && m.reflection <= 0.0f;
}

inline HitShade shadeHit(const Ctx& c, const Hit& hit, const V3& rd, const V3& org, uint32_t px, uint32_t py) {
  const Scene& s = *c.s;
  HitShade hs;
  const bool shadowsActive = c.o.shadows || c.o.envLights > 0;
  const int kind = kindOfGeom(s, hit.geomID);
  const V3 V = normalize(V3{-rd.x, -rd.y, -rd.z});
  const V3 Ng = hit.Ng;
  const V3 P{org.x + rd.x * hit.t, org.y + rd.y * hit.t, org.z + rd.z * hit.t};
  const float secEps = selfIntersectEps(P, rd, hit.t);
  if (kind == kMesh) {
    // rtcInterpolate0 of slots 0 (normal) and 1 (colour): (1-u-v) a0 + u a1 + v a2
    const uint32_t* tri = &s.geo.triIdx[3 * hit.primID];
    const float w0 = 1.0f - hit.u - hit.v;
    float nbuf[3], cbuf[4];
    for (int k = 0; k < 3; ++k)
      nbuf[k] = w0 * s.nrm[3 * tri[0] + k] + hit.u * s.nrm[3 * tri[1] + k] + hit.v * s.nrm[3 * tri[2] + k];
    for (int k = 0; k < 4; ++k)
      cbuf[k] = w0 * s.col[4 * tri[0] + k] + hit.u * s.col[4 * tri[1] + k] + hit.v * s.col[4 * tri[2] + k];
    const V3 NgF = faceForward(Ng, rd);
    V3 N = normalize(V3{nbuf[0], nbuf[1], nbuf[2]});
    if (dot(N, NgF) < 0.0f) N = V3{-N.x, -N.y, -N.z};
    const V3 C{cbuf[0], cbuf[1], cbuf[2]};
    const size_t bt = s.baseTri ? hit.primID % s.baseTri : 0;
    const Mat& triMat = s.triMat.empty() ? s.meshMat : s.meshMats[s.triMat[bt]];
    AOResult aov;
    AoShade ao = aoShadeForHit(c, P, Ng, N, C, secEps, hit.t, px, py, &hs.aoPatched, &aov);
    // hit_shader.hpp:221-242: under GI the constant ambient gives way to the
    // gathered indirect; toon finishes keep a unit ambient and get none
    if (c.o.gi && matToonLike(triMat)) {
      ao.ambLight = V3{1.0f, 1.0f, 1.0f};
    } else if (c.o.gi) {
      const float kd = matDiffuseWeight(triMat);
      hs.giRefl = V3{kd * C.x, kd * C.y, kd * C.z};
      hs.giElig = 1;
      ao.ambLight = V3{0.0f, 0.0f, 0.0f};
    }
    // hit_shader.hpp:243-270: traced-reflection ownership under pt2
    const bool pbrSpec = triMat.model == 1 && (triMat.pbrMetallic > 1e-4f || triMat.pbrSpecular > 1e-4f);
    const bool traceRefl = c.o.traceRefl() && (triMat.model == 1 ? pbrSpec : triMat.reflection > 0.0f);
    if (traceRefl) {
      if (triMat.model == 1) {
        hs.reflAmt = 1.0f;
        hs.reflF0 = principledF0(triMat, C);
        if (c.o.pt2Glossy) {
          const float a = triMat.pbrRoughness * triMat.pbrRoughness;
          hs.reflAlpha = a >= 0.015f ? a : 0.0f;
        }
      } else {
        hs.reflAmt = triMat.reflection;
        if (c.o.pt2Glossy && triMat.specular > 0.0f) hs.reflAlpha = ggxAlphaFromRoughness(triMat.roughness);
      }
    }
    hs.color = triMat.model == 1
                   ? shadePrincipled(s, triMat, C, N, V, c.lights, ao.ambLight, c.bg, ao.aoFactor, ao.diffuseAo, P,
                                     Ng, secEps, shadowsActive, c.o.shadowSamples, px, py, nullptr, traceRefl)
                   : shadeLocal(s, triMat, C, N, V, c.lights, ao.ambLight, c.bg, c.o.specularScale, ao.aoFactor,
                          ao.diffuseAo, P, Ng, secEps, shadowsActive, c.o.shadowSamples, px, py, traceRefl);
    hs.opacity = cbuf[3];
    if (c.o.aoWriteAov) {  // hit_shader.hpp:207-213
      hs.albedo = C;
      hs.normal = N;
      hs.bent = aov.bent;
      hs.contact = aov.contact;
      hs.shape = aov.shape;
      hs.avgHit = aov.avgHitDist;
    } else if (c.o.gi || c.o.aaMode == 1) {  // :214-220 (the adaptive-AA mask reads N)
      hs.albedo = C;
      hs.normal = N;
    }
    hs.group = s.triGroup.empty() ? 0 : s.triGroup[s.baseTri ? hit.primID % s.baseTri : hit.primID];
    if (c.o.edgeGbuffer) {
      hs.normal = N;
      hs.objectId = (static_cast<uint32_t>(hs.group) << 2) | static_cast<uint32_t>(kMesh);
      hs.materialId = s.triMat.empty() ? 0u : static_cast<uint32_t>(s.triMat[hit.primID % s.triMat.size()]);
    }
  } else {
    const float* fc = &s.color[kind][4 * hit.primID];
    const Mat& pm = s.mat[kind][hit.primID];
    V3 N = faceForward(normalize(Ng), rd);
    const V3 C{fc[0], fc[1], fc[2]};
    const bool fromEdge = s.fromEdge[kind][hit.primID] != 0;
    V3 aoFactor{1.0f, 1.0f, 1.0f};
    V3 ambLight = c.ambLight;
    float diffuseAo = 1.0f;
    if (!fromEdge) {
      AoShade ao = aoShadeForHit(c, P, Ng, N, C, secEps, hit.t, px, py, &hs.aoPatched);
      aoFactor = ao.aoFactor;
      ambLight = ao.ambLight;
      diffuseAo = ao.diffuseAo;
      // hit_shader.hpp:351-365 (pt1): a real primitive receives the
      // gathered indirect like the mesh
      if (c.o.gi && matToonLike(pm)) {
        ambLight = V3{1.0f, 1.0f, 1.0f};
      } else if (c.o.gi) {
        const float kd = matDiffuseWeight(pm);
        hs.giRefl = V3{kd * C.x, kd * C.y, kd * C.z};
        hs.giElig = 1;
        hs.normal = N;
        ambLight = V3{0.0f, 0.0f, 0.0f};
      }
    }
    const bool primShadows = !fromEdge && shadowsActive;
    // anisotropy tangent frame (hit_shader.hpp:373-425): sphere = meridian of
    // the world +y pole, cylinder = axis projected onto the tangent plane;
    // poles, caps and degenerate projections stay isotropic
    V3 anisoT{0.0f, 0.0f, 0.0f};
    bool tanValid = false;
    if (pm.model == 1 && pm.pbrAnisotropy != 0.0f && !fromEdge) {
      V3 t1{0.0f, 0.0f, 0.0f};
      if (kind == kSphere) {
        if (std::fabs(N.y) < 0.999f) {
          const V3 tPhi = safeNormalize(cross(V3{0.0f, 1.0f, 0.0f}, N));
          t1 = cross(N, tPhi);
          tanValid = true;
        }
      } else if (!s.axis[kind].empty()) {
        const V3 A = s.axis[kind][hit.primID];
        const V3 ngu = safeNormalize(Ng, N);
        if (std::fabs(dot(ngu, A)) < 0.99f) {
          const float andn = dot(A, N);
          const V3 proj{A.x - N.x * andn, A.y - N.y * andn, A.z - N.z * andn};
          if (dot(proj, proj) >= 1.0e-12f) {
            t1 = safeNormalize(proj);
            tanValid = true;
          }
        }
      }
      if (tanValid) {
        if (pm.pbrAnisotropyRotation != 0.0f) {
          const float ang = pm.pbrAnisotropyRotation * 6.2831853072f;
          const V3 t2 = cross(N, t1);
          const float ca = std::cos(ang), sa = std::sin(ang);
          t1 = V3{ca * t1.x + sa * t2.x, ca * t1.y + sa * t2.y, ca * t1.z + sa * t2.z};
        }
        anisoT = t1;
      }
    }
    // hit_shader.hpp:426-452: traced-reflection ownership, primitive path
    const bool pbrSpecP = pm.model == 1 && (pm.pbrMetallic > 1e-4f || pm.pbrSpecular > 1e-4f);
    const bool traceReflP = c.o.traceRefl() && !fromEdge && (pm.model == 1 ? pbrSpecP : pm.reflection > 0.0f);
    if (traceReflP) {
      if (pm.model == 1) {
        hs.reflAmt = 1.0f;
        hs.reflF0 = principledF0(pm, C);
        if (c.o.pt2Glossy) {
          const float a = pm.pbrRoughness * pm.pbrRoughness;
          hs.reflAlpha = a >= 0.015f ? a : 0.0f;
          if (tanValid) {
            hs.reflTan = anisoT;
            hs.reflAspect = principledAspect(pm.pbrAnisotropy);
          }
        }
      } else {
        hs.reflAmt = pm.reflection;
        if (c.o.pt2Glossy && pm.specular > 0.0f) hs.reflAlpha = ggxAlphaFromRoughness(pm.roughness);
      }
    }
    hs.color = pm.model == 1
                   ? shadePrincipled(s, pm, C, N, V, c.lights, ambLight, c.bg, aoFactor, diffuseAo, P, Ng, secEps,
                                     primShadows, c.o.shadowSamples, px, py, tanValid ? &anisoT : nullptr,
                                     traceReflP)
                   : shadeLocal(s, pm, C, N, V, c.lights, ambLight, c.bg, c.o.specularScale, aoFactor, diffuseAo,
                                P, Ng, secEps, primShadows, c.o.shadowSamples, px, py, traceReflP);
    hs.opacity = fc[3];
    hs.group = s.group[kind][hit.primID];
    if (c.o.aaMode == 1) hs.normal = N;  // hit_shader.hpp:321
    if (c.o.edgeGbuffer) {
      // global materialId: per-kind blocks after the mesh materials, the raw
      // primitive index inside (scene_build.cpp:104-123, curve_build.cpp:154-179)
      hs.normal = N;
      hs.objectId = (static_cast<uint32_t>(hs.group) << 2) | static_cast<uint32_t>(kind);
      const uint32_t meshMats = static_cast<uint32_t>(s.meshMats.size());
      if (kind == kSphere) hs.materialId = meshMats + hit.primID;
      else if (kind == kRound) hs.materialId = meshMats + s.baseSpheres + hit.primID;
      else hs.materialId = meshMats + s.baseSpheres + static_cast<uint32_t>(s.geo.rcIdx.size()) + hit.primID;
    }
    if (kind != kSphere) {
      const float op1 = s.opacity1[kind][hit.primID];
      if (op1 >= 0.0f) {
        float u = hit.u;
        if (u < 0.0f) u = 0.0f;
        if (u > 1.0f) u = 1.0f;
        hs.opacity = fc[3] * (1.0f - u) + op1 * u;
      }
    }
  }
  return hs;
}

struct PixelOut {
  float r, g, b, a, depth, viewZ;
  uint32_t geom, prim;
  bool capped;
  uint32_t rays;
  HitShade first;  // AOVs of the first hit (neutral values on a miss)
  V3 firstPos{0.0f, 0.0f, 0.0f};  // org + rd * nearDepth (transparency.hpp:410-411)
  // clip-cut G-buffer (transparency.hpp:424-428, 470-481)
  uint8_t clipCut = 0;
  float clipNearVz = 0.0f, clipFarVz = 0.0f;
};

// transparency.hpp:131-186: backface test, the any-hit confirmation of a
// clipped-away front, the first hit of a t range as view z
inline bool clipConfirmFront(const Scene& s, const V3& org, const V3& rd, float tMax) {
  Ray r;
  r.org = org; r.dir = rd;
  r.tnear = std::max(1.0e-4f, 1.0e-4f * tMax);
  r.tfar = tMax * (1.0f - 1.0e-4f);
  if (r.tnear >= r.tfar) return false;
  return s.bvh.occluded(r);
}
inline float clipProbeRange(const Scene& s, const V3& org, const V3& rd, const V3& camDir, float t0, float t1) {
  if (t0 >= t1) return 0.0f;
  Ray r;
  r.org = org; r.dir = rd; r.tnear = t0; r.tfar = t1;
  Hit h;
  if (!s.bvh.closest(r, h)) return 0.0f;
  return h.t * dot(rd, camDir);
}

// transparency.hpp:311-522 integratePixel (colour, first-hit depth/viewZ/ids)
// irradiance_cache.hpp:176-184 hashU32
inline uint32_t hashU32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7FEB352Du;
  x ^= x >> 15;
  x *= 0x846CA68Bu;
  x ^= x >> 16;
  return x;
}

// irradiance_cache.hpp:188-196 environmentRadiance with the pt1 sky
// (embree_renderer.cpp:590-601): the gather's miss term
inline V3 pt1Environment(const Ctx& c, const V3& wi) {
  const V3 sky{c.o.pt1SkyRadiance[0], c.o.pt1SkyRadiance[1], c.o.pt1SkyRadiance[2]};
  const V3 gr = c.o.pt1SkyMode == 1 ? V3{c.o.aoGround[0], c.o.aoGround[1], c.o.aoGround[2]} : sky;
  const float w = 0.5f * (dot(wi, c.aoUp) + 1.0f);
  const float e = c.o.giEnvIntensity;
  return V3{e * c.ambLight.x * (gr.x + (sky.x - gr.x) * w), e * c.ambLight.y * (gr.y + (sky.y - gr.y) * w),
            e * c.ambLight.z * (gr.z + (sky.z - gr.z) * w)};
}

// pt1_gather.hpp:117-227 pt1EvalVertex: the vertex's reflected direct light
// through one shadow ray per light (the centre ray; with a stream, pt2, an
// area light's ray is drawn from its cone), its reflectance kd * C, its
// emission * C when asked, and the normal faced toward the ray origin.
// Outline primitives end the path.
inline bool pt1EvalVertex(const Ctx& c, const Hit& h, const V3& O, const V3& wi, V3& rad, V3& alb, V3& Py,
                          V3& Ny, bool addEmission = false, uint32_t* r0 = nullptr, uint32_t* r1 = nullptr,
                          V3* emitted = nullptr) {
  const Scene& s = *c.s;
  const int kind = kindOfGeom(s, h.geomID);
  V3 C, NgSh;
  const Mat* m;
  if (kind == kMesh) {
    const uint32_t* tri = &s.geo.triIdx[3 * h.primID];
    const float w0 = 1.0f - h.u - h.v;
    float nb[3], cb[3];
    for (int k = 0; k < 3; ++k)
      nb[k] = w0 * s.nrm[3 * tri[0] + k] + h.u * s.nrm[3 * tri[1] + k] + h.v * s.nrm[3 * tri[2] + k];
    for (int k = 0; k < 3; ++k)
      cb[k] = w0 * s.col[4 * tri[0] + k] + h.u * s.col[4 * tri[1] + k] + h.v * s.col[4 * tri[2] + k];
    Ny = normalize(V3{nb[0], nb[1], nb[2]});
    C = V3{cb[0], cb[1], cb[2]};
    const size_t bt = s.baseTri ? h.primID % s.baseTri : 0;
    m = s.triMat.empty() ? &s.meshMat : &s.meshMats[s.triMat[bt]];
    NgSh = h.Ng;
  } else {
    if (s.fromEdge[kind][h.primID]) return false;
    const float* fc = &s.color[kind][4 * h.primID];
    m = &s.mat[kind][h.primID];
    C = V3{fc[0], fc[1], fc[2]};
    Ny = safeNormalize(h.Ng);
    NgSh = Ny;
  }
  const float kd = matDiffuseWeight(*m);
  if (dot(Ny, wi) > 0.0f) Ny = V3{-Ny.x, -Ny.y, -Ny.z};
  Py = V3{O.x + wi.x * h.t, O.y + wi.y * h.t, O.z + wi.z * h.t};
  const float eps = selfIntersectEps(Py, wi, h.t);
  V3 E{0.0f, 0.0f, 0.0f};
  for (const Light& l : c.lights) {
    const float ndl = dot(Ny, l.L);
    if (ndl <= 0.0f) continue;
    V3 ng = (dot(NgSh, Ny) < 0.0f) ? V3{-NgSh.x, -NgSh.y, -NgSh.z} : NgSh;
    ng = safeNormalize(ng, Ny);
    const V3 So{Py.x + ng.x * eps, Py.y + ng.y * eps, Py.z + ng.z * eps};
    V3 dir = l.L;
    if (r0 && l.radius > 0.0f) {
      tea2(*r0, *r1);
      dir = sampleLightDir(l, u32ToUnorm(*r0), u32ToUnorm(*r1));
    }
    const float sh = occludedQ(s, So, dir, eps, kInf) ? 0.0f : 1.0f;
    E.x += ndl * l.color.x * sh;
    E.y += ndl * l.color.y * sh;
    E.z += ndl * l.color.z * sh;
  }
  rad = V3{kd * C.x * E.x, kd * C.y * E.y, kd * C.z * E.z};
  alb = V3{kd * C.x, kd * C.y, kd * C.z};
  if (emitted) {
    *emitted = V3{0.0f, 0.0f, 0.0f};
    if (addEmission && m->emission > 0.0f) *emitted = V3{m->emission * C.x, m->emission * C.y, m->emission * C.z};
  }
  return true;
}

// ---- pt2 sampler (pt2_sampler.hpp): hash-based Owen-scrambled Sobol after
// Burley (JCGT 9(4), 2020) and the blue-noise pixel arrangement ----
inline uint32_t owenHash(uint32_t n, uint32_t seed) {
  n ^= n * 0x3d20adeau;
  n += seed;
  n *= (seed >> 16) | 1u;
  n ^= n * 0x05526c56u;
  n ^= n * 0x53a22864u;
  return n;
}
inline uint32_t owenHashBase4(uint32_t n, uint32_t seed) {
  n ^= n * 0x3d20adeau;
  n ^= (n >> 1) & (n << 1) & 0x55555555u;
  n += seed;
  n *= (seed >> 16) | 1u;
  n ^= (n >> 1) & (n << 1) & 0x55555555u;
  n ^= n * 0x05526c56u;
  n ^= n * 0x53a22864u;
  return n;
}
inline uint32_t reverseBits(uint32_t x) {
  uint32_t r = 0;
  for (int i = 0; i < 32; ++i) r |= ((x >> i) & 1u) << (31 - i);
  return r;
}
inline uint32_t expandBits16(uint32_t x) {
  x &= 0x0000ffffu;
  x = (x ^ (x << 8)) & 0x00ff00ffu;
  x = (x ^ (x << 4)) & 0x0f0f0f0fu;
  x = (x ^ (x << 2)) & 0x33333333u;
  x = (x ^ (x << 1)) & 0x55555555u;
  return x;
}
// dimension 1's direction numbers in reversed-bit order: Pascal's triangle mod 2
inline uint32_t sobolDir1(uint32_t i) {
  uint32_t v = 1u;
  for (uint32_t k = 0; k < i; ++k) v ^= v << 1;
  return v;
}
inline float sobolDim(uint32_t revIndex, int dim, uint32_t scramble) {
  uint32_t result = 0;
  if (dim == 0) {
    result = reverseBits(revIndex);
  } else {
    uint32_t i = 0;
    while (revIndex != 0u) {
      uint32_t j = 0;
      while (!(revIndex & (0x80000000u >> j))) ++j;
      result ^= sobolDir1(i + j);
      i += j + 1;
      revIndex <<= j;
      revIndex <<= 1;
    }
  }
  return static_cast<float>(reverseBits(owenHash(result, scramble))) * (1.0f / 4294967808.0f);
}
inline void sobol2D(uint32_t index, uint32_t seed, float& u1, float& u2) {
  index = owenHash(reverseBits(index), seed ^ 0xf8ade99au);
  u1 = sobolDim(index, 0, seed ^ 0xe0aaaf76u);
  u2 = sobolDim(index, 1, seed ^ 0x94964d4eu);
}
inline uint32_t nextPow2(uint32_t n) {
  uint32_t q = 1;
  while (q < n) q <<= 1;
  return q;
}

// ---- pt2 emissive NEE (pt2_emissive.hpp:279-520) ----
inline float emitPdfTri(const Scene& s, uint32_t ti, float dist2, float cosL) {
  if (cosL <= 1.0e-6f) return 0.0f;
  return s.emPdf[ti] * dist2 / (cosL * s.emTris[ti].area);
}

// one power-sampled emitter draw (exactly two tea2 draws), visibility, the
// balance-heuristic weight against the cosine gather
inline V3 emissiveNee(const Scene& s, const V3& P, const V3& N, const V3& Ng, float epsT, uint32_t& s0,
                      uint32_t& s1) {
  const V3 zero{0.0f, 0.0f, 0.0f};
  const float kPi = 3.14159265358979323846f;
  tea2(s0, s1);
  const float u = u32ToUnorm(s0);
  uint32_t lo = 0, hi = static_cast<uint32_t>(s.emCdf.size() - 1);
  while (lo < hi) {
    const uint32_t mid = (lo + hi) / 2;
    if (s.emCdf[mid] < u) lo = mid + 1;
    else hi = mid;
  }
  const uint32_t triCount = static_cast<uint32_t>(s.emTris.size());
  V3 dir, Le;
  float target, pdfSA;
  if (lo < triCount) {
    const Scene::EmitTri& t = s.emTris[lo];
    tea2(s0, s1);
    const float b0 = u32ToUnorm(s0), b1 = u32ToUnorm(s1);
    const float sq = std::sqrt(b0);
    const float w1 = 1.0f - sq, w2 = b1 * sq, w0 = 1.0f - w1 - w2;
    const V3 S{t.p0.x * w0 + t.p1.x * w1 + t.p2.x * w2, t.p0.y * w0 + t.p1.y * w1 + t.p2.y * w2,
               t.p0.z * w0 + t.p1.z * w1 + t.p2.z * w2};
    Le = V3{t.e0.x * w0 + t.e1.x * w1 + t.e2.x * w2, t.e0.y * w0 + t.e1.y * w1 + t.e2.y * w2,
            t.e0.z * w0 + t.e1.z * w1 + t.e2.z * w2};
    const V3 d{S.x - P.x, S.y - P.y, S.z - P.z};
    const float dist2 = dot(d, d);
    if (dist2 <= 1.0e-12f) return zero;
    const float dist = std::sqrt(dist2);
    dir = V3{d.x / dist, d.y / dist, d.z / dist};
    const float cosP = dot(N, dir);
    if (cosP <= 0.0f) return zero;
    const float cosL = std::fabs(dot(t.ng, dir));
    pdfSA = emitPdfTri(s, lo, dist2, cosL);
    if (pdfSA <= 0.0f) return zero;
    target = dist;
  } else {
    const Scene::EmitCsg& g = s.emCsg[lo - triCount];
    tea2(s0, s1);
    const float u1 = u32ToUnorm(s0), u2 = u32ToUnorm(s1);
    const float phi = 2.0f * kPi * u2;
    Le = g.Le;
    if (g.kind == 1) {
      const V3 d{g.p0.x - P.x, g.p0.y - P.y, g.p0.z - P.z};
      const float dc2 = dot(d, d);
      const float r2 = g.radius * g.radius;
      if (dc2 <= r2 * 1.0002f) return zero;
      const float dc = std::sqrt(dc2);
      const float sin2Max = r2 / dc2;
      const float cosMax = std::sqrt(std::fmax(0.0f, 1.0f - sin2Max));
      const float oneMinusCos = sin2Max / (1.0f + cosMax);
      const float cosT = 1.0f - u1 * oneMinusCos;
      const float sinT = std::sqrt(std::fmax(0.0f, 1.0f - cosT * cosT));
      const Frame fr = frameFromNormal(V3{d.x / dc, d.y / dc, d.z / dc});
      const float sx = sinT * std::cos(phi), sy = sinT * std::sin(phi);
      dir = V3{fr.t.x * sx + fr.b.x * sy + fr.n.x * cosT, fr.t.y * sx + fr.b.y * sy + fr.n.y * cosT,
               fr.t.z * sx + fr.b.z * sy + fr.n.z * cosT};
      pdfSA = s.emPdf[lo] / (2.0f * kPi * oneMinusCos);
      const float b = dot(d, dir);
      const float disc = std::fmax(0.0f, b * b - (dc2 - r2));
      target = b - std::sqrt(disc);
    } else {
      const Frame fr = frameFromNormal(g.axis);
      V3 S, nS;
      if (g.kind == 2) {
        nS = V3{fr.t.x * std::cos(phi) + fr.b.x * std::sin(phi), fr.t.y * std::cos(phi) + fr.b.y * std::sin(phi),
                fr.t.z * std::cos(phi) + fr.b.z * std::sin(phi)};
        const float hgt = u1 * g.len;
        S = V3{g.p0.x + g.axis.x * hgt + nS.x * g.radius, g.p0.y + g.axis.y * hgt + nS.y * g.radius,
               g.p0.z + g.axis.z * hgt + nS.z * g.radius};
      } else {
        const float rr = g.radius * std::sqrt(u1);
        S = V3{g.p0.x + (fr.t.x * std::cos(phi) + fr.b.x * std::sin(phi)) * rr,
               g.p0.y + (fr.t.y * std::cos(phi) + fr.b.y * std::sin(phi)) * rr,
               g.p0.z + (fr.t.z * std::cos(phi) + fr.b.z * std::sin(phi)) * rr};
        nS = g.axis;
      }
      const V3 d{S.x - P.x, S.y - P.y, S.z - P.z};
      const float dist2 = dot(d, d);
      if (dist2 <= 1.0e-12f) return zero;
      const float dist = std::sqrt(dist2);
      dir = V3{d.x / dist, d.y / dist, d.z / dist};
      const float cosL = std::fabs(dot(nS, dir));
      if (cosL <= 1.0e-6f) return zero;
      pdfSA = s.emPdf[lo] * dist2 / (cosL * g.area);
      target = dist;
    }
    const float cosP0 = dot(N, dir);
    if (cosP0 <= 0.0f) return zero;
    if (pdfSA <= 0.0f) return zero;
  }
  const float cosP = dot(N, dir);
  const float eps = selfIntersectEps(P, dir, epsT);
  V3 ng = (dot(Ng, N) < 0.0f) ? V3{-Ng.x, -Ng.y, -Ng.z} : Ng;
  ng = safeNormalize(ng, N);
  const V3 O{P.x + ng.x * eps, P.y + ng.y * eps, P.z + ng.z * eps};
  const float tf = target - 2.0f * eps;
  if (eps < tf && occludedQ(s, O, dir, eps, tf)) return zero;
  const float pdfCos = cosP * (1.0f / kPi);
  const float w = pdfSA / (pdfSA + pdfCos);
  const float k = w * cosP / (kPi * pdfSA);
  return V3{Le.x * k, Le.y * k, Le.z * k};
}

// pt2EmissiveHitWeight: the cosine side's balance weight of a first-bounce
// hit on an NEE-covered emitter; 1 otherwise
inline float emissiveHitWeight(const Scene& s, int kind, uint32_t prim, const V3& O, const V3& wi, float tfar,
                               float cosP, const V3& ngHit) {
  if (s.emEmpty()) return 1.0f;
  const float kPi = 3.14159265358979323846f;
  const float pdfCos = (cosP > 0.0f ? cosP : 0.0f) * (1.0f / kPi);
  if (pdfCos <= 0.0f) return 1.0f;
  const uint32_t triCount = static_cast<uint32_t>(s.emTris.size());
  if (kind == kMesh) {
    if (prim >= s.emTriIndex.size()) return 1.0f;
    const uint32_t ti = s.emTriIndex[prim];
    if (ti == 0xFFFFFFFFu) return 1.0f;
    const float cosL = std::fabs(dot(s.emTris[ti].ng, wi));
    const float pdfSA = emitPdfTri(s, ti, tfar * tfar, cosL);
    if (pdfSA <= 0.0f) return 1.0f;
    return pdfCos / (pdfCos + pdfSA);
  }
  if (kind == kSphere) {
    if (prim >= s.emSphereIndex.size()) return 1.0f;
    const uint32_t ci = s.emSphereIndex[prim];
    if (ci == 0xFFFFFFFFu) return 1.0f;
    const Scene::EmitCsg& g = s.emCsg[ci];
    const V3 d{g.p0.x - O.x, g.p0.y - O.y, g.p0.z - O.z};
    const float dc2 = dot(d, d);
    const float r2 = g.radius * g.radius;
    if (dc2 <= r2 * 1.0002f) return 1.0f;
    const float sin2Max = r2 / dc2;
    const float cosMax = std::sqrt(std::fmax(0.0f, 1.0f - sin2Max));
    const float oneMinusCos = sin2Max / (1.0f + cosMax);
    if (oneMinusCos <= 0.0f) return 1.0f;
    const float pdfSA = s.emPdf[triCount + ci] / (2.0f * kPi * oneMinusCos);
    if (pdfSA <= 0.0f) return 1.0f;
    return pdfCos / (pdfCos + pdfSA);
  }
  if (kind == kCone) {
    if (prim >= s.emCylIndex.size()) return 1.0f;
    const auto& ref = s.emCylIndex[prim];
    uint32_t part = ref[0];
    const uint32_t probe = ref[0] != 0xFFFFFFFFu ? ref[0] : ref[1] != 0xFFFFFFFFu ? ref[1] : ref[2];
    if (probe == 0xFFFFFFFFu) return 1.0f;
    const V3 axis = s.emCsg[probe].axis;
    const V3 ng = safeNormalize(ngHit, axis);
    const float nu = dot(ng, axis);
    if (nu >= 0.99f) part = ref[2];
    else if (nu <= -0.99f) part = ref[1];
    if (part == 0xFFFFFFFFu) return 1.0f;
    const float cosL = std::fabs(dot(ng, wi));
    if (cosL <= 1.0e-6f) return 1.0f;
    const float pdfSA = s.emPdf[triCount + part] * tfar * tfar / (cosL * s.emCsg[part].area);
    if (pdfSA <= 0.0f) return 1.0f;
    return pdfCos / (pdfCos + pdfSA);
  }
  return 1.0f;
}

// pt2's gather configuration at one point (Pt1GatherExt / Pt2GatherCfg)
// pt2_reservoir.hpp:36-42 Pt2Reservoir: one sample point (a first-bounce
// hit, or an anchor 1e7 along an escaped first segment), the full path
// radiance leaving it, the candidates it stands for (M) and its unbiased
// contribution weight W.
struct Reservoir {
  V3 pos{0.0f, 0.0f, 0.0f}, nrm{0.0f, 0.0f, 0.0f}, rad{0.0f, 0.0f, 0.0f};
  float M = 0.0f, W = 0.0f;
};
constexpr float kEnvAnchor = 1.0e7f;   // pt2_reservoir.hpp:33
constexpr float kPiF = 3.14159265358979323846f;
inline float lum3(const V3& c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; }
// pt2_reservoir.hpp:55-63 pt2TargetPdf: luminance times the receiver cosine
inline float targetPdf(const V3& P, const V3& N, const V3& sp, const V3& rad) {
  const V3 d{sp.x - P.x, sp.y - P.y, sp.z - P.z};
  const float l2 = dot(d, d);
  if (l2 <= 0.0f) return 0.0f;
  const float cs = dot(N, d) / std::sqrt(l2);
  if (cs <= 0.0f) return 0.0f;
  return lum3(rad) * cs;
}
// pt2_reservoir.hpp:72-89 pt2Jacobian: reconnection Jacobian of moving a
// sample's receiver, cosines at the sample's normal, clamped to [0, cap]
inline float reconnectJacobian(const V3& recvNew, const V3& recvOld, const V3& sp, const V3& sn, float cap) {
  const V3 a{recvNew.x - sp.x, recvNew.y - sp.y, recvNew.z - sp.z};
  const V3 b{recvOld.x - sp.x, recvOld.y - sp.y, recvOld.z - sp.z};
  const float ra2 = dot(a, a), rb2 = dot(b, b);
  if (ra2 <= 0.0f || rb2 <= 0.0f) return 0.0f;
  const float ca = dot(sn, a) / std::sqrt(ra2);
  const float cb = dot(sn, b) / std::sqrt(rb2);
  if (ca <= 0.0f || cb <= 0.0f) return 0.0f;
  const float j = (rb2 * ca) / (ra2 * cb);
  if (!std::isfinite(j) || j < 0.0f) return 0.0f;
  return j > cap ? cap : j;
}
// pt2_reservoir.hpp:94-99 pt2ReservoirUpdate: the streaming selection rule
inline bool reservoirTake(double& wSum, float& M, float w, float m, float u) {
  wSum += static_cast<double>(w);
  M += m;
  return w > 0.0f && static_cast<double>(u) * wSum <= static_cast<double>(w);
}

struct GatherExt {
  bool pt2 = false;
  uint32_t idxBase = 0, seed = 0;  // the point's Sobol section / scramble seed
  int sampleOffset = 0;
  V3* halfSum = nullptr;
  Reservoir* rsv = nullptr;        // ReSTIR candidate reservoir of the point, or null
};

// pt1_gather.hpp:268-523 pt1GatherPoint: E_stored = (1/spp) sum over
// cosine-hemisphere paths of the NEE radiance at each vertex and the sky
// where the path escapes; Russian roulette from the second vertex on.  With
// pt2 (ext): the first bounce from the scrambled Sobol point, the path's
// stream drives area-light jitter, vertices add their MIS-weighted emission,
// and each sample adds one emissive NEE draw at the origin.
inline V3 pt1GatherPoint(const Ctx& c, const V3& P, const V3& N, const V3& Ng, uint32_t seed, float epsT, int spp,
                         float* occOut, const GatherExt* ext = nullptr) {
  const Scene& s = *c.s;
  int nOcc = 0;
  const Frame f = frameFromNormal(N);
  const float eps = selfIntersectEps(P, N, epsT);
  const V3 O{P.x + N.x * eps, P.y + N.y * eps, P.z + N.z * eps};
  const int maxB = c.o.giBounces < 1 ? 1 : c.o.giBounces;
  const float maxD = c.o.giMaxDistance > 0.0f ? c.o.giMaxDistance : kInf;
  const bool pt2 = ext && ext->pt2;
  const bool emitNee = pt2 && c.o.pt2Emissive && c.o.pt2EmissiveNee && !s.emEmpty();
  const int sOff = ext ? ext->sampleOffset : 0;
  float cpx = 0.0f, cpy = 0.0f;
  if (c.o.pt1Ld) {
    uint32_t c0 = seed, c1 = 0x9E3779B9u;
    tea2(c0, c1);
    cpx = u32ToUnorm(c0);
    cpy = u32ToUnorm(c1);
  }
  V3 Esum{0.0f, 0.0f, 0.0f};
  // ReSTIR creation stage (pt1_gather.hpp:287-297, 451-470, 486-499): every
  // sample is one candidate streamed into the point's reservoir with RIS
  // weight pi * lum(L) (p_hat = lum(L) cos over the cosine pdf), selected by
  // its own tea2 chain
  Reservoir* rsv = ext ? ext->rsv : nullptr;
  uint32_t rs0 = 0, rs1 = 0;
  double rWSum = 0.0;
  V3 rPos{0.0f, 0.0f, 0.0f}, rNrm{0.0f, 0.0f, 0.0f}, rRad{0.0f, 0.0f, 0.0f};
  float rPHat = 0.0f;
  if (rsv) {
    rs0 = seed ^ 0x52455354u;
    rs1 = 0x47490001u;
  }
  for (int sI = 0; sI < spp; ++sI) {
    uint32_t s0 = seed, s1 = static_cast<uint32_t>(sI + sOff);
    tea2(s0, s1);
    float u1, u2;
    if (pt2) {
      sobol2D(ext->idxBase + static_cast<uint32_t>(sI + sOff), ext->seed, u1, u2);
    } else if (c.o.pt1Ld) {
      u1 = static_cast<float>(sI) / static_cast<float>(spp) + cpx;
      u2 = radicalInverse2(static_cast<uint32_t>(sI)) + cpy;
      if (u1 >= 1.0f) u1 -= 1.0f;
      if (u2 >= 1.0f) u2 -= 1.0f;
    } else {
      u1 = u32ToUnorm(s0);
      u2 = u32ToUnorm(s1);
    }
    V3 wi = cosineSampleHemisphere(u1, u2, f);
    const bool horizonOk = dot(wi, Ng) > 0.0f;
    if (!horizonOk) ++nOcc;
    const float cand0Cos = dot(wi, N);
    V3 org = O;
    float tnear = eps;
    V3 thr{1.0f, 1.0f, 1.0f}, L{0.0f, 0.0f, 0.0f};
    V3 candPos{0.0f, 0.0f, 0.0f}, candN{0.0f, 0.0f, 0.0f};
    bool candValid = false;
    for (int b = 1; horizonOk && b <= maxB; ++b) {
      Ray r;
      r.org = org; r.dir = wi; r.tnear = tnear; r.tfar = maxD;
      Hit h;
      if (!s.bvh.closest(r, h)) {
        const V3 env = pt1Environment(c, wi);
        L.x += thr.x * env.x;
        L.y += thr.y * env.y;
        L.z += thr.z * env.z;
        if (rsv && b == 1) {  // escaped: the candidate sits far along the segment
          candPos = V3{O.x + wi.x * kEnvAnchor, O.y + wi.y * kEnvAnchor, O.z + wi.z * kEnvAnchor};
          candN = V3{-wi.x, -wi.y, -wi.z};
          candValid = true;
        }
        break;
      }
      if (b == 1) ++nOcc;
      V3 rad, alb, Py, Ny, em{0.0f, 0.0f, 0.0f};
      if (!pt1EvalVertex(c, h, org, wi, rad, alb, Py, Ny, pt2 && c.o.pt2Emissive, pt2 ? &s0 : nullptr,
                         pt2 ? &s1 : nullptr, &em)) {
        if (rsv && b == 1) {  // absorbed by an outline: a zero-radiance candidate at the hit
          candPos = V3{org.x + wi.x * h.t, org.y + wi.y * h.t, org.z + wi.z * h.t};
          candN = V3{-wi.x, -wi.y, -wi.z};
          candValid = true;
        }
        break;
      }
      if (rsv && b == 1) {
        candPos = Py;
        candN = Ny;
        candValid = true;
      }
      float emW = 1.0f;
      if (emitNee && b == 1)
        emW = emissiveHitWeight(s, kindOfGeom(s, h.geomID), h.primID, org, wi, h.t, cand0Cos, h.Ng);
      L.x += thr.x * (rad.x + emW * em.x);
      L.y += thr.y * (rad.y + emW * em.y);
      L.z += thr.z * (rad.z + emW * em.z);
      if (b == maxB) break;
      thr.x *= alb.x;
      thr.y *= alb.y;
      thr.z *= alb.z;
      if (b >= 2) {
        tea2(s0, s1);
        float pc = std::fmax(thr.x, std::fmax(thr.y, thr.z));
        pc = std::fmin(0.95f, std::fmax(0.05f, pc));
        if (u32ToUnorm(s0) >= pc) break;
        const float inv = 1.0f / pc;
        thr.x *= inv;
        thr.y *= inv;
        thr.z *= inv;
      }
      tea2(s0, s1);
      const Frame fv = frameFromNormal(Ny);
      wi = cosineSampleHemisphere(u32ToUnorm(s0), u32ToUnorm(s1), fv);
      const float epsV = selfIntersectEps(Py, wi, h.t);
      org = V3{Py.x + Ny.x * epsV, Py.y + Ny.y * epsV, Py.z + Ny.z * epsV};
      tnear = epsV;
    }
    if (emitNee) {
      const V3 e = emissiveNee(s, P, N, Ng, epsT, s0, s1);
      L.x += e.x;
      L.y += e.y;
      L.z += e.z;
    }
    if (c.o.pt1Clamp > 0.0f) {
      const float lum = 0.2126f * L.x + 0.7152f * L.y + 0.0722f * L.z;
      if (lum > c.o.pt1Clamp) {
        const float k = c.o.pt1Clamp / lum;
        L.x *= k;
        L.y *= k;
        L.z *= k;
      }
    }
    if (rsv) {
      float w = 0.0f, pHat = 0.0f;
      if (candValid && cand0Cos > 0.0f) {
        pHat = lum3(L) * cand0Cos;
        w = lum3(L) * kPiF;
      }
      tea2(rs0, rs1);
      float unusedM = 0.0f;
      if (reservoirTake(rWSum, unusedM, w, 0.0f, u32ToUnorm(rs0))) {
        rPos = candPos;
        rNrm = candN;
        rRad = L;
        rPHat = pHat;
      }
    }
    Esum.x += L.x;
    Esum.y += L.y;
    Esum.z += L.z;
    if (ext && ext->halfSum && sI < spp / 2) {
      ext->halfSum->x += L.x;
      ext->halfSum->y += L.y;
      ext->halfSum->z += L.z;
    }
  }
  if (rsv) {  // W = wSum / (M p_hat(selected)), M = every candidate
    rsv->pos = rPos;
    rsv->nrm = rNrm;
    rsv->rad = rRad;
    rsv->M = static_cast<float>(spp > 0 ? spp : 1);
    rsv->W = (rPHat > 0.0f && rWSum > 0.0)
                 ? static_cast<float>(rWSum / (static_cast<double>(rsv->M) * static_cast<double>(rPHat)))
                 : 0.0f;
  }
  const float invN = 1.0f / static_cast<float>(spp > 0 ? spp : 1);
  if (occOut) *occOut = static_cast<float>(nOcc) * invN;
  return V3{Esum.x * invN, Esum.y * invN, Esum.z * invN};
}

inline PixelOut integratePixel(const Ctx& c, const V3& org, const V3& rd, uint32_t px, uint32_t py,
                               const V3& camDir) {
  PixelOut po{};
  po.first.group = -1;  // background sentinel (transparency.hpp:337)
  po.geom = kInvalid;
  po.prim = kInvalid;
  V3 Cf{0.0f, 0.0f, 0.0f};
  float Af = 0.0f, nearDepth = 0.0f, firstViewZ = 0.0f;
  V3 base = c.bg;
  float baseCov = c.o.transparentBackground ? 0.0f : 1.0f;
  // clipRangeT (transparency.hpp:118-129)
  float ctn = 0.0f, ctf = kInf;
  bool clipOn = false;
  if (!(c.clipNear <= -kInf && c.clipFar >= kInf)) {
    const float cosr = dot(rd, camDir);
    if (!(cosr <= 1.0e-6f)) {
      clipOn = true;
      if (c.clipNear > 0.0f) ctn = c.clipNear / cosr;
      if (c.clipFar < kInf) ctf = c.clipFar / cosr;
    }
  }
  const float kOpaque = 1.0f - 1e-4f;
  float tnear = ctn;
  const int maxIters = c.o.transparency ? (c.o.maxTransparentLayers + 1) : 1;
  for (int iter = 0; iter < maxIters; ++iter) {
    Ray r;
    r.org = org; r.dir = rd; r.tnear = tnear; r.tfar = ctf;
    Hit h;
    ++po.rays;
    if (!c.s->bvh.closest(r, h)) break;
    const HitShade hs = shadeHit(c, h, rd, org, px, py);
    if (nearDepth == 0.0f) {
      nearDepth = h.t;
      firstViewZ = h.t * dot(rd, camDir);
      po.geom = h.geomID;
      po.prim = h.primID;
      po.first = hs;
      po.firstPos = V3{org.x + rd.x * h.t, org.y + rd.y * h.t, org.z + rd.z * h.t};
      // a backface first hit whose clipped-away front exists (:424-428)
      if (clipOn && ctn > 0.0f && c.o.edgeGbuffer && dot(h.Ng, rd) > 0.0f &&
          clipConfirmFront(*c.s, org, rd, ctn))
        po.clipCut = 1;
    }
    if (!c.o.transparency || hs.opacity >= kOpaque) {
      base = hs.color;
      baseCov = 1.0f;
      break;
    }
    const float w = (1.0f - Af) * hs.opacity;
    Cf.x += w * hs.color.x;
    Cf.y += w * hs.color.y;
    Cf.z += w * hs.color.z;
    Af += w;
    if (Af >= kOpaque) break;
    const V3 hitP{org.x + rd.x * h.t, org.y + rd.y * h.t, org.z + rd.z * h.t};
    const float dirMax = std::fmax(std::fabs(rd.x), std::fmax(std::fabs(rd.y), std::fabs(rd.z)));
    const float epsScale = std::fmax(std::fmax(std::fabs(hitP.x), std::fabs(hitP.y)),
                                     std::fmax(std::fabs(hitP.z), dirMax * h.t));
    tnear = h.t + epsScale * 0x1.0fp-21f;
    if (iter == maxIters - 1) po.capped = true;
  }
  // background under clipping: what the planes removed along the ray (:470-481)
  if (clipOn && c.o.edgeGbuffer && nearDepth == 0.0f) {
    if (ctn > 0.0f)
      po.clipNearVz = clipProbeRange(*c.s, org, rd, camDir, std::max(1.0e-4f, 1.0e-6f * ctn), ctn * (1.0f - 1.0e-6f));
    if (ctf < kInf) po.clipFarVz = clipProbeRange(*c.s, org, rd, camDir, ctf * (1.0f + 1.0e-6f), kInf);
  }
  const float floorW = (1.0f - Af) * baseCov;
  float outA = Af + floorW;
  outA = std::fmin(1.0f, std::fmax(0.0f, outA));
  po.r = Cf.x + floorW * base.x;
  po.g = Cf.y + floorW * base.y;
  po.b = Cf.z + floorW * base.z;
  po.a = outA;
  po.depth = nearDepth;
  po.viewZ = firstViewZ;
  return po;
}

}  // namespace
}  // namespace oracle

using namespace oracle;

// Centre record of one output pixel for the adaptive-AA mask: colour before
// fog, view z, first-hit geomID / section (background: kInvalid / -1) and
// shading normal (zero when the path leaves it unset).
struct AaCentre {
  float r, g, b, a, viewZ;
  uint32_t geom;
  int group;
  V3 normal;
};

// aaPairNeedsRefine (adaptive_aa.hpp:65-111) with the default AaMaskParams
// (normal delta 0.3, depth factor 3, absolute floor 12 output pixels).
inline bool aaPairRefine(const AaCentre& a, const AaCentre& b, float za0, float zb1, float thr,
                         float pixelWorldSize, bool persp) {
  if (a.geom != b.geom || a.group != b.group) return true;
  if (std::fabs(a.r - b.r) > thr || std::fabs(a.g - b.g) > thr || std::fabs(a.b - b.b) > thr ||
      std::fabs(a.a - b.a) > thr)
    return true;
  if (a.geom == kInvalid || b.geom == kInvalid) return false;
  const V3 na = a.normal, nb = b.normal;
  const float la = na.x * na.x + na.y * na.y + na.z * na.z;
  const float lb = nb.x * nb.x + nb.y * nb.y + nb.z * nb.z;
  if (la > 0.0f && lb > 0.0f) {
    const float dd = na.x * nb.x + na.y * nb.y + na.z * nb.z;
    if (1.0f - dd > 0.3f) return true;
  }
  const float step = std::fabs(b.viewZ - a.viewZ);
  const float sa = std::fabs(a.viewZ - za0);
  const float sb = std::fabs(zb1 - b.viewZ);
  const float slope = sa < sb ? sa : sb;
  float absTerm = 12.0f * pixelWorldSize;
  if (persp) {
    const float zmin = std::fabs(a.viewZ) < std::fabs(b.viewZ) ? std::fabs(a.viewZ) : std::fabs(b.viewZ);
    absTerm *= zmin;
  }
  const float th = 3.0f * slope > absTerm ? 3.0f * slope : absTerm;
  return step > th;
}

// buildAaMask (adaptive_aa.hpp:121-161, edges mode off): horizontal then
// vertical pairs with the outer view z (linear extrapolation at the border),
// then dilateMask3x3 (:35-56).
inline void buildAaMask(int Wf, int Hf, const AaCentre* c, float thr, float pixelWorldSize, bool persp,
                        uint8_t* mask) {
  auto at = [&](int x, int y) -> const AaCentre& { return c[static_cast<size_t>(y) * Wf + x]; };
  std::vector<uint8_t> raw(static_cast<size_t>(Wf) * Hf, 0);
  for (int y = 0; y < Hf; ++y)
    for (int x = 0; x + 1 < Wf; ++x) {
      const AaCentre &a = at(x, y), &b = at(x + 1, y);
      const float za0 = x > 0 ? at(x - 1, y).viewZ : 2.0f * a.viewZ - b.viewZ;
      const float zb1 = x + 2 < Wf ? at(x + 2, y).viewZ : 2.0f * b.viewZ - a.viewZ;
      if (aaPairRefine(a, b, za0, zb1, thr, pixelWorldSize, persp))
        raw[size_t(y) * Wf + x] = raw[size_t(y) * Wf + x + 1] = 1;
    }
  for (int y = 0; y + 1 < Hf; ++y)
    for (int x = 0; x < Wf; ++x) {
      const AaCentre &a = at(x, y), &b = at(x, y + 1);
      const float za0 = y > 0 ? at(x, y - 1).viewZ : 2.0f * a.viewZ - b.viewZ;
      const float zb1 = y + 2 < Hf ? at(x, y + 2).viewZ : 2.0f * b.viewZ - a.viewZ;
      if (aaPairRefine(a, b, za0, zb1, thr, pixelWorldSize, persp))
        raw[size_t(y) * Wf + x] = raw[size_t(y + 1) * Wf + x] = 1;
    }
  for (int y = 0; y < Hf; ++y)
    for (int x = 0; x < Wf; ++x) {
      uint8_t v = 0;
      for (int dy = -1; dy <= 1 && !v; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int xx = x + dx, yy = y + dy;
          if (xx < 0 || yy < 0 || xx >= Wf || yy >= Hf) continue;
          if (raw[size_t(yy) * Wf + xx]) {
            v = 1;
            break;
          }
        }
      mask[size_t(y) * Wf + x] = v;
    }
}

// experimental/irradiance_cache/denoise_atrous.cpp:27-220 denoiseAtrous on the
// final-resolution linear colour (4 floats per pixel): edge-avoiding a-trous
// wavelet (B3 spline, 2^i hole spacing) with normal, luminance-variance and
// (GI only, absent here) position edge-stops; illumination demodulated by the
// albedo when given.  normal / albedo: 3 floats per pixel.
inline void denoiseAtrous(int W, int H, float* color, const float* normal, const float* albedo, int iters,
                          float sigmaNIn, float sigmaLIn, const float* position = nullptr, float sigmaZIn = 1.0f) {
  const size_t N = static_cast<size_t>(W) * H;
  if (W <= 0 || H <= 0 || iters <= 0 || normal == nullptr) return;
  const float kEps = 1.0e-3f;
  auto luminance = [](float r, float g, float b) { return 0.2126f * r + 0.7152f * g + 0.0722f * b; };
  const float sigmaN = sigmaNIn;
  const float sigmaL = std::max(1.0e-4f, sigmaLIn);
  const float sigmaZ = std::max(1.0e-4f, sigmaZIn);
  std::vector<unsigned char> valid(N, 0);
  for (size_t p = 0; p < N; ++p) {
    const float nx = normal[p * 3], ny = normal[p * 3 + 1], nz = normal[p * 3 + 2];
    valid[p] = (nx * nx + ny * ny + nz * nz) > 0.25f ? 1 : 0;
  }
  std::vector<float> irr(N * 3);
  for (size_t p = 0; p < N; ++p)
    for (int c = 0; c < 3; ++c) {
      float v = color[p * 4 + c];
      if (albedo) {
        const float a = albedo[p * 3 + c];
        v /= (a > kEps ? a : kEps);
      }
      irr[p * 3 + c] = v;
    }
  // position guide: the largest step to a valid 4-neighbour (floor kEps)
  std::vector<float> posGrad;
  if (position) {
    posGrad.assign(N, kEps);
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const size_t p = static_cast<size_t>(y) * W + x;
        if (!valid[p]) continue;
        const V3 pp{position[p * 3], position[p * 3 + 1], position[p * 3 + 2]};
        float g = kEps;
        const int nb[4][2] = {{1, 0}, {-1, 0}, {0, 1}, {0, -1}};
        for (auto& dd : nb) {
          const int qx = x + dd[0], qy = y + dd[1];
          if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
          const size_t q = static_cast<size_t>(qy) * W + qx;
          if (!valid[q]) continue;
          const V3 pq{position[q * 3], position[q * 3 + 1], position[q * 3 + 2]};
          g = std::max(g, length(pp - pq));
        }
        posGrad[p] = g;
      }
  }
  std::vector<float> var(N, 0.0f);
  for (int y = 0; y < H; ++y)
    for (int x = 0; x < W; ++x) {
      const size_t p = static_cast<size_t>(y) * W + x;
      if (!valid[p]) continue;
      float sm = 0.0f, s2 = 0.0f;
      int n = 0;
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int qx = x + dx, qy = y + dy;
          if (qx < 0 || qx >= W || qy < 0 || qy >= H) continue;
          const size_t q = static_cast<size_t>(qy) * W + qx;
          if (!valid[q]) continue;
          const float l = luminance(irr[q * 3], irr[q * 3 + 1], irr[q * 3 + 2]);
          sm += l;
          s2 += l * l;
          ++n;
        }
      if (n > 0) {
        const float mean = sm / n;
        var[p] = std::max(0.0f, s2 / n - mean * mean);
      }
    }
  const float h5[5] = {0.0625f, 0.25f, 0.375f, 0.25f, 0.0625f};
  std::vector<float> next(N * 3), lum(N);
  for (int it = 0; it < iters; ++it) {
    const int step = 1 << it;
    for (size_t p = 0; p < N; ++p) lum[p] = luminance(irr[p * 3], irr[p * 3 + 1], irr[p * 3 + 2]);
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        const size_t p = static_cast<size_t>(y) * W + x;
        if (!valid[p]) {
          for (int c = 0; c < 3; ++c) next[p * 3 + c] = irr[p * 3 + c];
          continue;
        }
        const V3 np{normal[p * 3], normal[p * 3 + 1], normal[p * 3 + 2]};
        const V3 pp = position ? V3{position[p * 3], position[p * 3 + 1], position[p * 3 + 2]} : V3{0, 0, 0};
        const float lp = lum[p];
        const float lDenom = sigmaL * std::sqrt(var[p]) + kEps;
        const float zDenom = position ? (sigmaZ * posGrad[p] * step + kEps) : 1.0f;
        float sum[3] = {0.0f, 0.0f, 0.0f};
        float wsum = 0.0f;
        for (int dy = -2; dy <= 2; ++dy) {
          const int qy = y + dy * step;
          if (qy < 0 || qy >= H) continue;
          for (int dx = -2; dx <= 2; ++dx) {
            const int qx = x + dx * step;
            if (qx < 0 || qx >= W) continue;
            const size_t q = static_cast<size_t>(qy) * W + qx;
            if (!valid[q]) continue;
            float w = h5[dx + 2] * h5[dy + 2];
            const V3 nq{normal[q * 3], normal[q * 3 + 1], normal[q * 3 + 2]};
            const float nd = std::max(0.0f, dot(np, nq));
            w *= std::pow(nd, sigmaN);
            if (position) {
              const V3 pq{position[q * 3], position[q * 3 + 1], position[q * 3 + 2]};
              w *= std::exp(-length(pp - pq) / zDenom);
            }
            w *= std::exp(-std::fabs(lp - lum[q]) / lDenom);
            sum[0] += w * irr[q * 3];
            sum[1] += w * irr[q * 3 + 1];
            sum[2] += w * irr[q * 3 + 2];
            wsum += w;
          }
        }
        for (int c = 0; c < 3; ++c) next[p * 3 + c] = wsum > 0.0f ? sum[c] / wsum : irr[p * 3 + c];
      }
    irr.swap(next);
  }
  for (size_t p = 0; p < N; ++p) {
    if (!valid[p]) continue;
    for (int c = 0; c < 3; ++c) {
      float v = irr[p * 3 + c];
      if (albedo) v *= albedo[p * 3 + c];
      color[p * 4 + c] = std::max(0.0f, v);
    }
  }
}

// Runs fn(row) for rows [0, n) on nt threads (rows handed out one at a time).
inline void forRows(int n, int nt, const std::function<void(int)>& fn) {
  std::atomic<int> next{0};
  auto w = [&]() {
    for (int y = next.fetch_add(1); y < n; y = next.fetch_add(1)) fn(y);
  };
  std::vector<std::thread> pool;
  for (int i = 1; i < nt; ++i) pool.emplace_back(w);
  w();
  for (auto& th : pool) th.join();
}

// The camera basis of the render grid (Pt1CameraBasis, pt1_gbuffer.hpp:33-42).
struct Cam {
  V3 pos, dir, right, up;
  bool ortho;
  float halfW, halfH, persHalfW, persHalfH;
};

// A gather grid's first hits (Pt1GBuffer, pt1_gbuffer.hpp:70-80).
struct GiGrid {
  int w = 0, h = 0;
  std::vector<float> pos, nrm, gnrm, dep;
  std::vector<uint8_t> hit;
};

// pt1_gbuffer.hpp:83-196 tracePt1GBuffer: one primary ray per point of a
// w x h grid over the render grid's image plane, closest hit in [0, inf):
// mesh hits take the interpolated vertex normal, real primitives their
// geometric normal; both normals face the viewer; outline primitives and
// misses stay zero.
inline void tracePt1GBuffer(const Ctx& c, const Cam& cam, int w, int h, GiGrid& g, int nt) {
  const Scene& s = *c.s;
  const size_t n = static_cast<size_t>(w) * h;
  g.w = w;
  g.h = h;
  g.pos.assign(n * 3, 0.0f);
  g.nrm.assign(n * 3, 0.0f);
  g.gnrm.assign(n * 3, 0.0f);
  g.dep.assign(n, 0.0f);
  g.hit.assign(n, 0);
  forRows(h, nt, [&](int py) {
    const float v = 1.0f - 2.0f * (static_cast<float>(py) + 0.5f) / static_cast<float>(h);
    for (int px = 0; px < w; ++px) {
      const float u = 2.0f * (static_cast<float>(px) + 0.5f) / static_cast<float>(w) - 1.0f;
      V3 org, rd;
      if (cam.ortho) {
        org = cam.pos + cam.right * (u * cam.halfW) + cam.up * (v * cam.halfH);
        rd = cam.dir;
      } else {
        org = cam.pos;
        rd = normalize(cam.dir + cam.right * (u * cam.persHalfW) + cam.up * (v * cam.persHalfH));
      }
      Ray r;
      r.org = org; r.dir = rd; r.tnear = 0.0f; r.tfar = kInf;
      Hit hh;
      if (!s.bvh.closest(r, hh)) continue;
      const int kind = kindOfGeom(s, hh.geomID);
      V3 N, Ng;
      if (kind == kMesh) {
        const uint32_t* tri = &s.geo.triIdx[3 * hh.primID];
        const float w0 = 1.0f - hh.u - hh.v;
        float nb[3];
        for (int k = 0; k < 3; ++k)
          nb[k] = w0 * s.nrm[3 * tri[0] + k] + hh.u * s.nrm[3 * tri[1] + k] + hh.v * s.nrm[3 * tri[2] + k];
        N = safeNormalize(V3{nb[0], nb[1], nb[2]});
        Ng = safeNormalize(hh.Ng);
      } else {
        if (s.fromEdge[kind][hh.primID]) continue;
        N = safeNormalize(hh.Ng);
        Ng = N;
      }
      if (dot(N, rd) > 0.0f) N = V3{-N.x, -N.y, -N.z};
      if (dot(Ng, rd) > 0.0f) Ng = V3{-Ng.x, -Ng.y, -Ng.z};
      const size_t pix = static_cast<size_t>(py) * w + px;
      const V3 P{org.x + rd.x * hh.t, org.y + rd.y * hh.t, org.z + rd.z * hh.t};
      g.pos[3 * pix] = P.x; g.pos[3 * pix + 1] = P.y; g.pos[3 * pix + 2] = P.z;
      g.nrm[3 * pix] = N.x; g.nrm[3 * pix + 1] = N.y; g.nrm[3 * pix + 2] = N.z;
      g.gnrm[3 * pix] = Ng.x; g.gnrm[3 * pix + 1] = Ng.y; g.gnrm[3 * pix + 2] = Ng.z;
      g.dep[pix] = hh.t;
      g.hit[pix] = 1;
    }
  });
}

// pt1_gather.hpp:525-614 gatherPt1Grid: E and the first-bounce hit fraction
// at every marked point of a W x H grid, seeded hashU32(pix ^
// hashU32(pt1Seed)); the primary hit distance scales the origin epsilon;
// gnrm null: the shading normal is the horizon normal.  pt2 (pt2.pt2): each
// point's sampler (pt2MakePixelSampler: blue-noise section of length sppPow2
// along the scrambled Morton curve, or its own sequence), the sample offset
// of a refinement pass, and the half sums for adaptive spp.
struct GridPt2 {
  bool pt2 = false;
  uint32_t sppPow2 = 1;
  int sampleOffset = 0;
  std::vector<float>* halfE = nullptr;
  std::vector<Reservoir>* rsv = nullptr;  // ReSTIR: one reservoir per grid point
};
inline void gatherGrid(const Ctx& c, int W, int H, const float* pos, const float* nrm, const float* gnrm,
                       const uint8_t* mark, const float* dep, int spp, std::vector<float>& E,
                       std::vector<float>& occ, int nt, const GridPt2& g2 = GridPt2()) {
  const size_t n = static_cast<size_t>(W) * H;
  E.assign(n * 3, 0.0f);
  occ.assign(n, 0.0f);
  if (g2.halfE) g2.halfE->assign(n * 3, 0.0f);
  if (g2.rsv) g2.rsv->assign(n, Reservoir{});
  const uint32_t seedMix = hashU32(c.o.pt1Seed);
  forRows(H, nt, [&](int py) {
    for (int px = 0; px < W; ++px) {
      const size_t pix = static_cast<size_t>(py) * W + px;
      if (!mark[pix]) continue;
      const V3 P{pos[3 * pix], pos[3 * pix + 1], pos[3 * pix + 2]};
      const V3 N{nrm[3 * pix], nrm[3 * pix + 1], nrm[3 * pix + 2]};
      const V3 Ng = gnrm ? V3{gnrm[3 * pix], gnrm[3 * pix + 1], gnrm[3 * pix + 2]} : N;
      const uint32_t seed = hashU32(static_cast<uint32_t>(pix) ^ seedMix);
      const float tEps = dep[pix] > 0.0f ? dep[pix] : 1.0f;
      float o = 0.0f;
      GatherExt ext;
      V3 half{0.0f, 0.0f, 0.0f};
      if (g2.pt2) {
        ext.pt2 = true;
        if (c.o.pt2Pattern == 1) {
          const uint32_t morton = (expandBits16(static_cast<uint32_t>(px)) << 1) |
                                  expandBits16(static_cast<uint32_t>(py));
          ext.idxBase = reverseBits(owenHashBase4(reverseBits(morton), seedMix)) * g2.sppPow2;
          ext.seed = seedMix;
        } else {
          ext.idxBase = 0;
          ext.seed = seed;
        }
        ext.sampleOffset = g2.sampleOffset;
        if (g2.halfE) ext.halfSum = &half;
        if (g2.rsv) ext.rsv = &(*g2.rsv)[pix];
      }
      const V3 e = pt1GatherPoint(c, P, N, Ng, seed, tEps, spp, &o, g2.pt2 ? &ext : nullptr);
      E[3 * pix] = e.x; E[3 * pix + 1] = e.y; E[3 * pix + 2] = e.z;
      occ[pix] = o;
      if (g2.halfE) {
        (*g2.halfE)[3 * pix] = half.x; (*g2.halfE)[3 * pix + 1] = half.y; (*g2.halfE)[3 * pix + 2] = half.z;
      }
    }
  });
}

// pt2_adaptive.hpp:30-121: refinement mask (|lum(E) - lum(halfSum)/(spp/2)|
// above threshold x sqrt(lum) for dark points, x lum otherwise; every point
// when spp < 2), one 3x3 dilation, and the weighted-mean merge
inline void adaptiveMask(int W, int H, const std::vector<float>& E, const std::vector<float>& halfE,
                         const uint8_t* elig, int spp, float threshold, std::vector<uint8_t>& mask) {
  const size_t n = static_cast<size_t>(W) * H;
  mask.assign(n, 0);
  const int nHalf = spp / 2;
  if (nHalf < 1) {
    for (size_t i = 0; i < n; ++i) mask[i] = elig[i] ? 1 : 0;
    return;
  }
  const float invHalf = 1.0f / static_cast<float>(nHalf);
  for (size_t p = 0; p < n; ++p) {
    if (!elig[p]) continue;
    const float lumA = 0.2126f * E[3 * p] + 0.7152f * E[3 * p + 1] + 0.0722f * E[3 * p + 2];
    const float lumH = (0.2126f * halfE[3 * p] + 0.7152f * halfE[3 * p + 1] + 0.0722f * halfE[3 * p + 2]) * invHalf;
    const float diff = std::fabs(lumA - lumH);
    const float norm = lumA < 1.0f ? std::sqrt(std::fmax(lumA, 1.0e-4f)) : lumA;
    if (diff > threshold * norm) mask[p] = 1;
  }
}
inline void dilateMask(int W, int H, const std::vector<uint8_t>& in, const uint8_t* elig, std::vector<uint8_t>& out) {
  out.assign(in.size(), 0);
  for (int py = 0; py < H; ++py)
    for (int px = 0; px < W; ++px) {
      const size_t pix = static_cast<size_t>(py) * W + px;
      if (!elig[pix]) continue;
      uint8_t v = in[pix];
      for (int dy = -1; dy <= 1 && !v; ++dy) {
        const int ny = py + dy;
        if (ny < 0 || ny >= H) continue;
        for (int dx = -1; dx <= 1 && !v; ++dx) {
          const int nx = px + dx;
          if (nx < 0 || nx >= W) continue;
          v = in[static_cast<size_t>(ny) * W + nx];
        }
      }
      out[pix] = v;
    }
}

// pt1_denoise.cpp:20-80 denoisePt1E without OIDN: non-finite E scrubbed to
// zero, then the a-trous filter on E (alpha 1) with the normal and position
// guides and no albedo demodulation.
inline void denoisePt1E(int w, int h, std::vector<float>& E, const float* nrm, const float* pos, const Opt& o) {
  const size_t n = static_cast<size_t>(w) * h;
  for (float& v : E)
    if (!std::isfinite(v)) v = 0.0f;
  std::vector<float> rgba(n * 4);
  for (size_t p = 0; p < n; ++p) {
    rgba[4 * p] = E[3 * p]; rgba[4 * p + 1] = E[3 * p + 1]; rgba[4 * p + 2] = E[3 * p + 2]; rgba[4 * p + 3] = 1.0f;
  }
  denoiseAtrous(w, h, rgba.data(), nrm, nullptr, std::max(0, o.denoiseIters), o.denoiseSigmaN, o.denoiseSigmaL,
                pos, o.denoiseSigmaZ);
  for (size_t p = 0; p < n; ++p) {
    E[3 * p] = rgba[4 * p]; E[3 * p + 1] = rgba[4 * p + 1]; E[3 * p + 2] = rgba[4 * p + 2];
  }
}

// pt1_upsample.hpp:40-199 upsampleJointBilateral: E and the hit fraction of
// every eligible render-grid pixel from the 2x2 gather points around its
// centre (bilinear x max(0, N.Nh)^normalPow x exp(-|z - zh| / (depthScale z +
// 1e-6))); dead weights fall back to the quad's nearest valid point, then
// (fallbackR > 0) the window's; patch marks dead or weak (below thresh) pixels.
inline void upsampleJointBilateral(int W, int H, const float* fnrm, const float* fdep, const uint8_t* felig,
                                   const GiGrid& lo, const std::vector<float>& Elo, const std::vector<float>& occLo,
                                   float normalPow, float depthScale, int fallbackR, std::vector<float>& E,
                                   std::vector<float>& occ, std::vector<uint8_t>* patch, float thresh) {
  const size_t n = static_cast<size_t>(W) * H;
  E.assign(n * 3, 0.0f);
  occ.assign(n, 0.0f);
  if (patch) patch->assign(n, 0);
  const int hw = lo.w, hh = lo.h;
  for (int py = 0; py < H; ++py) {
    const float sy = (static_cast<float>(py) + 0.5f) * hh / H - 0.5f;
    const int by = static_cast<int>(std::floor(sy));
    const float fy = sy - static_cast<float>(by);
    for (int px = 0; px < W; ++px) {
      const size_t pix = static_cast<size_t>(py) * W + px;
      if (!felig[pix]) continue;
      const float sx = (static_cast<float>(px) + 0.5f) * hw / W - 0.5f;
      const int bx = static_cast<int>(std::floor(sx));
      const float fx = sx - static_cast<float>(bx);
      const V3 Nf{fnrm[3 * pix], fnrm[3 * pix + 1], fnrm[3 * pix + 2]};
      const float zf = fdep[pix];
      float wSum = 0.0f, oSum = 0.0f, bestBilin = -1.0f;
      V3 eSum{0.0f, 0.0f, 0.0f};
      long bestPix = -1;
      for (int dy = 0; dy < 2; ++dy)
        for (int dx = 0; dx < 2; ++dx) {
          const int hx = std::min(std::max(bx + dx, 0), hw - 1), hy = std::min(std::max(by + dy, 0), hh - 1);
          const size_t hp = static_cast<size_t>(hy) * hw + hx;
          if (!lo.hit[hp]) continue;
          const float wb = (dx ? fx : 1.0f - fx) * (dy ? fy : 1.0f - fy);
          if (wb > bestBilin) {
            bestBilin = wb;
            bestPix = static_cast<long>(hp);
          }
          const V3 Nh{lo.nrm[3 * hp], lo.nrm[3 * hp + 1], lo.nrm[3 * hp + 2]};
          const float wn = std::pow(std::fmax(0.0f, dot(Nf, Nh)), normalPow);
          const float wz = std::exp(-std::fabs(zf - lo.dep[hp]) / (depthScale * zf + 1e-6f));
          const float w = wb * wn * wz;
          wSum += w;
          eSum.x += w * Elo[3 * hp];
          eSum.y += w * Elo[3 * hp + 1];
          eSum.z += w * Elo[3 * hp + 2];
          oSum += w * occLo[hp];
        }
      long src = -1;
      if (wSum >= 1e-6f) {
        if (patch && wSum < thresh) (*patch)[pix] = 1;
        const float inv = 1.0f / wSum;
        E[3 * pix] = eSum.x * inv; E[3 * pix + 1] = eSum.y * inv; E[3 * pix + 2] = eSum.z * inv;
        occ[pix] = oSum * inv;
        continue;
      }
      if (patch) (*patch)[pix] = 1;
      if (bestPix >= 0) {
        src = bestPix;
      } else if (fallbackR > 0) {
        float bestD2 = 1e30f;
        for (int wy = by - fallbackR + 1; wy <= by + fallbackR; ++wy) {
          if (wy < 0 || wy >= hh) continue;
          for (int wx = bx - fallbackR + 1; wx <= bx + fallbackR; ++wx) {
            if (wx < 0 || wx >= hw) continue;
            const size_t hp = static_cast<size_t>(wy) * hw + wx;
            if (!lo.hit[hp]) continue;
            const float ddx = static_cast<float>(wx) - sx, ddy = static_cast<float>(wy) - sy;
            const float d2 = ddx * ddx + ddy * ddy;
            if (d2 < bestD2) {
              bestD2 = d2;
              src = static_cast<long>(hp);
            }
          }
        }
      }
      if (src >= 0) {
        E[3 * pix] = Elo[3 * src]; E[3 * pix + 1] = Elo[3 * src + 1]; E[3 * pix + 2] = Elo[3 * src + 2];
        occ[pix] = occLo[src];
      }
    }
  }
}

// pt1_upsample.hpp:214-248 smoothPatchedPixels: each marked pixel's E
// becomes the guide-weighted mean of its (2r+1)^2 eligible neighbourhood in a
// snapshot (itself at weight 1; weights below 1e-4 dropped).
inline void smoothPatchedPixels(int W, int H, const std::vector<uint8_t>& mask, const float* fnrm, const float* fdep,
                                const uint8_t* felig, float normalPow, float depthScale, int radius,
                                std::vector<float>& E, std::vector<float>& occ) {
  const std::vector<float> Es = E, os = occ;
  for (int py = 0; py < H; ++py)
    for (int px = 0; px < W; ++px) {
      const size_t pix = static_cast<size_t>(py) * W + px;
      if (!mask[pix]) continue;
      const V3 Nf{fnrm[3 * pix], fnrm[3 * pix + 1], fnrm[3 * pix + 2]};
      const float zf = fdep[pix];
      float wSum = 1.0f, oSum = os[pix];
      V3 eSum{Es[3 * pix], Es[3 * pix + 1], Es[3 * pix + 2]};
      for (int dy = -radius; dy <= radius; ++dy) {
        const int ny = py + dy;
        if (ny < 0 || ny >= H) continue;
        for (int dx = -radius; dx <= radius; ++dx) {
          if (dx == 0 && dy == 0) continue;
          const int nx = px + dx;
          if (nx < 0 || nx >= W) continue;
          const size_t q = static_cast<size_t>(ny) * W + nx;
          if (!felig[q]) continue;
          const V3 Nn{fnrm[3 * q], fnrm[3 * q + 1], fnrm[3 * q + 2]};
          const float wn = std::pow(std::fmax(0.0f, dot(Nf, Nn)), normalPow);
          const float wz = std::exp(-std::fabs(zf - fdep[q]) / (depthScale * zf + 1e-6f));
          const float w = wn * wz;
          if (w < 1e-4f) continue;
          wSum += w;
          eSum.x += w * Es[3 * q];
          eSum.y += w * Es[3 * q + 1];
          eSum.z += w * Es[3 * q + 2];
          oSum += w * os[q];
        }
      }
      const float inv = 1.0f / wSum;
      E[3 * pix] = eSum.x * inv; E[3 * pix + 1] = eSum.y * inv; E[3 * pix + 2] = eSum.z * inv;
      occ[pix] = oSum * inv;
    }
}

// pt2_sampler.hpp:71-78 pt2HashHp
inline uint32_t hashHp(uint32_t i) {
  i ^= i >> 16;
  i *= 0x21f0aaadu;
  i ^= i >> 15;
  i *= 0xd35a2d97u;
  i ^= i >> 15;
  return i ^ 0xe6fe3bebu;
}

// pt2_spatial.hpp:66-271 pt2SpatialRound: every eligible point restarts
// from its own previous-round reservoir and streams in K neighbours (8 in
// round 0, then 5) on a per-point rotated golden-angle spiral whose radius
// halves each round (floor 3), rejecting incompatible normals (< 0.5) and
// depths (> 10 %), empty reservoirs and samples nearer than 4 x the
// receiver spacing; W is normalised by the balance-heuristic mixture over
// the contributors (with `unbiased`, a contributor that cannot see the
// selected sample counts zero).  In the last round (Eout) E is the
// balance-MIS sum over all contributors' samples; ineligible points keep E.
inline void spatialRound(const Ctx& c, int W, int H, const float* pos, const float* nrm, const float* dep,
                         const uint8_t* elig, const std::vector<Reservoir>& in, std::vector<Reservoir>& out,
                         int round, float* Eout, int nt) {
  const Opt& o = c.o;
  const int K = round == 0 ? 8 : 5;
  float radius = o.pt2Radius / static_cast<float>(1 << round);
  if (radius < 3.0f) radius = 3.0f;
  const float kGolden = 2.399963230f;
  const uint32_t salt = hashHp(hashU32(o.pt1Seed) ^ (0x53504154u + static_cast<uint32_t>(round)));
  forRows(H, nt, [&](int py) {
    for (int px = 0; px < W; ++px) {
      const size_t pix = static_cast<size_t>(py) * W + px;
      if (!elig[pix]) {
        out[pix] = Reservoir{};
        continue;
      }
      const V3 P{pos[3 * pix], pos[3 * pix + 1], pos[3 * pix + 2]};
      const V3 N{nrm[3 * pix], nrm[3 * pix + 1], nrm[3 * pix + 2]};
      const float d0 = dep[pix];
      uint32_t s0 = hashHp(static_cast<uint32_t>(pix) ^ salt), s1 = 0x52535452u;
      Reservoir dst;
      double wSum = 0.0;
      float Mtot = 0.0f;
      V3 cPos[9], cN[9], sPos[9], sRad[9];
      float cM[9], sW[9], sJ[9];
      int nc = 0;
      {
        const Reservoir& own = in[pix];
        const float m = own.M > o.pt2MCap ? o.pt2MCap : own.M;
        const float w = targetPdf(P, N, own.pos, own.rad) * own.W * m;
        tea2(s0, s1);
        if (reservoirTake(wSum, Mtot, w, m, u32ToUnorm(s0))) {
          dst.pos = own.pos;
          dst.nrm = own.nrm;
          dst.rad = own.rad;
        }
        cPos[nc] = P; cN[nc] = N; cM[nc] = m;
        sPos[nc] = own.pos; sRad[nc] = own.rad; sW[nc] = own.W; sJ[nc] = 1.0f;
        ++nc;
      }
      tea2(s0, s1);
      const float rot = u32ToUnorm(s0) * 6.2831853f;
      for (int k = 0; k < K; ++k) {
        const float ang = rot + static_cast<float>(k) * kGolden;
        const float rr = std::sqrt((static_cast<float>(k) + 0.5f) / static_cast<float>(K)) * radius;
        const int nx = px + static_cast<int>(std::lround(std::cos(ang) * rr));
        const int ny = py + static_cast<int>(std::lround(std::sin(ang) * rr));
        if (nx < 0 || nx >= W || ny < 0 || ny >= H) continue;
        const size_t q = static_cast<size_t>(ny) * W + nx;
        if (q == pix || !elig[q]) continue;
        const V3 Nn{nrm[3 * q], nrm[3 * q + 1], nrm[3 * q + 2]};
        if (dot(N, Nn) < 0.5f) continue;
        if (std::fabs(d0 - dep[q]) > 0.1f * d0) continue;
        const Reservoir& nb = in[q];
        if (nb.M <= 0.0f) continue;
        const V3 Pn{pos[3 * q], pos[3 * q + 1], pos[3 * q + 2]};
        const V3 pq{Pn.x - P.x, Pn.y - P.y, Pn.z - P.z};
        const V3 ps{nb.pos.x - Pn.x, nb.pos.y - Pn.y, nb.pos.z - Pn.z};
        if (dot(ps, ps) < 4.0f * 4.0f * dot(pq, pq)) continue;
        const float j = reconnectJacobian(P, Pn, nb.pos, nb.nrm, 10.0f);
        const float m = nb.M > o.pt2MCap ? o.pt2MCap : nb.M;
        const float w = targetPdf(P, N, nb.pos, nb.rad) * nb.W * m * j;
        tea2(s0, s1);
        if (reservoirTake(wSum, Mtot, w, m, u32ToUnorm(s0))) {
          dst.pos = nb.pos;
          dst.nrm = nb.nrm;
          dst.rad = nb.rad;
        }
        cPos[nc] = Pn; cN[nc] = Nn; cM[nc] = m;
        sPos[nc] = nb.pos; sRad[nc] = nb.rad; sW[nc] = nb.W; sJ[nc] = j;
        ++nc;
      }
      float piSum = 0.0f;
      if (wSum > 0.0) {
        for (int k = 0; k < nc; ++k) {
          float pk = targetPdf(cPos[k], cN[k], dst.pos, dst.rad);
          if (pk <= 0.0f) continue;
          if (o.pt2Unbiased) {
            const V3 toS{dst.pos.x - cPos[k].x, dst.pos.y - cPos[k].y, dst.pos.z - cPos[k].z};
            const float dist2 = dot(toS, toS);
            if (dist2 <= 0.0f) continue;
            const float dist = std::sqrt(dist2);
            const V3 dir{toS.x / dist, toS.y / dist, toS.z / dist};
            if (dot(cN[k], dir) <= 0.0f) {
              pk = 0.0f;
            } else {
              const float eps = selfIntersectEps(cPos[k], dir, dist);
              const V3 O{cPos[k].x + cN[k].x * eps, cPos[k].y + cN[k].y * eps, cPos[k].z + cN[k].z * eps};
              if (occludedQ(*c.s, O, dir, eps, dist - 2.0f * eps)) pk = 0.0f;
            }
          }
          piSum += pk * cM[k];
        }
      }
      float Wn = 0.0f;
      if (piSum > 0.0f && wSum > 0.0) Wn = static_cast<float>(wSum) / piSum;
      dst.W = (o.pt2WClamp > 0.0f && Wn > o.pt2WClamp) ? o.pt2WClamp : Wn;
      dst.M = Mtot > o.pt2MCap ? o.pt2MCap : Mtot;
      out[pix] = dst;
      if (!Eout) continue;
      V3 E{0.0f, 0.0f, 0.0f};
      for (int k = 0; k < nc; ++k) {
        if (sW[k] <= 0.0f || sJ[k] <= 0.0f) continue;
        const float pq = targetPdf(P, N, sPos[k], sRad[k]);
        if (pq <= 0.0f) continue;
        float denom = 0.0f;
        for (int j2 = 0; j2 < nc; ++j2) denom += cM[j2] * targetPdf(cPos[j2], cN[j2], sPos[k], sRad[k]);
        if (denom <= 0.0f) continue;
        const float mis = cM[k] * pq / denom;
        const float l = lum3(sRad[k]);
        if (l <= 0.0f) continue;
        const float g = mis * sW[k] * sJ[k] * (pq / l) * (1.0f / kPiF);
        E.x += sRad[k].x * g;
        E.y += sRad[k].y * g;
        E.z += sRad[k].z * g;
      }
      Eout[3 * pix] = E.x;
      Eout[3 * pix + 1] = E.y;
      Eout[3 * pix + 2] = E.z;
    }
  });
}

// pt2_spatial.hpp:278-296 pt2SpatialResampleAndResolve: the rounds, ping-pong,
// the last one writing E
inline void spatialResample(const Ctx& c, int W, int H, const float* pos, const float* nrm, const float* dep,
                            const uint8_t* elig, std::vector<Reservoir>& rsv, std::vector<float>& E, int nt) {
  std::vector<Reservoir> pong(rsv.size());
  std::vector<Reservoir>* cur = &rsv;
  std::vector<Reservoir>* nxt = &pong;
  for (int r = 0; r < c.o.pt2Rounds; ++r) {
    spatialRound(c, W, H, pos, nrm, dep, elig, *cur, *nxt, r, r == c.o.pt2Rounds - 1 ? E.data() : nullptr, nt);
    std::swap(cur, nxt);
  }
}

// embree_renderer.cpp:560-1086 runPt1GiPass: the gather on the render grid
// (k = 1) or on a ceil(W/k) x ceil(H/k) grid with its own primary rays (with
// pt2's adaptive refinement), the denoise of E at gather resolution, the
// upsample, the edge patch, the [E] composite colour += giIntensity *
// (kd * pigment) * E, then pt2's traced mirror and glossy reflection.
struct ReflPix {  // the first hit's traced-reflection record per render-grid pixel
  std::vector<float> amt, alpha, aspect, f0, tan;
};
inline V3 schlick3(const V3& F0, float u) { return schlickF(F0, u); }
inline V3 reflectedRadiance(const Ctx& c, const V3& O, const V3& d, float tn, uint32_t r0, uint32_t r1) {
  Ray r;
  r.org = O; r.dir = d; r.tnear = tn; r.tfar = kInf;
  Hit h;
  if (!c.s->bvh.closest(r, h)) return pt1Environment(c, d);
  tea2(r0, r1);
  V3 rad, alb, Py, Ny, em;
  if (!pt1EvalVertex(c, h, O, d, rad, alb, Py, Ny, c.o.pt2Emissive, &r0, &r1, &em)) return V3{0.0f, 0.0f, 0.0f};
  const V3 sky = pt1Environment(c, d);
  return V3{rad.x + alb.x * sky.x, rad.y + alb.y * sky.y, rad.z + alb.z * sky.z};
}
// Smith Lambda of GGX (pt2_glossy.hpp:41-56) and visible-normal sampling
// (Heitz, JCGT 7(4) 2018)
inline float ggxLambdaIso(float alpha, float cosT) {
  const float c2 = std::fmax(cosT * cosT, 1.0e-12f);
  const float t2 = (1.0f - c2) / c2;
  return 0.5f * (std::sqrt(1.0f + alpha * alpha * t2) - 1.0f);
}
inline float ggxLambdaAn(float ax, float ay, const V3& w) {
  const float z2 = std::fmax(w.z * w.z, 1.0e-12f);
  const float t2 = (ax * ax * w.x * w.x + ay * ay * w.y * w.y) / z2;
  return 0.5f * (std::sqrt(1.0f + t2) - 1.0f);
}
inline V3 sampleGgxVndf(const V3& wo, float ax, float ay, float u1, float u2) {
  const V3 Vh = safeNormalize(V3{ax * wo.x, ay * wo.y, wo.z});
  const V3 T1 = Vh.z < 0.999f ? safeNormalize(cross(V3{0.0f, 0.0f, 1.0f}, Vh)) : V3{1.0f, 0.0f, 0.0f};
  const V3 T2 = cross(Vh, T1);
  const float r = std::sqrt(u1);
  const float phi = 2.0f * 3.14159265358979323846f * u2;
  const float t1 = r * std::cos(phi);
  float t2 = r * std::sin(phi);
  const float sw = 0.5f * (1.0f + Vh.z);
  t2 = (1.0f - sw) * std::sqrt(std::fmax(0.0f, 1.0f - t1 * t1)) + sw * t2;
  const float t3 = std::sqrt(std::fmax(0.0f, 1.0f - t1 * t1 - t2 * t2));
  const V3 Nh{t1 * T1.x + t2 * T2.x + t3 * Vh.x, t1 * T1.y + t2 * T2.y + t3 * Vh.y,
              t1 * T1.z + t2 * T2.z + t3 * Vh.z};
  return safeNormalize(V3{ax * Nh.x, ay * Nh.y, std::fmax(0.0f, Nh.z)});
}

inline void runPt1GiPass(const Ctx& c, const Cam& cam, int W, int H, const std::vector<float>& pos,
                         const std::vector<float>& nrm, const std::vector<float>& refl, const std::vector<float>& dep,
                         const std::vector<uint8_t>& elig, std::vector<float>& color, int nt,
                         uint64_t* patchedOut, const ReflPix* rp, int ss) {
  const Opt& o = c.o;
  const int k = std::max(1, o.pt1GatherDiv);
  const int spp = std::max(1, o.pt1Spp);
  const bool pt2 = o.pt2();
  // ReSTIR rounds (pt2Rounds > 0) exclude adaptive spp (embree_renderer.cpp:626-636)
  const bool restir = pt2 && o.pt2Rounds > 0;
  const bool adapt = pt2 && o.pt2Adaptive && !restir && spp >= 2;
  const int extra = adapt ? spp * (std::max(2, o.pt2AdaptiveMul) - 1) : 0;
  std::vector<float> E, occ;
  // the gather over a grid with pt2's adaptive refinement (embree_renderer.cpp:674-706)
  // or its ReSTIR reservoirs and spatial rounds (:735-767, 861-890)
  auto gather = [&](int gw, int gh, const float* gp, const float* gn, const float* gg, const uint8_t* ge,
                    const float* gd, std::vector<float>& Eo, std::vector<float>& oo) {
    GridPt2 g2;
    g2.pt2 = pt2;
    g2.sppPow2 = nextPow2(static_cast<uint32_t>(spp + extra));
    std::vector<float> halfE;
    if (adapt) g2.halfE = &halfE;
    std::vector<Reservoir> rsv;
    if (restir) g2.rsv = &rsv;
    gatherGrid(c, gw, gh, gp, gn, gg, ge, gd, spp, Eo, oo, nt, g2);
    if (restir) spatialResample(c, gw, gh, gp, gn, gd, ge, rsv, Eo, nt);
    if (!adapt) return;
    std::vector<uint8_t> m0, m1;
    adaptiveMask(gw, gh, Eo, halfE, ge, spp, o.pt2AdaptiveThresh, m0);
    dilateMask(gw, gh, m0, ge, m1);
    dilateMask(gw, gh, m1, ge, m0);
    size_t nref = 0;
    for (uint8_t v : m0) nref += v;
    if (nref == 0) return;
    GridPt2 gr = g2;
    gr.halfE = nullptr;
    gr.sampleOffset = spp;
    std::vector<float> Er, occr;
    gatherGrid(c, gw, gh, gp, gn, gg, m0.data(), gd, extra, Er, occr, nt, gr);
    const float wB = static_cast<float>(spp) / static_cast<float>(spp + extra);
    const float wR = 1.0f - wB;
    for (size_t p = 0; p < m0.size(); ++p) {
      if (!m0[p]) continue;
      for (int q = 0; q < 3; ++q) Eo[3 * p + q] = Eo[3 * p + q] * wB + Er[3 * p + q] * wR;
      oo[p] = oo[p] * wB + occr[p] * wR;
    }
  };
  if (k > 1) {
    const int hw = (W + k - 1) / k, hh = (H + k - 1) / k;
    GiGrid g;
    tracePt1GBuffer(c, cam, hw, hh, g, nt);
    std::vector<float> Eh, occh;
    gather(hw, hh, g.pos.data(), g.nrm.data(), g.gnrm.data(), g.hit.data(), g.dep.data(), Eh, occh);
    if (o.pt1Denoise) denoisePt1E(hw, hh, Eh, g.nrm.data(), g.pos.data(), o);
    std::vector<uint8_t> patch;
    upsampleJointBilateral(W, H, nrm.data(), dep.data(), elig.data(), g, Eh, occh, o.pt1UpNormalPow,
                           o.pt1UpDepthScale, k <= 2 ? 0 : k, E, occ, o.pt1EdgePatch ? &patch : nullptr,
                           o.pt1EdgePatchThresh);
    if (o.pt1EdgePatch) {
      uint64_t count = 0;
      for (uint8_t m : patch) count += m;
      if (patchedOut) *patchedOut = count;
      if (count > 0) {
        std::vector<float> Ep, occp;
        const int pspp = spp * std::max(1, o.pt1EdgePatchSppMul);
        GridPt2 gp2;
        gp2.pt2 = pt2;
        gp2.sppPow2 = nextPow2(static_cast<uint32_t>(pspp));
        gatherGrid(c, W, H, pos.data(), nrm.data(), nullptr, patch.data(), dep.data(), pspp, Ep, occp, nt, gp2);
        for (size_t i = 0; i < patch.size(); ++i) {
          if (!patch[i]) continue;
          E[3 * i] = Ep[3 * i]; E[3 * i + 1] = Ep[3 * i + 1]; E[3 * i + 2] = Ep[3 * i + 2];
          occ[i] = occp[i];
        }
        smoothPatchedPixels(W, H, patch, nrm.data(), dep.data(), elig.data(), o.pt1UpNormalPow, o.pt1UpDepthScale,
                            2, E, occ);
      }
    }
  } else {
    gather(W, H, pos.data(), nrm.data(), nullptr, elig.data(), dep.data(), E, occ);
    if (o.pt1Denoise) denoisePt1E(W, H, E, nrm.data(), pos.data(), o);
  }
  const float gI = o.giIntensity;
  const size_t n = static_cast<size_t>(W) * H;
  for (size_t pix = 0; pix < n; ++pix) {
    if (!elig[pix]) continue;
    color[4 * pix] += gI * refl[3 * pix] * E[3 * pix];
    color[4 * pix + 1] += gI * refl[3 * pix + 1] * E[3 * pix + 1];
    color[4 * pix + 2] += gI * refl[3 * pix + 2] * E[3 * pix + 2];
  }
  if (!rp) return;
  // pt2_reflect.hpp: one mirror ray per first hit that owns a mirror lobe
  auto incident = [&](const V3& P) {
    return cam.ortho ? cam.dir : safeNormalize(V3{P.x - cam.pos.x, P.y - cam.pos.y, P.z - cam.pos.z});
  };
  forRows(H, nt, [&](int py) {
    for (int px = 0; px < W; ++px) {
      const size_t pix = static_cast<size_t>(py) * W + px;
      const float kk = rp->amt[pix];
      if (kk <= 0.0f || rp->alpha[pix] > 0.0f) continue;
      const V3 P{pos[3 * pix], pos[3 * pix + 1], pos[3 * pix + 2]};
      const V3 N{nrm[3 * pix], nrm[3 * pix + 1], nrm[3 * pix + 2]};
      const V3 wi = incident(P);
      const float indot = dot(wi, N);
      const V3 rdir = safeNormalize(V3{wi.x - 2.0f * indot * N.x, wi.y - 2.0f * indot * N.y, wi.z - 2.0f * indot * N.z});
      const float t0 = dep[pix] > 0.0f ? dep[pix] : 1.0f;
      const float eps = selfIntersectEps(P, rdir, t0);
      const V3 O{P.x + N.x * eps, P.y + N.y * eps, P.z + N.z * eps};
      const V3 L = reflectedRadiance(c, O, rdir, eps, static_cast<uint32_t>(pix) ^ 0x52464c54u, 0x4e454531u);
      float cosI = -indot;
      if (cosI < 0.0f) cosI = 0.0f;
      if (cosI > 1.0f) cosI = 1.0f;
      const V3 F = schlick3(V3{rp->f0[3 * pix], rp->f0[3 * pix + 1], rp->f0[3 * pix + 2]}, cosI);
      color[4 * pix] += kk * F.x * L.x;
      color[4 * pix + 1] += kk * F.y * L.y;
      color[4 * pix + 2] += kk * F.z * L.z;
    }
  });
  if (!o.pt2Glossy) return;
  bool anyGlossy = false;
  for (size_t i = 0; i < n && !anyGlossy; ++i) anyGlossy = rp->amt[i] > 0.0f && rp->alpha[i] > 0.0f;
  if (!anyGlossy) return;
  // pt2_glossy.hpp: spp VNDF-sampled reflection rays per glossy pixel
  const int gspp = std::max(1, o.pt2GlossySpp);
  const uint32_t seedMix = hashU32(o.pt1Seed ^ 0x474c5359u);
  std::vector<float> Es(n * 3, 0.0f);
  forRows(H, nt, [&](int py) {
    for (int px = 0; px < W; ++px) {
      const size_t pix = static_cast<size_t>(py) * W + px;
      const float alpha = rp->alpha[pix];
      if (rp->amt[pix] <= 0.0f || alpha <= 0.0f) continue;
      const V3 P{pos[3 * pix], pos[3 * pix + 1], pos[3 * pix + 2]};
      const V3 N{nrm[3 * pix], nrm[3 * pix + 1], nrm[3 * pix + 2]};
      const V3 wiV = incident(P);
      bool aniso = false;
      float ax = alpha, ay = alpha;
      Frame f;
      if (!rp->tan.empty()) {
        const V3 T{rp->tan[3 * pix], rp->tan[3 * pix + 1], rp->tan[3 * pix + 2]};
        const float aspect = rp->aspect[pix];
        if (aspect != 1.0f && dot(T, T) > 0.5f) {
          aniso = true;
          f = Frame{T, cross(N, T), N};
          ax = alpha / aspect;
          if (ax > 1.0f) ax = 1.0f;
          ay = alpha * aspect;
        }
      }
      if (!aniso) f = frameFromNormal(N);
      const V3 woW{-wiV.x, -wiV.y, -wiV.z};
      V3 wo{dot(woW, f.t), dot(woW, f.b), dot(woW, f.n)};
      if (wo.z < 1.0e-4f) wo.z = 1.0e-4f;
      wo = safeNormalize(wo);
      const float lamO = aniso ? ggxLambdaAn(ax, ay, wo) : ggxLambdaIso(alpha, wo.z);
      const float t0 = dep[pix] > 0.0f ? dep[pix] : 1.0f;
      const uint32_t seedPix = hashU32(static_cast<uint32_t>(pix)) ^ seedMix;
      const V3 F0{rp->f0[3 * pix], rp->f0[3 * pix + 1], rp->f0[3 * pix + 2]};
      V3 sum{0.0f, 0.0f, 0.0f};
      for (int sI = 0; sI < gspp; ++sI) {
        float u1, u2;
        sobol2D(static_cast<uint32_t>(sI), seedPix, u1, u2);
        const V3 wm = sampleGgxVndf(wo, ax, ay, u1, u2);
        const float owm = dot(wo, wm);
        const V3 wl{2.0f * owm * wm.x - wo.x, 2.0f * owm * wm.y - wo.y, 2.0f * owm * wm.z - wo.z};
        if (wl.z <= 0.0f) continue;
        const float lamI = aniso ? ggxLambdaAn(ax, ay, wl) : ggxLambdaIso(alpha, wl.z);
        const float weight = (1.0f + lamO) / (1.0f + lamO + lamI);
        const V3 rdir = safeNormalize(V3{f.t.x * wl.x + f.b.x * wl.y + f.n.x * wl.z,
                                         f.t.y * wl.x + f.b.y * wl.y + f.n.y * wl.z,
                                         f.t.z * wl.x + f.b.z * wl.y + f.n.z * wl.z});
        const float eps = selfIntersectEps(P, rdir, t0);
        const V3 O{P.x + N.x * eps, P.y + N.y * eps, P.z + N.z * eps};
        const V3 L = reflectedRadiance(c, O, rdir, eps, static_cast<uint32_t>(pix) ^ 0x474c5359u,
                                       0x4e454532u + static_cast<uint32_t>(sI));
        const V3 F = schlick3(F0, owm);
        sum.x += weight * F.x * L.x;
        sum.y += weight * F.y * L.y;
        sum.z += weight * F.z * L.z;
      }
      const float inv = 1.0f / static_cast<float>(gspp);
      Es[3 * pix] = sum.x * inv; Es[3 * pix + 1] = sum.y * inv; Es[3 * pix + 2] = sum.z * inv;
    }
  });
  if (o.pt1Denoise && o.pt2GlossyDenoise) {
    if (ss <= 1 || W % ss != 0 || H % ss != 0) {
      denoisePt1E(W, H, Es, nrm.data(), pos.data(), o);
    } else {
      // embree_renderer.cpp:990-1078: glossy-masked downsample to the output
      // grid, denoise there, joint-bilateral upsample over the glossy pixels
      const int Wo = W / ss, Ho = H / ss;
      const size_t no = static_cast<size_t>(Wo) * Ho;
      GiGrid g;
      g.w = Wo;
      g.h = Ho;
      g.nrm.assign(no * 3, 0.0f);
      g.dep.assign(no, 0.0f);
      g.hit.assign(no, 0);
      g.pos.assign(no * 3, 0.0f);
      std::vector<float> Eo(no * 3, 0.0f);
      for (int oy = 0; oy < Ho; ++oy)
        for (int ox = 0; ox < Wo; ++ox) {
          const size_t op = static_cast<size_t>(oy) * Wo + ox;
          V3 eS{0, 0, 0}, nS{0, 0, 0}, pS{0, 0, 0};
          float zS = 0.0f;
          int cnt = 0;
          for (int sy = 0; sy < ss; ++sy)
            for (int sx = 0; sx < ss; ++sx) {
              const size_t pix = static_cast<size_t>(oy * ss + sy) * W + (ox * ss + sx);
              if (rp->amt[pix] <= 0.0f || rp->alpha[pix] <= 0.0f) continue;
              ++cnt;
              eS.x += Es[3 * pix]; eS.y += Es[3 * pix + 1]; eS.z += Es[3 * pix + 2];
              nS.x += nrm[3 * pix]; nS.y += nrm[3 * pix + 1]; nS.z += nrm[3 * pix + 2];
              pS.x += pos[3 * pix]; pS.y += pos[3 * pix + 1]; pS.z += pos[3 * pix + 2];
              zS += dep[pix];
            }
          if (cnt == 0) continue;
          const float inv = 1.0f / static_cast<float>(cnt);
          Eo[3 * op] = eS.x * inv; Eo[3 * op + 1] = eS.y * inv; Eo[3 * op + 2] = eS.z * inv;
          const V3 nA = safeNormalize(V3{nS.x * inv, nS.y * inv, nS.z * inv});
          g.nrm[3 * op] = nA.x; g.nrm[3 * op + 1] = nA.y; g.nrm[3 * op + 2] = nA.z;
          g.dep[op] = zS * inv;
          g.pos[3 * op] = pS.x * inv; g.pos[3 * op + 1] = pS.y * inv; g.pos[3 * op + 2] = pS.z * inv;
          g.hit[op] = 1;
        }
      denoisePt1E(Wo, Ho, Eo, g.nrm.data(), g.pos.data(), o);
      std::vector<uint8_t> gel(n, 0);
      for (size_t i = 0; i < n; ++i) gel[i] = (rp->amt[i] > 0.0f && rp->alpha[i] > 0.0f) ? 1 : 0;
      const std::vector<float> occLow(no, 1.0f);
      std::vector<float> Eup, occUp;
      upsampleJointBilateral(W, H, nrm.data(), dep.data(), gel.data(), g, Eo, occLow, o.pt1UpNormalPow,
                             o.pt1UpDepthScale, 0, Eup, occUp, nullptr, 0.0f);
      Es.swap(Eup);
    }
  }
  for (size_t pix = 0; pix < n; ++pix) {
    if (rp->amt[pix] <= 0.0f || rp->alpha[pix] <= 0.0f) continue;
    color[4 * pix] += rp->amt[pix] * Es[3 * pix];
    color[4 * pix + 1] += rp->amt[pix] * Es[3 * pix + 1];
    color[4 * pix + 2] += rp->amt[pix] * Es[3 * pix + 2];
  }
}

extern "C" {

void* oracle_scene_create(const ubr_scene_desc* d) {
  if (!d) return nullptr;
  return buildScene(*d);
}

void oracle_scene_destroy(void* s) { delete static_cast<Scene*>(s); }

uint64_t oracle_scene_bvh_nodes(void* s) { return static_cast<Scene*>(s)->bvh.nodeCount(); }

uint32_t oracle_scene_geom_id(void* s, int kind) { return static_cast<Scene*>(s)->geo.geomID[kind]; }

// Closest hits for n rays: rays = 8 floats each (ox oy oz tnear dx dy dz tfar).
// Outputs: t, geomID, primID, u, v, Ng (3 per ray). Any output may be NULL.
int oracle_intersect(void* sp, const float* rays, uint64_t n, float* t, uint32_t* geom,
                     uint32_t* prim, float* u, float* v, float* ng) {
  const Scene& s = *static_cast<Scene*>(sp);
  for (uint64_t i = 0; i < n; ++i) {
    const float* q = rays + 8 * i;
    Ray r;
    r.org = V3(q[0], q[1], q[2]); r.tnear = q[3];
    r.dir = V3(q[4], q[5], q[6]); r.tfar = q[7];
    Hit h;
    const bool hit = s.bvh.closest(r, h);
    if (t) t[i] = hit ? h.t : kInf;
    if (geom) geom[i] = hit ? h.geomID : kInvalid;
    if (prim) prim[i] = hit ? h.primID : kInvalid;
    if (u) u[i] = hit ? h.u : 0.0f;
    if (v) v[i] = hit ? h.v : 0.0f;
    if (ng) { ng[3 * i] = h.Ng.x; ng[3 * i + 1] = h.Ng.y; ng[3 * i + 2] = h.Ng.z; }
  }
  return 0;
}

int oracle_occluded(void* sp, const float* rays, uint64_t n, uint8_t* out) {
  const Scene& s = *static_cast<Scene*>(sp);
  for (uint64_t i = 0; i < n; ++i) {
    const float* q = rays + 8 * i;
    Ray r;
    r.org = V3(q[0], q[1], q[2]); r.tnear = q[3];
    r.dir = V3(q[4], q[5], q[6]); r.tfar = q[7];
    out[i] = s.bvh.occluded(r) ? 1 : 0;
  }
  return 0;
}

// EmbreeRenderer::occluded (embree_renderer.cpp:294-357) with its argument
// filter excludeFaceFilter (:76-133): segment i is occluded when a hit on the
// trimmed open segment is not on one of its excluded mesh faces, not grazing
// (|cos| <= grazeCos) and not coincident (plane within `coplanar` of the start).
int oracle_occluded_filtered(void* sp, const float* segs, uint64_t n, float eps, float grazeCos, float coplanar,
                             const uint32_t* offs, const int32_t* faces, uint8_t* out) {
  const Scene& s = *static_cast<Scene*>(sp);
  const bool meshPresent = s.geo.geomID[kMesh] != kInvalid;
  for (uint64_t i = 0; i < n; ++i) {
    const float* q = segs + 6 * i;
    const V3 p(q[0], q[1], q[2]), e(q[3], q[4], q[5]);
    const V3 d = e - p;
    const float len = std::sqrt(dot(d, d));
    out[i] = 0;
    if (len <= 0.0f) continue;
    const V3 dir(d.x / len, d.y / len, d.z / len);
    const float tnear = std::max(eps * len, eps);
    const float tfar = len * (1.0f - eps);
    if (tnear >= tfar) continue;
    Ray r;
    r.org = p; r.dir = dir; r.tnear = tnear; r.tfar = tfar;
    const int nFaces = (offs && faces && meshPresent) ? int(offs[i + 1] - offs[i]) : 0;
    const int32_t* fl = (offs && faces) ? faces + offs[i] : nullptr;
    if (nFaces == 0 && grazeCos <= 0.0f && coplanar <= 0.0f) {
      out[i] = s.bvh.occluded(r) ? 1 : 0;
      continue;
    }
    auto accept = [&](int kind, uint32_t prim, const Hit& h) {
      if (nFaces > 0 && kind == kMesh) {
        uint32_t pr = prim;
        if (s.baseTri > 0) pr %= uint32_t(s.baseTri);
        for (int k = 0; k < nFaces; ++k)
          if (uint32_t(fl[k]) == pr) return false;
      }
      if (grazeCos > 0.0f || coplanar > 0.0f) {
        const float nx = h.Ng.x, ny = h.Ng.y, nz = h.Ng.z;
        const float dx = r.dir.x, dy = r.dir.y, dz = r.dir.z;
        const float nlen = std::sqrt(nx * nx + ny * ny + nz * nz);
        const float dlen = std::sqrt(dx * dx + dy * dy + dz * dz);
        if (nlen > 0.0f && dlen > 0.0f) {
          const float dDotN = nx * dx + ny * dy + nz * dz;
          const float c = std::fabs(dDotN) / (nlen * dlen);
          if (grazeCos > 0.0f && c <= grazeCos) return false;
          if (coplanar > 0.0f) {
            const float perp = h.t * std::fabs(dDotN) / nlen;
            if (perp <= coplanar) return false;
          }
        }
      }
      return true;
    };
    out[i] = s.bvh.occludedIf(r, accept) ? 1 : 0;
  }
  return 0;
}

// One coarse-grid AO lookup on a hand-built grid (the unit cases of the
// reference's tests/test_ao_coarse.cpp:97-204): returns 1 and fills out[0..6]
// = openness, bent.xyz, contact, shape, avgHitDist when accepted, 0 when the
// guides reject.  bent / contact / shape / avg may be NULL (legacy grid).
int oracle_coarse_ao_lookup(int w, int h, const float* openness, const float* normal, const float* depth,
                            const uint8_t* hit, const float* bent, const float* contact, const float* shape,
                            const float* avg, int latW, int latH, uint32_t px, uint32_t py, const float* N, float z,
                            float* out) {
  CoarseAo g;
  const size_t n = static_cast<size_t>(w) * h;
  g.w = w;
  g.h = h;
  g.openness.assign(openness, openness + n);
  g.normal.assign(normal, normal + 3 * n);
  g.depth.assign(depth, depth + n);
  g.hit.assign(hit, hit + n);
  g.quality = bent != nullptr;
  if (g.quality) {
    g.bent.assign(bent, bent + 3 * n);
    g.contact.assign(contact, contact + n);
    g.shape.assign(shape, shape + n);
    g.avgHitDist.assign(avg, avg + n);
  }
  float op = 0.0f;
  AOResult aov;
  if (!sampleCoarseAo(g, latW, latH, px, py, V3{N[0], N[1], N[2]}, z, op, aov)) return 0;
  const float r[7] = {op, aov.bent.x, aov.bent.y, aov.bent.z, aov.contact, aov.shape, aov.avgHitDist};
  for (int k = 0; k < 7; ++k) out[k] = r[k];
  return 1;
}

// The adaptive-AA mask of hand-built centre records (rgba 4, normal 3 floats
// per output pixel): the predicates the reference's mask tests drive
// (tests/test_adaptive_aa.cpp:233-316).
int oracle_aa_mask(int Wf, int Hf, const float* rgba, const float* viewZ, const uint32_t* geom, const int32_t* group,
                   const float* normal, float threshold, float pixelWorldSize, int perspective, uint8_t* mask) {
  if (Wf <= 0 || Hf <= 0) return -1;
  const size_t n = static_cast<size_t>(Wf) * Hf;
  std::vector<AaCentre> c(n);
  for (size_t i = 0; i < n; ++i)
    c[i] = AaCentre{rgba[4 * i], rgba[4 * i + 1], rgba[4 * i + 2], rgba[4 * i + 3], viewZ[i], geom[i], group[i],
                    V3{normal[3 * i], normal[3 * i + 1], normal[3 * i + 2]}};
  buildAaMask(Wf, Hf, c.data(), threshold, pixelWorldSize, perspective != 0, mask);
  return 0;
}

// The frame: embree_renderer.cpp:1260-1427 pixel loop (rows [row0, row1) of the
// hi-res grid, all rows when row1 <= row0; the adaptive-AA passes of
// :1379-1670 when asked for), then pipeline.cpp:126-129 fog, :182-192 box
// downsample, :254 assumed gamma.  `threads` <= 0 uses all cores.  Returns 0,
// or -3 for adaptive AA together with the edge G-buffer (not restated).
int oracle_render_rows(void* sp, const ubr_render_desc* rdsc, ubr_frame* fr, int threads, int row0,
                       int row1) {
  const Scene& s = *static_cast<Scene*>(sp);
  const ubr_render_desc& d = *rdsc;
  const int ss = std::max(1, d.supersample);
  const int W = d.width * ss, H = d.height * ss;
  // computeCameraBasis (embree_renderer.cpp:375-386)
  const float aspect = static_cast<float>(W) / static_cast<float>(H);
  const V3 camPos{d.cam_position[0], d.cam_position[1], d.cam_position[2]};
  const V3 dir = normalize(V3{d.cam_direction[0], d.cam_direction[1], d.cam_direction[2]});
  const V3 right = normalize(cross(dir, V3{d.cam_up[0], d.cam_up[1], d.cam_up[2]}));
  const V3 trueUp = normalize(cross(right, dir));
  const float halfH = d.cam_height * 0.5f;
  const float halfW = halfH * aspect;
  const float persHalfH = std::tan(radians(d.cam_fovy) * 0.5f);
  const float persHalfW = persHalfH * aspect;

  Ctx c;
  c.s = &s;
  c.o.aoSamples = d.ao_samples; c.o.aoDistance = d.ao_distance; c.o.aoIntensity = d.ao_intensity;
  c.o.aoFalloffPower = d.ao_falloff_power; c.o.aoMultiScale = d.ao_multiscale != 0;
  c.o.aoBentNormal = d.ao_bent_normal != 0; c.o.aoMultibounce = d.ao_multibounce != 0;
  c.o.aoLowDiscrepancy = d.ao_low_discrepancy != 0;
  c.o.gi = d.gi != 0;
  c.o.pt1Spp = d.pt1_spp; c.o.giBounces = d.gi_bounces; c.o.pt1SkyMode = d.pt1_sky_mode;
  c.o.giMaxDistance = d.gi_max_distance; c.o.giIntensity = d.gi_intensity;
  c.o.giEnvIntensity = d.gi_env_intensity; c.o.pt1Clamp = d.pt1_clamp; c.o.pt1Seed = d.pt1_seed;
  for (int k = 0; k < 3; ++k) c.o.pt1SkyRadiance[k] = d.pt1_sky_radiance[k];
  c.o.pt1Ld = d.pt1_ld != 0;
  {
    // pt1GatherDiv: -1 = the supersample factor (pipeline.cpp), 0 = pt1HalfRes ? 2 : 1 (embree_renderer.cpp:717-719)
    int k = d.pt1_gather_div;
    if (k < 0) k = std::max(1, d.supersample);
    if (k == 0) k = d.pt1_half_res ? 2 : 1;
    c.o.pt1GatherDiv = std::max(1, k);
  }
  c.o.pt1Denoise = d.pt1_denoise != 0;
  c.o.pt1EdgePatch = d.pt1_edge_patch != 0;
  c.o.pt1UpNormalPow = d.pt1_upsample_normal_pow;
  c.o.pt1UpDepthScale = d.pt1_upsample_depth_scale;
  c.o.pt1EdgePatchThresh = d.pt1_edge_patch_thresh;
  c.o.pt1EdgePatchSppMul = d.pt1_edge_patch_spp_mul;
  c.o.giIntegrator = d.gi_integrator;
  c.o.pt2Pattern = d.pt2_pattern;
  c.o.pt2Emissive = d.pt2_emissive != 0;
  c.o.pt2EmissiveNee = d.pt2_emissive_nee != 0;
  c.o.pt2Reflect = d.pt2_reflect != 0;
  c.o.pt2Glossy = d.pt2_glossy != 0;
  c.o.pt2GlossySpp = d.pt2_glossy_spp;
  c.o.pt2GlossyDenoise = d.pt2_glossy_denoise != 0;
  c.o.pt2Adaptive = d.pt2_adaptive != 0;
  c.o.pt2AdaptiveThresh = d.pt2_adaptive_thresh;
  c.o.pt2AdaptiveMul = d.pt2_adaptive_mul;
  c.o.pt2Rounds = d.pt2_rounds;
  c.o.pt2Radius = d.pt2_radius;
  c.o.pt2Unbiased = d.pt2_unbiased != 0;
  c.o.pt2MCap = d.pt2_m_cap;
  c.o.pt2WClamp = d.pt2_w_clamp;
  c.o.denoiseIters = d.denoise_iters;
  c.o.denoiseSigmaN = d.denoise_sigma_n;
  c.o.denoiseSigmaZ = d.denoise_sigma_z;
  c.o.denoiseSigmaL = d.denoise_sigma_l;
  for (int k = 0; k < 3; ++k) { c.o.aoSky[k] = d.ao_sky_color[k]; c.o.aoGround[k] = d.ao_ground_color[k]; }
  c.o.aoDiffuseFactor = d.ao_diffuse_factor;
  c.o.shadows = d.shadows != 0; c.o.shadowSamples = d.shadow_samples; c.o.envLights = d.env_lights;
  c.o.specularScale = d.specular_scale; c.o.transparency = d.transparency != 0;
  c.o.transparentBackground = d.transparent_background != 0;
  c.o.maxTransparentLayers = d.max_transparent_layers;
  c.o.aoWriteAov = d.ao_write_aov != 0;
  c.o.aaMode = d.aa_mode;
  c.o.edgeGbuffer = d.edge_gbuffer != 0;
  // buildSceneLights (embree_renderer.cpp:436-458)
  for (uint32_t i = 0; i < d.light_count; ++i) {
    const ubr_light& dl = d.lights[i];
    Light l;
    l.L = normalize(V3{-dl.direction[0], -dl.direction[1], -dl.direction[2]});
    l.color = V3{dl.color[0] * dl.intensity, dl.color[1] * dl.intensity, dl.color[2] * dl.intensity};
    l.highlight = dl.casts_highlight != 0;
    l.radius = (d.gi_integrator == 2 && dl.angular_radius > 0.0f) ? dl.angular_radius : radians(d.light_radius_deg);
    c.lights.push_back(l);
  }
  // buildEnvDomeLights (ao/env_dome.hpp:33-64)
  if (d.env_lights > 0) {
    for (Light& l : c.lights) l.color = l.color * d.env_key_scale;
    const int n = d.env_lights;
    const float cosMax = std::cos(radians(d.env_angle));
    const float ga = 3.14159265f * (3.0f - std::sqrt(5.0f));
    float cosSum = 0.0f;
    std::vector<V3> dirs;
    for (int i = 0; i < n; ++i) {
      const float z = 1.0f - (1.0f - cosMax) * ((i + 0.5f) / n);
      const float r = std::sqrt(std::max(0.0f, 1.0f - z * z));
      const float t = ga * i;
      V3 dd = normalize(dir * z + right * (r * std::cos(t)) + trueUp * (r * std::sin(t)));
      dirs.push_back(dd);
      cosSum += z;
    }
    const float perLight = cosSum > 0.0f ? d.env_intensity / cosSum : 0.0f;
    for (const V3& dd : dirs) {
      Light l;
      l.L = V3{-dd.x, -dd.y, -dd.z};
      l.color = V3{perLight, perLight, perLight};
      l.highlight = false;
      l.radius = radians(d.light_radius_deg);
      c.lights.push_back(l);
    }
  }
  c.ambLight = V3{d.ambient_color[0], d.ambient_color[1], d.ambient_color[2]};
  c.bg = V3{d.background[0], d.background[1], d.background[2]};
  c.aoUp = d.ao_use_camera_up ? trueUp : safeNormalize(V3{d.ao_up[0], d.ao_up[1], d.ao_up[2]}, trueUp);
  c.wHi = W;
  c.frameW = W;
  c.frameH = H;
  c.clipNear = d.clip_near;
  c.clipFar = d.clip_far;

  const size_t npix = static_cast<size_t>(W) * H;
  std::vector<float> color(npix * 4, 0.0f), viewZ(npix, 0.0f), depth(npix, 0.0f);
  std::vector<uint32_t> hg(npix, kInvalid), hp(npix, kInvalid);
  // AO AOVs (allocateFrameBuffers, embree_renderer.cpp:500-505 defaults)
  const bool aov = d.ao_write_aov != 0;
  std::vector<float> aAlb, aNrm, aBent, aCon, aShp, aAvg;
  if (aov) {
    aAlb.assign(npix * 3, 0.0f); aNrm.assign(npix * 3, 0.0f); aBent.assign(npix * 3, 0.0f);
    aCon.assign(npix, 1.0f); aShp.assign(npix, 1.0f); aAvg.assign(npix, 0.0f);
  }
  if (row1 <= row0) { row0 = 0; row1 = H; }
  // storePixelResult (embree_renderer.cpp:213-250): one hi-res sample
  float* patchMask = nullptr;  // set once the coarse AO grid is active
  // GI seeds per hi-res pixel (storeShadingChannels, embree_renderer.cpp:184-193)
  std::vector<float> giPos, giNrm, giRef, giDep;
  std::vector<uint8_t> giEl;
  ReflPix rp;
  const bool reflOn = c.o.gi && c.o.traceRefl();
  if (c.o.gi) {
    giPos.assign(npix * 3, 0.0f); giNrm.assign(npix * 3, 0.0f); giRef.assign(npix * 3, 0.0f);
    giDep.assign(npix, 0.0f); giEl.assign(npix, 0);
    if (reflOn) {
      rp.amt.assign(npix, 0.0f); rp.alpha.assign(npix, 0.0f); rp.aspect.assign(npix, 1.0f);
      rp.f0.assign(npix * 3, 1.0f); rp.tan.assign(npix * 3, 0.0f);
    }
  }
  auto store = [&](size_t pix, const PixelOut& po) {
    if (c.o.gi) {
      for (int k = 0; k < 3; ++k) {
        giPos[3 * pix + k] = (&po.firstPos.x)[k];
        giNrm[3 * pix + k] = (&po.first.normal.x)[k];
        giRef[3 * pix + k] = (&po.first.giRefl.x)[k];
      }
      giDep[pix] = po.depth;
      giEl[pix] = po.geom == kInvalid ? 0 : po.first.giElig;
      if (reflOn) {  // storeShadingChannels (embree_renderer.cpp:194-216)
        rp.amt[pix] = po.first.reflAmt;
        rp.alpha[pix] = po.first.reflAlpha;
        rp.aspect[pix] = po.first.reflAspect;
        for (int k = 0; k < 3; ++k) {
          rp.f0[3 * pix + k] = (&po.first.reflF0.x)[k];
          rp.tan[3 * pix + k] = (&po.first.reflTan.x)[k];
        }
      }
    }
    color[4 * pix] = po.r; color[4 * pix + 1] = po.g; color[4 * pix + 2] = po.b; color[4 * pix + 3] = po.a;
    depth[pix] = po.depth;
    viewZ[pix] = po.viewZ;
    hg[pix] = po.geom;
    hp[pix] = po.prim;
    if (patchMask) patchMask[pix] = static_cast<float>(po.first.aoPatched);
    if (c.o.edgeGbuffer) {  // storeGBufChannels (embree_renderer.cpp:240-262)
      if (fr->gb_object_id) fr->gb_object_id[pix] = po.first.objectId;
      if (fr->gb_material_id) fr->gb_material_id[pix] = po.first.materialId;
      if (fr->gb_surf_alpha) fr->gb_surf_alpha[pix] = po.geom == kInvalid ? 1.0f : po.first.opacity;
      if (fr->gb_normal) {
        fr->gb_normal[3 * pix] = po.first.normal.x;
        fr->gb_normal[3 * pix + 1] = po.first.normal.y;
        fr->gb_normal[3 * pix + 2] = po.first.normal.z;
      }
      if (fr->gb_clip_cut) fr->gb_clip_cut[pix] = po.clipCut;
      if (fr->gb_clip_near_vz) fr->gb_clip_near_vz[pix] = po.clipNearVz;
      if (fr->gb_clip_far_vz) fr->gb_clip_far_vz[pix] = po.clipFarVz;
    }
    if (aov) {
      const HitShade& f = po.first;
      const float a3[3][3] = {{f.albedo.x, f.albedo.y, f.albedo.z}, {f.normal.x, f.normal.y, f.normal.z},
                              {f.bent.x, f.bent.y, f.bent.z}};
      for (int k = 0; k < 3; ++k) {
        aAlb[3 * pix + k] = a3[0][k];
        aNrm[3 * pix + k] = a3[1][k];
        aBent[3 * pix + k] = a3[2][k];
      }
      aCon[pix] = f.contact;
      aShp[pix] = f.shape;
      aAvg[pix] = f.avgHit;
    }
  };
  // primary ray through lattice point (px, py) of a Wl x Hl lattice
  auto rayAtL = [&](int px, int py, int Wl, int Hl, V3& org, V3& rd) {
    const float v = 1.0f - 2.0f * (static_cast<float>(py) + 0.5f) / static_cast<float>(Hl);
    const float u = 2.0f * (static_cast<float>(px) + 0.5f) / static_cast<float>(Wl) - 1.0f;
    if (d.cam_orthographic) {
      org = camPos + right * (u * halfW) + trueUp * (v * halfH);
      rd = dir;
    } else {
      org = camPos;
      rd = normalize(dir + right * (u * persHalfW) + trueUp * (v * persHalfH));
    }
  };
  auto rayAt = [&](int px, int py, V3& org, V3& rd) { rayAtL(px, py, W, H, org, rd); };
  int nThreads = threads > 0 ? threads : static_cast<int>(std::thread::hardware_concurrency());
  if (nThreads < 1) nThreads = 1;
  auto parallelRange = [&](int n, const std::function<void(int)>& fn) {
    std::atomic<int> next{0};
    auto w = [&]() {
      for (int y = next.fetch_add(1); y < n; y = next.fetch_add(1)) fn(y);
    };
    std::vector<std::thread> pool;
    for (int i = 1; i < nThreads; ++i) pool.emplace_back(w);
    w();
    for (auto& th : pool) th.join();
  };
  // Coarse-grid AO pre-pass (embree_renderer.cpp:527-553; pipeline.cpp:68
  // resolves -1 to the supersample factor): the first-hit G-buffer of a
  // ceil(W / div) x ceil(H / div) grid (pt1_gbuffer.hpp:83-196, no clip
  // range, mesh hits and non-outline primitives eligible) and one AO gather
  // per eligible cell seeded on the coarse lattice (ao_coarse.hpp:73-140).
  CoarseAo coarse;
  {
    const int div = d.ao_res_div < 0 ? ss : d.ao_res_div;
    bool eligible = !s.geo.triIdx.empty();
    for (int k = 1; k < 4 && !eligible; ++k)
      for (uint8_t fe : s.fromEdge[k])
        if (!fe) {
          eligible = true;
          break;
        }
    if (div > 1 && d.ao_samples > 0 && eligible) {
      const int hw = (W + div - 1) / div, hh = (H + div - 1) / div;
      const size_t nc = static_cast<size_t>(hw) * hh;
      coarse.w = hw;
      coarse.h = hh;
      coarse.quality = c.o.aoEnhanced() || c.o.aoWriteAov;
      coarse.openness.assign(nc, 1.0f);
      coarse.normal.assign(nc * 3, 0.0f);
      coarse.depth.assign(nc, 0.0f);
      coarse.hit.assign(nc, 0);
      if (coarse.quality) {
        coarse.bent.assign(nc * 3, 0.0f);
        coarse.contact.assign(nc, 1.0f);
        coarse.shape.assign(nc, 1.0f);
        coarse.avgHitDist.assign(nc, 0.0f);
      }
      parallelRange(hh, [&](int cy) {
        for (int cx = 0; cx < hw; ++cx) {
          V3 org, rd;
          rayAtL(cx, cy, hw, hh, org, rd);
          Ray r;
          r.org = org; r.dir = rd; r.tnear = 0.0f; r.tfar = kInf;
          Hit h;
          if (!s.bvh.closest(r, h)) continue;
          const int kind = kindOfGeom(s, h.geomID);
          V3 N, Ng;
          if (kind == kMesh) {
            const uint32_t* tri = &s.geo.triIdx[3 * h.primID];
            const float w0 = 1.0f - h.u - h.v;
            float nb[3];
            for (int k = 0; k < 3; ++k)
              nb[k] = w0 * s.nrm[3 * tri[0] + k] + h.u * s.nrm[3 * tri[1] + k] + h.v * s.nrm[3 * tri[2] + k];
            N = safeNormalize(V3{nb[0], nb[1], nb[2]});
            Ng = safeNormalize(h.Ng);
          } else {
            if (s.fromEdge[kind][h.primID]) continue;
            N = safeNormalize(h.Ng);
            Ng = N;
          }
          if (dot(N, rd) > 0.0f) N = V3{-N.x, -N.y, -N.z};
          if (dot(Ng, rd) > 0.0f) Ng = V3{-Ng.x, -Ng.y, -Ng.z};
          const size_t cp = static_cast<size_t>(cy) * hw + cx;
          const V3 P{org.x + rd.x * h.t, org.y + rd.y * h.t, org.z + rd.z * h.t};
          const float secEps = selfIntersectEps(P, N, h.t);
          AOResult aov;
          float op;
          if (c.o.aoEnhanced()) {
            aov = computeAOQuality(s, P, Ng, N, secEps, c.o.aoSamples, c.o.aoDistance, c.o.aoFalloffPower,
                                   c.o.aoMultiScale, c.o.aoLowDiscrepancy, uint32_t(cx), uint32_t(cy), hw);
            op = aov.openness;
          } else {
            op = computeAO(s, P, Ng, N, secEps, c.o.aoSamples, c.o.aoDistance, uint32_t(cx), uint32_t(cy), hw);
            if (c.o.aoWriteAov)
              aov = computeAOQuality(s, P, Ng, N, secEps, c.o.aoSamples, c.o.aoDistance, 0.0f, false, false,
                                     uint32_t(cx), uint32_t(cy), hw);
          }
          coarse.openness[cp] = op;
          coarse.normal[cp * 3] = N.x;
          coarse.normal[cp * 3 + 1] = N.y;
          coarse.normal[cp * 3 + 2] = N.z;
          coarse.depth[cp] = h.t;
          coarse.hit[cp] = 1;
          if (coarse.quality) {
            coarse.bent[cp * 3] = aov.bent.x;
            coarse.bent[cp * 3 + 1] = aov.bent.y;
            coarse.bent[cp * 3 + 2] = aov.bent.z;
            coarse.contact[cp] = aov.contact;
            coarse.shape[cp] = aov.shape;
            coarse.avgHitDist[cp] = aov.avgHitDist;
          }
        }
      });
      c.coarse = &coarse;
      patchMask = fr->ao_patch_mask;
      if (patchMask) std::fill(patchMask, patchMask + npix, 0.0f);
    }
  }
  const bool coarseOn = c.coarse != nullptr;
  // Adaptive AA (embree_renderer.cpp:1379-1670, render/adaptive_aa.hpp):
  // centre sample per output pixel, refinement mask, flagged blocks shaded
  // per subpixel, the others replicate a centre re-shaded with ss^2 AO and
  // soft-shadow samples; aaDepth > ss shades each flagged cell as the box
  // average of kFine^2 samples of a finer lattice (:1542-1590).
  const bool adaptive = d.aa_mode == 1 && (ss > 1 || d.aa_depth > 1) && W % ss == 0 && H % ss == 0;
  // adaptive AA with the edge G-buffer probes replicated subpixels
  // (embree_renderer.cpp:1611-1640); not restated
  if (adaptive && d.edge_gbuffer) return -3;
  if (adaptive) {
    const int Wf = W / ss, Hf = H / ss, cSub = ss / 2;
    const int kFine = std::max(1, (d.aa_depth + ss - 1) / ss);
    Ctx cf = c;
    cf.wHi = W * kFine;  // seeds live on the (W k) x (H k) lattice
    auto shadeCell = [&](int px, int py) -> PixelOut {
      PixelOut acc{};
      for (int b = 0; b < kFine; ++b)
        for (int a = 0; a < kFine; ++a) {
          const int pxk = px * kFine + a, pyk = py * kFine + b;
          V3 org, rd;
          rayAtL(pxk, pyk, W * kFine, H * kFine, org, rd);
          const PixelOut pr = integratePixel(cf, org, rd, uint32_t(pxk), uint32_t(pyk), dir);
          if (a == 0 && b == 0) {
            acc = pr;  // discrete fields and AOVs: the first sample
          } else {
            acc.r += pr.r;
            acc.g += pr.g;
            acc.b += pr.b;
            acc.a += pr.a;
            acc.depth += pr.depth;
            acc.viewZ += pr.viewZ;
          }
        }
      const float inv = 1.0f / static_cast<float>(kFine * kFine);
      acc.r *= inv;
      acc.g *= inv;
      acc.b *= inv;
      acc.a *= inv;
      acc.depth *= inv;
      acc.viewZ *= inv;
      return acc;
    };
    int nt0 = threads > 0 ? threads : static_cast<int>(std::thread::hardware_concurrency());
    if (nt0 < 1) nt0 = 1;
    auto parallelRows = [&](int n, const std::function<void(int)>& fn) {
      std::atomic<int> next{0};
      auto w = [&]() {
        for (int y = next.fetch_add(1); y < n; y = next.fetch_add(1)) fn(y);
      };
      std::vector<std::thread> pool;
      for (int i = 1; i < nt0; ++i) pool.emplace_back(w);
      w();
      for (auto& th : pool) th.join();
    };
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<PixelOut> centers(static_cast<size_t>(Wf) * Hf);
    parallelRows(Hf, [&](int Y) {
      for (int X = 0; X < Wf; ++X) {
        V3 org, rd;
        rayAt(X * ss + cSub, Y * ss + cSub, org, rd);
        centers[static_cast<size_t>(Y) * Wf + X] =
            integratePixel(c, org, rd, uint32_t(X * ss + cSub), uint32_t(Y * ss + cSub), dir);
      }
    });
    // buildAaMask (adaptive_aa.hpp:121-190) over the centre records
    const float pixelWorldSize = d.cam_orthographic ? (d.cam_height / static_cast<float>(Hf))
                                                    : (2.0f * persHalfH / static_cast<float>(Hf));
    std::vector<AaCentre> rec(centers.size());
    for (size_t i = 0; i < centers.size(); ++i) {
      const PixelOut& po = centers[i];
      rec[i] = AaCentre{po.r, po.g, po.b, po.a, po.viewZ, po.geom, po.first.group, po.first.normal};
    }
    std::vector<uint8_t> mask(centers.size(), 0);
    buildAaMask(Wf, Hf, rec.data(), d.aa_threshold, pixelWorldSize, !d.cam_orthographic, mask.data());
    if (fr->aa_mask) for (size_t i = 0; i < mask.size(); ++i) fr->aa_mask[i] = float(mask[i]);
    // replication context: ss^2 AO and (stochastic) soft-shadow samples
    const bool soft = d.shadow_samples > 1 && d.light_radius_deg > 0.0f;
    const bool needBoost = ss > 1 && ((d.ao_samples > 0 && !coarseOn) || soft);
    Ctx cb = c;
    cb.o.aoSamples = c.o.aoSamples * (coarseOn ? 1 : ss * ss);
    cb.o.shadowSamples = c.o.shadowSamples * (soft ? ss * ss : 1);
    parallelRows(Hf, [&](int Y) {
      for (int X = 0; X < Wf; ++X) {
        const size_t XY = static_cast<size_t>(Y) * Wf + X;
        if (!mask[XY]) {
          PixelOut rep = centers[XY];
          if (needBoost) {
            V3 org, rd;
            rayAt(X * ss + cSub, Y * ss + cSub, org, rd);
            rep = integratePixel(cb, org, rd, uint32_t(X * ss + cSub), uint32_t(Y * ss + cSub), dir);
          }
          for (int j = 0; j < ss; ++j)
            for (int i = 0; i < ss; ++i) store(static_cast<size_t>(Y * ss + j) * W + (X * ss + i), rep);
          continue;
        }
        for (int j = 0; j < ss; ++j)
          for (int i = 0; i < ss; ++i) {
            const int px = X * ss + i, py = Y * ss + j;
            if (kFine == 1 && i == cSub && j == cSub) {
              store(static_cast<size_t>(py) * W + px, centers[XY]);
              continue;
            }
            if (kFine > 1) {
              store(static_cast<size_t>(py) * W + px, shadeCell(px, py));
              continue;
            }
            V3 org, rd;
            rayAt(px, py, org, rd);
            store(static_cast<size_t>(py) * W + px, integratePixel(c, org, rd, uint32_t(px), uint32_t(py), dir));
          }
      }
    });
    const auto t1 = std::chrono::steady_clock::now();
    fr->render_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    row0 = row1 = 0;  // the pixel loop below has nothing left to do
  }
  std::atomic<int> nextRow{row0};
  std::atomic<uint64_t> rays{0}, capped{0}, occRays{0};
  auto worker = [&]() {
    uint64_t myRays = 0, myCapped = 0;
    const uint64_t occ0 = tOccRays;
    for (;;) {
      const int py = nextRow.fetch_add(1);
      if (py >= row1) break;
      const float v = 1.0f - 2.0f * (static_cast<float>(py) + 0.5f) / static_cast<float>(H);
      for (int px = 0; px < W; ++px) {
        const float u = 2.0f * (static_cast<float>(px) + 0.5f) / static_cast<float>(W) - 1.0f;
        V3 org, rd;
        if (d.cam_orthographic) {
          org = camPos + right * (u * halfW) + trueUp * (v * halfH);
          rd = dir;
        } else {
          org = camPos;
          rd = normalize(dir + right * (u * persHalfW) + trueUp * (v * persHalfH));
        }
        const PixelOut po = integratePixel(c, org, rd, static_cast<uint32_t>(px), static_cast<uint32_t>(py), dir);
        const size_t pix = static_cast<size_t>(py) * W + px;
        store(pix, po);
        myRays += po.rays;
        myCapped += po.capped ? 1 : 0;
      }
    }
    rays += myRays;
    capped += myCapped;
    occRays += tOccRays - occ0;
  };
  int nt = threads > 0 ? threads : static_cast<int>(std::thread::hardware_concurrency());
  if (nt < 1) nt = 1;
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::thread> pool;
  for (int i = 1; i < nt; ++i) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
  const auto t1 = std::chrono::steady_clock::now();
  if (!adaptive) fr->render_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  fr->rays_primary = rays.load();
  fr->capped_rays = capped.load();
  fr->rays_occlusion = occRays.load();

  // embree_renderer.cpp:1708-1712: the GI pass before fog
  if (c.o.gi) {
    const Cam cam{camPos, dir, right, trueUp, d.cam_orthographic != 0, halfW, halfH, persHalfW, persHalfH};
    uint64_t patched = 0;
    runPt1GiPass(c, cam, W, H, giPos, giNrm, giRef, giDep, giEl, color, nt, &patched, reflOn ? &rp : nullptr,
                 ss);
    fr->gi_patched_pixels = patched;
  }
  // fog.cpp:7-36 applyFog on the hi-res viewZ (pipeline.cpp:126-129)
  if (d.fog_enabled) {
    for (size_t i = 0; i < npix; ++i) {
      const float z = viewZ[i];
      if (z <= 0.0f) continue;
      float f;
      const float denom = d.fog_end - d.fog_start;
      if (denom <= 0.0f) f = z < d.fog_end ? 1.0f : 0.0f;
      else {
        f = (d.fog_end - z) / denom;
        if (f < 0.0f) f = 0.0f;
        if (f > 1.0f) f = 1.0f;
      }
      float* cc = &color[4 * i];
      if (d.transparent_background) {
        cc[3] *= f;
      } else {
        cc[0] = d.fog_color[0] * (1.0f - f) + cc[0] * f;
        cc[1] = d.fog_color[1] * (1.0f - f) + cc[1] * f;
        cc[2] = d.fog_color[2] * (1.0f - f) + cc[2] * f;
      }
    }
  }
  // image_ops.cpp:9-35 boxDownsample
  std::vector<float> fin;
  if (ss > 1) {
    const int ow = W / ss, oh = H / ss;
    fin.assign(static_cast<size_t>(ow) * oh * 4, 0.0f);
    const float inv = 1.0f / static_cast<float>(ss * ss);
    for (int y = 0; y < oh; ++y)
      for (int x = 0; x < ow; ++x)
        for (int ch = 0; ch < 4; ++ch) {
          float acc = 0.0f;
          for (int dy = 0; dy < ss; ++dy)
            for (int dx = 0; dx < ss; ++dx) {
              const float vv = color[(static_cast<size_t>(y * ss + dy) * W + (x * ss + dx)) * 4 + ch];
              acc += std::isfinite(vv) ? vv : 0.0f;
            }
          fin[(static_cast<size_t>(y) * ow + x) * 4 + ch] = acc * inv;
        }
  } else {
    fin.swap(color);
  }
  // pipeline.cpp:224-252: the a-trous denoiser on the final-resolution linear
  // colour, guided by the AO AOV normal / albedo (without GI the reference
  // allocates those planes only for aoWriteAov)
  if (d.denoiser != 0 && aov) {
    const int ow = W / ss, oh = H / ss;
    const size_t no = static_cast<size_t>(ow) * oh;
    std::vector<float> dn(no * 3), da(no * 3);
    auto downTo = [&](const std::vector<float>& src, std::vector<float>& dst) {
      if (ss == 1) {
        dst = src;
        return;
      }
      const float inv = 1.0f / static_cast<float>(ss * ss);
      for (int y = 0; y < oh; ++y)
        for (int x = 0; x < ow; ++x)
          for (int q = 0; q < 3; ++q) {
            float acc = 0.0f;
            for (int dy = 0; dy < ss; ++dy)
              for (int dx = 0; dx < ss; ++dx) {
                const float vv = src[(static_cast<size_t>(y * ss + dy) * W + (x * ss + dx)) * 3 + q];
                acc += std::isfinite(vv) ? vv : 0.0f;
              }
            dst[(static_cast<size_t>(y) * ow + x) * 3 + q] = acc * inv;
          }
    };
    downTo(aNrm, dn);
    downTo(aAlb, da);
    denoiseAtrous(ow, oh, fin.data(), dn.data(), d.denoise_demodulate_albedo ? da.data() : nullptr,
                  std::max(0, d.denoise_iters), d.denoise_sigma_n, d.denoise_sigma_l);
  }
  // image_ops.cpp:37-46 applyAssumedGamma
  const float g = d.assumed_gamma;
  if (!(std::fabs(g - 1.0f) <= 1.0e-4f)) {
    const size_t np = fin.size() / 4;
    for (size_t i = 0; i < np; ++i)
      for (int ch = 0; ch < 3; ++ch) {
        float vv = fin[4 * i + ch];
        fin[4 * i + ch] = (vv > 0.0f) ? std::pow(vv, g) : 0.0f;
      }
  }
  // AO AOVs box-averaged to the output (pipeline.cpp:182-206)
  if (aov) {
    auto down = [&](const std::vector<float>& src, int ch, float* dst) {
      if (!dst) return;
      if (ss == 1) {
        std::memcpy(dst, src.data(), src.size() * sizeof(float));
        return;
      }
      const int ow = W / ss, oh = H / ss;
      const float inv = 1.0f / static_cast<float>(ss * ss);
      for (int y = 0; y < oh; ++y)
        for (int x = 0; x < ow; ++x)
          for (int q = 0; q < ch; ++q) {
            float acc = 0.0f;
            for (int dy = 0; dy < ss; ++dy)
              for (int dx = 0; dx < ss; ++dx) {
                const float vv = src[(static_cast<size_t>(y * ss + dy) * W + (x * ss + dx)) * ch + q];
                acc += std::isfinite(vv) ? vv : 0.0f;
              }
            dst[(static_cast<size_t>(y) * ow + x) * ch + q] = acc * inv;
          }
    };
    down(aAlb, 3, fr->albedo);
    down(aNrm, 3, fr->normal);
    down(aBent, 3, fr->bent_normal);
    down(aCon, 1, fr->contact_ao);
    down(aShp, 1, fr->shape_ao);
    down(aAvg, 1, fr->avg_hit_dist);
  }
  if (fr->color) std::memcpy(fr->color, fin.data(), fin.size() * sizeof(float));
  if (fr->depth) std::memcpy(fr->depth, depth.data(), npix * sizeof(float));
  if (fr->view_z) std::memcpy(fr->view_z, viewZ.data(), npix * sizeof(float));
  if (fr->hit_geom) std::memcpy(fr->hit_geom, hg.data(), npix * sizeof(uint32_t));
  if (fr->hit_prim) std::memcpy(fr->hit_prim, hp.data(), npix * sizeof(uint32_t));
  return 0;
}

int oracle_render(void* sp, const ubr_render_desc* d, ubr_frame* fr, int threads) {
  return oracle_render_rows(sp, d, fr, threads, 0, 0);
}

}  // extern "C"

// scene_build.cu -- ubr_scene_build: scene flattening + GPU LBVH.
//
// Host side: flatten ubr_scene_desc into per-kind primitive arrays in the
// reference's primID order (render/scene_build.cpp:16-129 for the mesh and
// spheres, render/curve_build.cpp:41-267 for open-cylinder chains and capped
// cylinders), deduplicate materials into one table, upload.
// Device side: a linear BVH (Karras, "Maximizing Parallelism in the
// Construction of BVHs, Octrees, and k-d Trees", HPG 2012):
//   k_prim_bounds  per-primitive AABB + centroid, centroid-bounds reduction
//   k_morton       30-bit Morton code << idxBits | primitive index (unique)
//   radix sort     CUB DeviceRadixSort over the used key bits only
//   k_hierarchy    binary radix tree from longest common prefixes
//   k_refit        leaves write their box into the parent, the second
//                  arrival at each node (atomic counter) unions and climbs
// The result replaces the Embree HIGH-quality BVH the reference commits
// (scene_build.cpp:138-163); hits do not depend on the tree, only on the
// intersectors, except for exact-t ties which resolve to the lowest
// (geomID, primID).
#include <cub/cub.cuh>

#include <array>
#include <chrono>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <map>
#include <unordered_map>
#include <vector>

#include "ubr_context.h"

namespace ubr {

namespace {

struct HostScene {
  std::vector<float> pos, nrm;        // 3 per baked vertex
  std::vector<float4> col;            // per baked vertex
  std::vector<uint32_t> idx;          // 3 per triangle (baked)
  std::vector<uint32_t> triMat;       // per base triangle (material index)
  std::vector<uint8_t> triMatId;      // per base triangle: the caller's Mesh::triMaterialId
  uint32_t meshMat = 0;
  uint32_t baseTri = 0;
  std::vector<float4> sph;            // (c, r)
  uint32_t baseSph = 0;               // spheres per instance
  std::vector<float4> rcV;            // round curve vertices (xyz, r)
  std::vector<uint32_t> rcIdx;
  std::vector<uint8_t> rcFlags;
  std::vector<float4> rcClip;         // 2 per segment
  std::vector<float4> ccV;
  std::vector<uint32_t> ccIdx;
  std::vector<float4> color[4];
  std::vector<uint32_t> mat[4];
  std::vector<uint8_t> fromEdge[4];
  std::vector<float> opacity1[4];
  std::vector<uint16_t> group[4];     // CueMol section per primitive (primID order)
  std::vector<float4> axis[4];        // cylinder unit axis (anisotropic principled scenes only)
  std::vector<uint16_t> triGroup;     // per base triangle
  std::vector<ubr_material> mats;
  uint32_t geomID[4] = {kInvalid, kInvalid, kInvalid, kInvalid};
  bool principled = false;
  bool opaque = true;
  std::vector<int> openIdx, capIdx;   // scratch of the cylinder split

  // Empty every table but keep its storage: a host thread that builds many
  // scenes reuses the same pages (first touch of fresh pages was half of the
  // flatten time of a 40k-primitive scene).
  void reset() {
    auto clr = [](auto&... v) { (v.clear(), ...); };
    clr(pos, nrm, col, idx, triMat, triMatId, sph, rcV, rcIdx, rcFlags, rcClip, ccV, ccIdx, triGroup, mats,
        openIdx, capIdx);
    for (int k = 0; k < 4; ++k) clr(color[k], mat[k], fromEdge[k], opacity1[k], group[k], axis[k]);
    meshMat = baseTri = baseSph = 0;
    for (int k = 0; k < 4; ++k) geomID[k] = kInvalid;
    principled = false;
    opaque = true;
  }
  size_t capacityBytes() const {
    size_t b = 0;
    auto add = [&](const auto&... v) { ((b += v.capacity() * sizeof(v[0])), ...); };
    add(pos, nrm, col, idx, triMat, triMatId, sph, rcV, rcIdx, rcFlags, rcClip, ccV, ccIdx, triGroup, mats,
        openIdx, capIdx);
    for (int k = 0; k < 4; ++k) add(color[k], mat[k], fromEdge[k], opacity1[k], group[k], axis[k]);
    return b;
  }
};

struct MatKey {
  ubr_material m;
  bool operator==(const MatKey& o) const { return std::memcmp(&m, &o.m, sizeof(m)) == 0; }
};
struct MatHash {
  size_t operator()(const MatKey& k) const {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&k.m);
    size_t h = 1469598103934665603ull;
    for (size_t i = 0; i < sizeof(k.m); ++i) h = (h ^ p[i]) * 1099511628211ull;
    return h;
  }
};

struct MatTable {
  std::unordered_map<MatKey, uint32_t, MatHash> map;
  std::vector<ubr_material>* out;
  ubr_material last{};
  uint32_t lastId = kInvalid;
  uint32_t get(const ubr_material& m) {
    // runs of one material (the common case) skip the hash lookup
    if (lastId != kInvalid && std::memcmp(&m, &last, sizeof(ubr_material)) == 0) return lastId;
    MatKey k{m};
    auto it = map.find(k);
    uint32_t id;
    if (it != map.end()) {
      id = it->second;
    } else {
      id = static_cast<uint32_t>(out->size());
      out->push_back(m);
      map.emplace(k, id);
    }
    last = m;
    lastId = id;
    return id;
  }
};

f3 ld3(const float* p, size_t i) { return f3{p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }

// The per-primitive side tables of `kind` for n base primitives repeated over
// ni instances (colour, material index, from-edge flag, group, opacity at the
// far end), written in place: every instance's block equals the base block.
template <class MatOf>
void fillSide(HostScene& s, int kind, size_t n, size_t ni, const float* color, const uint8_t* fromEdge,
              const uint16_t* group, const float* opacity1, MatOf matOf) {
  s.color[kind].resize(n * ni);
  s.mat[kind].resize(n * ni);
  s.fromEdge[kind].resize(n * ni);
  s.group[kind].resize(n * ni);
  if (opacity1) s.opacity1[kind].resize(n * ni);
  float4* c = s.color[kind].data();
  uint32_t* m = s.mat[kind].data();
  uint8_t* fe = s.fromEdge[kind].data();
  uint16_t* g = s.group[kind].data();
  std::memcpy(c, color, n * sizeof(float4));
  for (size_t i = 0; i < n; ++i) m[i] = matOf(i);
  for (size_t i = 0; i < n; ++i) fe[i] = fromEdge && fromEdge[i] ? 1 : 0;
  if (group) std::memcpy(g, group, n * sizeof(uint16_t));
  else std::memset(g, 0, n * sizeof(uint16_t));
  if (opacity1) std::memcpy(s.opacity1[kind].data(), opacity1, n * sizeof(float));
  for (size_t ci = 1; ci < ni; ++ci) {
    std::memcpy(c + ci * n, c, n * sizeof(float4));
    std::memcpy(m + ci * n, m, n * sizeof(uint32_t));
    std::memcpy(fe + ci * n, fe, n);
    std::memcpy(g + ci * n, g, n * sizeof(uint16_t));
    if (opacity1) std::memcpy(s.opacity1[kind].data() + ci * n, opacity1, n * sizeof(float));
  }
}

// curve_build.cpp:41-267, restated: open cylinders are chained into polylines
// through endpoints quantised at 1e-4 (a vertex of degree 2 continues a chain
// when group and opacity-gradient kind agree); each chain emits chainLen + 1
// vertices whose radius is that of the segment ending there; segments carry
// neighbour flags (bit0 left, bit1 right).  Capped cylinders become single
// cone segments.  Both in instance-major order.
void flattenCylinders(const ubr_scene_desc& d, const std::vector<f3>& offs, HostScene& s,
                      MatTable& mt) {
  const size_t n = d.cylinder_count;
  if (n == 0) return;
  std::vector<int>& openIdx = s.openIdx;
  std::vector<int>& capIdx = s.capIdx;
  for (size_t i = 0; i < n; ++i) {
    if (d.cyl_open && d.cyl_open[i]) openIdx.push_back(int(i));
    else capIdx.push_back(int(i));
  }
  auto op1 = [&](int i) { return d.cyl_opacity1 ? d.cyl_opacity1[i] : -1.0f; };
  auto grp = [&](int i) { return d.cyl_group ? d.cyl_group[i] : uint16_t(0); };
  // per-segment axes only when an anisotropic principled cylinder exists
  // (curve_build.cpp:45-54): the tangent frame of its highlight
  bool axisTables = false;
  for (size_t i = 0; i < n && !axisTables; ++i)
    axisTables = d.cyl_material[i].model == 1 && d.cyl_material[i].pbr_anisotropy != 0.0f;
  auto pushAxis = [&](int kind, f3 a) {
    const f3 u = safeNormalize(a);
    s.axis[kind].push_back(make_float4(u.x, u.y, u.z, 0.0f));
  };
  auto side = [&](int kind, int i) {
    s.color[kind].push_back(make_float4(d.cyl_color[4 * i], d.cyl_color[4 * i + 1],
                                        d.cyl_color[4 * i + 2], d.cyl_color[4 * i + 3]));
    s.mat[kind].push_back(mt.get(d.cyl_material[i]));
    s.fromEdge[kind].push_back(d.cyl_from_edge && d.cyl_from_edge[i] ? 1 : 0);
    s.group[kind].push_back(grp(i));
    s.opacity1[kind].push_back(op1(i));
  };
  if (!openIdx.empty()) {
    const size_t no = openIdx.size();
    const float eps = 1.0e-4f;
    using Key = std::array<long long, 3>;
    auto keyOf = [&](const f3& p) {
      return Key{std::llround(p.x / eps), std::llround(p.y / eps), std::llround(p.z / eps)};
    };
    for (const f3& off : offs) {
      std::vector<f3> a0(no), a1(no);
      for (size_t i = 0; i < no; ++i) {
        a0[i] = ld3(d.cyl_p0, openIdx[i]) + off;
        a1[i] = ld3(d.cyl_p1, openIdx[i]) + off;
      }
      std::map<Key, std::vector<std::pair<int, int>>> inc;
      for (int i = 0; i < int(no); ++i) {
        inc[keyOf(a0[i])].push_back({i, 0});
        inc[keyOf(a1[i])].push_back({i, 1});
      }
      std::vector<int> next(no, -1), prev(no, -1);
      for (int sg = 0; sg < int(no); ++sg) {
        const auto& ends = inc[keyOf(a1[sg])];
        if (ends.size() != 2) continue;
        int t = -1;
        for (const auto& e : ends)
          if (e.first != sg) t = (e.second == 0) ? e.first : -1;
        if (t >= 0 && t != sg && grp(openIdx[sg]) == grp(openIdx[t]) &&
            (op1(openIdx[sg]) < 0.0f) == (op1(openIdx[t]) < 0.0f))
          next[sg] = t;
      }
      for (int sg = 0; sg < int(no); ++sg)
        if (next[sg] >= 0) prev[next[sg]] = sg;
      std::vector<char> visited(no, 0);
      auto emit = [&](int start) {
        std::vector<int> chain;
        for (int sg = start; sg >= 0 && !visited[sg]; sg = next[sg]) {
          visited[sg] = 1;
          chain.push_back(sg);
        }
        const uint32_t base = uint32_t(s.rcV.size());
        const f3 q = a0[chain[0]];
        s.rcV.push_back(make_float4(q.x, q.y, q.z, d.cyl_radius[openIdx[chain[0]]]));
        for (int cs : chain)
          s.rcV.push_back(make_float4(a1[cs].x, a1[cs].y, a1[cs].z, d.cyl_radius[openIdx[cs]]));
        const int nc = int(chain.size());
        for (int j = 0; j < nc; ++j) {
          s.rcIdx.push_back(base + uint32_t(j));
          uint8_t fl = 0;
          if (j > 0) fl |= 1u;
          if (j < nc - 1) fl |= 2u;
          s.rcFlags.push_back(fl);
          side(kRound, openIdx[chain[j]]);
          if (axisTables) pushAxis(kRound, a1[chain[j]] - a0[chain[j]]);
        }
      };
      for (int sg = 0; sg < int(no); ++sg)
        if (prev[sg] < 0 && !visited[sg]) emit(sg);
      for (int sg = 0; sg < int(no); ++sg)
        if (!visited[sg]) emit(sg);
    }
    // bisector clip planes at chain joints
    auto vtx = [&](uint32_t i) { return f3{s.rcV[i].x, s.rcV[i].y, s.rcV[i].z}; };
    for (size_t sg = 0; sg < s.rcIdx.size(); ++sg) {
      const uint32_t v = s.rcIdx[sg];
      const f3 p0 = vtx(v), p1 = vtx(v + 1);
      const f3 dir = normalize(p1 - p0);
      f3 cl{0, 0, 0}, cr{0, 0, 0};
      if (s.rcFlags[sg] & 1u) cl = normalize(dir + normalize(p0 - vtx(v - 1)));
      if (s.rcFlags[sg] & 2u) cr = normalize(dir + normalize(vtx(v + 2) - p1));
      s.rcClip.push_back(make_float4(cl.x, cl.y, cl.z, 0.0f));
      s.rcClip.push_back(make_float4(cr.x, cr.y, cr.z, 0.0f));
    }
  }
  if (capIdx.empty()) return;
  // capped cylinders: one cone segment each, side tables written in place
  const size_t nc = capIdx.size(), ni = offs.size();
  s.ccV.resize(2 * nc * ni);
  s.ccIdx.resize(nc * ni);
  s.color[kCone].resize(nc * ni);
  s.mat[kCone].resize(nc * ni);
  s.fromEdge[kCone].resize(nc * ni);
  s.group[kCone].resize(nc * ni);
  s.opacity1[kCone].resize(nc * ni);
  for (size_t j = 0; j < nc; ++j) {
    const int i = capIdx[j];
    s.color[kCone][j] = make_float4(d.cyl_color[4 * i], d.cyl_color[4 * i + 1], d.cyl_color[4 * i + 2],
                                    d.cyl_color[4 * i + 3]);
    s.mat[kCone][j] = mt.get(d.cyl_material[i]);
    s.fromEdge[kCone][j] = d.cyl_from_edge && d.cyl_from_edge[i] ? 1 : 0;
    s.group[kCone][j] = grp(i);
    s.opacity1[kCone][j] = op1(i);
  }
  for (size_t ci = 1; ci < ni; ++ci) {
    std::copy_n(s.color[kCone].begin(), nc, s.color[kCone].begin() + ci * nc);
    std::copy_n(s.mat[kCone].begin(), nc, s.mat[kCone].begin() + ci * nc);
    std::copy_n(s.fromEdge[kCone].begin(), nc, s.fromEdge[kCone].begin() + ci * nc);
    std::copy_n(s.group[kCone].begin(), nc, s.group[kCone].begin() + ci * nc);
    std::copy_n(s.opacity1[kCone].begin(), nc, s.opacity1[kCone].begin() + ci * nc);
  }
  for (size_t ci = 0; ci < ni; ++ci) {
    const f3 off = offs[ci];
    for (size_t j = 0; j < nc; ++j) {
      const int i = capIdx[j];
      const size_t k = ci * nc + j;
      const f3 a = ld3(d.cyl_p0, i) + off, b = ld3(d.cyl_p1, i) + off;
      const float r = d.cyl_radius[i];
      s.ccV[2 * k] = make_float4(a.x, a.y, a.z, r);
      s.ccV[2 * k + 1] = make_float4(b.x, b.y, b.z, r);
      s.ccIdx[k] = uint32_t(2 * k);
      if (axisTables) pushAxis(kCone, ld3(d.cyl_p1, i) - ld3(d.cyl_p0, i));
    }
  }
}

// pt2BuildEmissiveLights (integrator/pt2/pt2_emissive.hpp:104-277): the
// base mesh triangles whose material emits (corners and colours as the
// caller gave them, un-offset), then the real emissive spheres and capped
// cylinders in primID order (instance offset outer, scene order inner) --
// a sphere as one record, a capped cylinder as its lateral surface and two
// disk caps -- each weighted by area x luminance(emitted radiance) in one CDF
// accumulated in double.  Records in the EmitD layout (gi.cuh).
struct HostEmit {
  std::vector<float4> rec;
  std::vector<float> cdf, pdf;
  std::vector<uint32_t> triIndex, sphereIndex;
  std::vector<uint4> cylIndex;
  uint32_t triCount = 0;
};

void buildEmitters(const ubr_scene_desc& d, const std::vector<f3>& offs, HostEmit& e) {
  auto lum = [](f3 c) { return 0.2126f * c.x + 0.7152f * c.y + 0.0722f * c.z; };
  const uint64_t nt = d.mesh_vertex_count >= 3 ? d.mesh_triangle_count : 0;
  auto triMat = [&](uint64_t t) -> const ubr_material& {
    return d.mesh_tri_material ? d.mesh_materials[d.mesh_tri_material[t]] : d.mesh_material;
  };
  bool meshEm = d.mesh_material.emission > 0.0f;
  for (uint32_t i = 0; i < d.mesh_material_count && d.mesh_materials; ++i)
    meshEm = meshEm || d.mesh_materials[i].emission > 0.0f;
  bool csgEm = false;
  for (uint64_t i = 0; i < d.sphere_count; ++i)
    csgEm = csgEm || (!(d.sphere_from_edge && d.sphere_from_edge[i]) && d.sphere_material[i].emission > 0.0f &&
                      d.sphere_center_radius[4 * i + 3] > 0.0f);
  for (uint64_t i = 0; i < d.cylinder_count; ++i)
    csgEm = csgEm || (!(d.cyl_from_edge && d.cyl_from_edge[i]) && !(d.cyl_open && d.cyl_open[i]) &&
                      d.cyl_material[i].emission > 0.0f && d.cyl_radius[i] > 0.0f);
  if (!(meshEm && nt > 0) && !csgEm) return;
  std::vector<float> power;
  if (meshEm && nt > 0) {
    e.triIndex.assign(nt, 0xFFFFFFFFu);
    for (uint64_t t = 0; t < nt; ++t) {
      const ubr_material& mm = triMat(t);
      if (mm.emission <= 0.0f) continue;
      uint32_t vi[3];
      for (int k = 0; k < 3; ++k) vi[k] = d.mesh_index ? d.mesh_index[3 * t + k] : uint32_t(3 * t + k);
      f3 P[3], Em[3];
      for (int k = 0; k < 3; ++k) {
        P[k] = ld3(d.mesh_positions, vi[k]);
        const float* cc = d.mesh_colors ? d.mesh_colors + 4 * size_t(vi[k]) : nullptr;
        Em[k] = cc ? f3{mm.emission * cc[0], mm.emission * cc[1], mm.emission * cc[2]} : f3{0.0f, 0.0f, 0.0f};
      }
      const f3 a = P[1] - P[0], b = P[2] - P[0];
      const f3 cr{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
      const float len = std::sqrt(cr.x * cr.x + cr.y * cr.y + cr.z * cr.z);
      if (len <= 0.0f) continue;
      const float area = 0.5f * len;
      const f3 avg{(Em[0].x + Em[1].x + Em[2].x) / 3.0f, (Em[0].y + Em[1].y + Em[2].y) / 3.0f,
                   (Em[0].z + Em[1].z + Em[2].z) / 3.0f};
      const float pw = area * lum(avg);
      if (pw <= 0.0f) continue;
      e.triIndex[t] = uint32_t(power.size());
      e.rec.push_back(make_float4(P[0].x, P[0].y, P[0].z, area));
      e.rec.push_back(make_float4(P[1].x, P[1].y, P[1].z, 0.0f));
      e.rec.push_back(make_float4(P[2].x, P[2].y, P[2].z, 0.0f));
      for (int k = 0; k < 3; ++k) e.rec.push_back(make_float4(Em[k].x, Em[k].y, Em[k].z, 0.0f));
      e.rec.push_back(make_float4(cr.x / len, cr.y / len, cr.z / len, 0.0f));
      power.push_back(pw);
    }
    if (power.empty()) e.triIndex.clear();
  }
  e.triCount = uint32_t(power.size());
  if (csgEm) {
    const float kPi = 3.14159265358979323846f;
    auto pushCsg = [&](f3 p0, f3 axis, int kind, f3 Le, float radius, float len, float area) {
      e.rec.push_back(make_float4(p0.x, p0.y, p0.z, area));
      e.rec.push_back(make_float4(axis.x, axis.y, axis.z, float(kind)));
      e.rec.push_back(make_float4(Le.x, Le.y, Le.z, radius));
      e.rec.push_back(make_float4(len, 0.0f, 0.0f, 0.0f));
      for (int k = 4; k < kEmitF4; ++k) e.rec.push_back(make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    };
    const uint32_t nCsg0 = uint32_t(power.size());
    e.sphereIndex.assign(d.sphere_count * offs.size(), 0xFFFFFFFFu);
    uint32_t prim = 0;
    for (const f3& off : offs)
      for (uint64_t i = 0; i < d.sphere_count; ++i, ++prim) {
        const ubr_material& m = d.sphere_material[i];
        const float r = d.sphere_center_radius[4 * i + 3];
        if ((d.sphere_from_edge && d.sphere_from_edge[i]) || !(m.emission > 0.0f) || !(r > 0.0f)) continue;
        const f3 Le{m.emission * d.sphere_color[4 * i], m.emission * d.sphere_color[4 * i + 1],
                    m.emission * d.sphere_color[4 * i + 2]};
        const float area = 4.0f * kPi * r * r;
        const float pw = area * lum(Le);
        if (!(pw > 0.0f)) continue;
        e.sphereIndex[prim] = uint32_t(power.size()) - e.triCount;
        const float* q = d.sphere_center_radius + 4 * i;
        pushCsg(f3{q[0] + off.x, q[1] + off.y, q[2] + off.z}, f3{0.0f, 0.0f, 1.0f}, 1, Le, r, 0.0f, area);
        power.push_back(pw);
      }
    std::vector<uint32_t> capIdx;
    for (uint64_t i = 0; i < d.cylinder_count; ++i)
      if (!(d.cyl_open && d.cyl_open[i])) capIdx.push_back(uint32_t(i));
    const uint32_t none = 0xFFFFFFFFu;
    e.cylIndex.assign(capIdx.size() * offs.size(), make_uint4(none, none, none, 0));
    prim = 0;
    for (const f3& off : offs)
      for (uint32_t i : capIdx) {
        const uint32_t me = prim++;
        const ubr_material& m = d.cyl_material[i];
        const float r = d.cyl_radius[i];
        if ((d.cyl_from_edge && d.cyl_from_edge[i]) || !(m.emission > 0.0f) || !(r > 0.0f)) continue;
        const f3 p0 = ld3(d.cyl_p0, i) + off, p1 = ld3(d.cyl_p1, i) + off;
        const f3 dd = p1 - p0;
        const float len = std::sqrt(dd.x * dd.x + dd.y * dd.y + dd.z * dd.z);
        if (!(len > 0.0f)) continue;
        const f3 axis{dd.x / len, dd.y / len, dd.z / len};
        const f3 Le{m.emission * d.cyl_color[4 * i], m.emission * d.cyl_color[4 * i + 1],
                    m.emission * d.cyl_color[4 * i + 2]};
        const float l = lum(Le);
        uint4& ref = e.cylIndex[me];
        const float aSide = 2.0f * kPi * r * len;
        if (aSide * l > 0.0f) {
          ref.x = uint32_t(power.size()) - e.triCount;
          pushCsg(p0, axis, 2, Le, r, len, aSide);
          power.push_back(aSide * l);
        }
        const float aCap = kPi * r * r;
        if (aCap * l > 0.0f) {
          ref.y = uint32_t(power.size()) - e.triCount;
          pushCsg(p0, axis, 3, Le, r, 0.0f, aCap);
          power.push_back(aCap * l);
          ref.z = uint32_t(power.size()) - e.triCount;
          pushCsg(p1, axis, 3, Le, r, 0.0f, aCap);
          power.push_back(aCap * l);
        }
      }
    if (uint32_t(power.size()) == nCsg0) {
      e.sphereIndex.clear();
      e.cylIndex.clear();
    }
  }
  if (power.empty()) {
    e = HostEmit{};
    return;
  }
  double total = 0.0;
  for (float pw : power) total += pw;
  double acc = 0.0;
  for (float pw : power) {
    acc += pw;
    e.cdf.push_back(float(acc / total));
    e.pdf.push_back(float(pw / total));
  }
  e.cdf.back() = 1.0f;
}

ubr_status validate(Context* c, const ubr_scene_desc& d) {
  if (d.abi_version != UBR_ABI_VERSION) return setError(c, UBR_INVALID_ARGUMENT, "scene desc: abi_version mismatch");
  if (d.mesh_triangle_count > 0 && d.mesh_vertex_count >= 3 && !d.mesh_positions)
    return setError(c, UBR_INVALID_ARGUMENT, "scene desc: mesh_positions is NULL");
  if (d.mesh_index) {
    for (uint64_t i = 0; i < 3 * d.mesh_triangle_count; ++i)
      if (d.mesh_index[i] >= d.mesh_vertex_count)
        return setError(c, UBR_INVALID_ARGUMENT, "scene desc: mesh_index out of range");
  } else if (d.mesh_triangle_count * 3 > d.mesh_vertex_count) {
    return setError(c, UBR_INVALID_ARGUMENT, "scene desc: de-indexed mesh needs 3 vertices per triangle");
  }
  if (d.mesh_tri_material) {
    for (uint64_t i = 0; i < d.mesh_triangle_count; ++i)
      if (d.mesh_tri_material[i] >= d.mesh_material_count)
        return setError(c, UBR_INVALID_ARGUMENT, "scene desc: mesh_tri_material out of range");
  }
  if (d.sphere_count && (!d.sphere_center_radius || !d.sphere_color || !d.sphere_material))
    return setError(c, UBR_INVALID_ARGUMENT, "scene desc: sphere arrays missing");
  if (d.cylinder_count && (!d.cyl_p0 || !d.cyl_p1 || !d.cyl_radius || !d.cyl_color || !d.cyl_material))
    return setError(c, UBR_INVALID_ARGUMENT, "scene desc: cylinder arrays missing");
  if (d.instance_count && !d.instance_offsets)
    return setError(c, UBR_INVALID_ARGUMENT, "scene desc: instance_offsets missing");
  return UBR_OK;
}

ubr_status flatten(Context* c, const ubr_scene_desc& d, HostScene& s) {
  std::vector<f3> offs;
  for (uint64_t i = 0; i < d.instance_count; ++i) offs.push_back(ld3(d.instance_offsets, i));
  if (offs.empty()) offs.push_back(f3{0, 0, 0});
  const uint64_t total = (d.mesh_triangle_count + d.sphere_count + d.cylinder_count) * offs.size();
  if (total >= (1ull << 30)) return setError(c, UBR_INVALID_ARGUMENT, "scene too large (>= 2^30 primitives)");
  MatTable mt;
  mt.out = &s.mats;
  uint32_t nextGeom = 0;
  const uint64_t baseV = d.mesh_vertex_count, baseT = d.mesh_triangle_count;
  if (baseV >= 3 && baseT > 0) {
    s.geomID[kMesh] = nextGeom++;
    // baked per instance (scene_build.cpp:150-152), written in place
    const size_t nInst = offs.size();
    s.pos.resize(3 * baseV * nInst);
    s.nrm.resize(3 * baseV * nInst);
    s.col.resize(baseV * nInst);
    s.idx.resize(3 * baseT * nInst);
    for (size_t ci = 0; ci < nInst; ++ci) {
      const f3 off = offs[ci];
      float* pos = s.pos.data() + 3 * baseV * ci;
      float* nrm = s.nrm.data() + 3 * baseV * ci;
      float4* col = s.col.data() + baseV * ci;
      for (uint64_t v = 0; v < baseV; ++v) {
        const f3 p = ld3(d.mesh_positions, v) + off;
        pos[3 * v] = p.x;
        pos[3 * v + 1] = p.y;
        pos[3 * v + 2] = p.z;
      }
      if (d.mesh_normals) std::memcpy(nrm, d.mesh_normals, 3 * baseV * sizeof(float));
      else std::memset(nrm, 0, 3 * baseV * sizeof(float));
      if (d.mesh_colors) {
        std::memcpy(col, d.mesh_colors, baseV * sizeof(float4));
      } else {
        for (uint64_t v = 0; v < baseV; ++v) col[v] = make_float4(0, 0, 0, 1);
      }
      uint32_t* idx = s.idx.data() + 3 * baseT * ci;
      const uint32_t vb = uint32_t(ci * baseV);
      if (d.mesh_index) {
        for (uint64_t k = 0; k < 3 * baseT; ++k) idx[k] = vb + d.mesh_index[k];
      } else {
        for (uint64_t k = 0; k < 3 * baseT; ++k) idx[k] = vb + uint32_t(k);
      }
    }
    s.baseTri = uint32_t(baseT);
    if (d.mesh_tri_group) s.triGroup.assign(d.mesh_tri_group, d.mesh_tri_group + baseT);
    s.meshMat = mt.get(d.mesh_material);
    if (d.mesh_tri_material) {
      std::vector<uint32_t> remap(d.mesh_material_count);
      for (uint32_t i = 0; i < d.mesh_material_count; ++i) remap[i] = mt.get(d.mesh_materials[i]);
      s.triMat.resize(baseT);
      for (uint64_t t = 0; t < baseT; ++t) s.triMat[t] = remap[d.mesh_tri_material[t]];
      s.triMatId.assign(d.mesh_tri_material, d.mesh_tri_material + baseT);
    }
  }
  if (d.sphere_count > 0) {
    s.geomID[kSphere] = nextGeom++;
    const size_t n = d.sphere_count, ni = offs.size();
    s.baseSph = uint32_t(n);
    s.sph.resize(n * ni);
    // side tables: one block per instance, all equal to the base spheres'
    fillSide(s, kSphere, n, ni, d.sphere_color, d.sphere_from_edge, d.sphere_group, nullptr,
             [&](size_t i) { return mt.get(d.sphere_material[i]); });
    for (size_t ci = 0; ci < ni; ++ci) {
      const f3 off = offs[ci];
      float4* out = s.sph.data() + ci * n;
      for (size_t i = 0; i < n; ++i) {
        const float* q = d.sphere_center_radius + 4 * i;
        out[i] = make_float4(q[0] + off.x, q[1] + off.y, q[2] + off.z, q[3]);
      }
    }
  }
  flattenCylinders(d, offs, s, mt);
  if (!s.rcIdx.empty()) s.geomID[kRound] = nextGeom++;
  if (!s.ccIdx.empty()) s.geomID[kCone] = nextGeom++;
  for (const ubr_material& m : s.mats)
    if (m.model == 1) s.principled = true;
  // a scene whose every surface is opaque renders in one transparency round
  const float kOpaque = 1.0f - 1e-4f;
  for (const float4& c : s.col)
    if (!(c.w >= kOpaque)) s.opaque = false;
  for (int k = 1; k < 4; ++k) {
    for (const float4& c : s.color[k])
      if (!(c.w >= kOpaque)) s.opaque = false;
    for (float o1 : s.opacity1[k])
      if (o1 >= 0.0f && !(o1 >= kOpaque)) s.opaque = false;
  }
  return UBR_OK;
}

// ---------------------------------------------------------------------------
// device build

struct BuildIn {
  const float* pos;
  const uint32_t* idx;
  const float4* sph;
  const float4* rcV;
  const uint32_t* rcIdx;
  const uint8_t* rcFlags;
  const float4* ccV;
  const uint32_t* ccIdx;
  uint32_t nTri, nSph, nRc, nCc;
};

__device__ __forceinline__ void globalToRef(const BuildIn& in, uint32_t g, int& kind, uint32_t& prim) {
  if (g < in.nTri) { kind = kMesh; prim = g; return; }
  g -= in.nTri;
  if (g < in.nSph) { kind = kSphere; prim = g; return; }
  g -= in.nSph;
  if (g < in.nRc) { kind = kRound; prim = g; return; }
  kind = kCone;
  prim = g - in.nRc;
}

__device__ __forceinline__ int orderedInt(float f) {
  int i = __float_as_int(f);
  return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float orderedFloat(int i) {
  return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF);
}

__global__ void k_prim_bounds(BuildIn in, uint32_t n, float4* boxLo, float4* boxHi, int* cbounds) {
  __shared__ int sm[6][32];
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  float3 lo = make_float3(1e30f, 1e30f, 1e30f), hi = make_float3(-1e30f, -1e30f, -1e30f);
  float3 cen = make_float3(0, 0, 0);
  const bool valid = g < n;
  if (valid) {
    int kind;
    uint32_t prim;
    globalToRef(in, g, kind, prim);
    auto grow = [&](float x, float y, float z, float r) {
      lo.x = fminf(lo.x, x - r); lo.y = fminf(lo.y, y - r); lo.z = fminf(lo.z, z - r);
      hi.x = fmaxf(hi.x, x + r); hi.y = fmaxf(hi.y, y + r); hi.z = fmaxf(hi.z, z + r);
    };
    if (kind == kMesh) {
      for (int k = 0; k < 3; ++k) {
        const uint32_t v = in.idx[3 * prim + k];
        grow(in.pos[3 * v], in.pos[3 * v + 1], in.pos[3 * v + 2], 0.0f);
      }
    } else if (kind == kSphere) {
      const float4 q = in.sph[prim];
      grow(q.x, q.y, q.z, q.w);
    } else {
      const float4* V = kind == kRound ? in.rcV : in.ccV;
      const uint32_t v = kind == kRound ? in.rcIdx[prim] : in.ccIdx[prim];
      const float4 a = V[v], b = V[v + 1];
      grow(a.x, a.y, a.z, a.w);
      grow(b.x, b.y, b.z, b.w);
    }
    // conservative padding: relative to the extent and the magnitude
    const float m = 1e-6f * fmaxf(fmaxf(fmaxf(fabsf(lo.x), fabsf(lo.y)), fmaxf(fabsf(lo.z), fabsf(hi.x))),
                                  fmaxf(fmaxf(fabsf(hi.y), fabsf(hi.z)), 1.0f));
    const float ex = (hi.x - lo.x) * 1e-6f + m, ey = (hi.y - lo.y) * 1e-6f + m, ez = (hi.z - lo.z) * 1e-6f + m;
    lo.x -= ex; lo.y -= ey; lo.z -= ez;
    hi.x += ex; hi.y += ey; hi.z += ez;
    boxLo[g] = make_float4(lo.x, lo.y, lo.z, 0.0f);
    boxHi[g] = make_float4(hi.x, hi.y, hi.z, 0.0f);
    cen = make_float3(0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z));
  }
  // block reduction of centroid bounds
  int v[6];
  v[0] = valid ? orderedInt(cen.x) : 0x7FFFFFFF;
  v[1] = valid ? orderedInt(cen.y) : 0x7FFFFFFF;
  v[2] = valid ? orderedInt(cen.z) : 0x7FFFFFFF;
  v[3] = valid ? orderedInt(cen.x) : int(0x80000000);
  v[4] = valid ? orderedInt(cen.y) : int(0x80000000);
  v[5] = valid ? orderedInt(cen.z) : int(0x80000000);
  for (int o = 16; o > 0; o >>= 1) {
    for (int k = 0; k < 3; ++k) v[k] = min(v[k], __shfl_xor_sync(0xFFFFFFFFu, v[k], o));
    for (int k = 3; k < 6; ++k) v[k] = max(v[k], __shfl_xor_sync(0xFFFFFFFFu, v[k], o));
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0)
    for (int k = 0; k < 6; ++k) sm[k][warp] = v[k];
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    for (int k = 0; k < 6; ++k) v[k] = lane < nw ? sm[k][lane] : (k < 3 ? 0x7FFFFFFF : int(0x80000000));
    for (int o = 16; o > 0; o >>= 1) {
      for (int k = 0; k < 3; ++k) v[k] = min(v[k], __shfl_xor_sync(0xFFFFFFFFu, v[k], o));
      for (int k = 3; k < 6; ++k) v[k] = max(v[k], __shfl_xor_sync(0xFFFFFFFFu, v[k], o));
    }
    if (lane == 0) {
      for (int k = 0; k < 3; ++k) atomicMin(&cbounds[k], v[k]);
      for (int k = 3; k < 6; ++k) atomicMax(&cbounds[k], v[k]);
    }
  }
}

__device__ __forceinline__ uint32_t expandBits10(uint32_t v) {
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void k_morton(uint32_t n, int idxBits, const float4* boxLo, const float4* boxHi,
                         const int* cbounds, unsigned long long* keys) {
  const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= n) return;
  const float4 lo = boxLo[g], hi = boxHi[g];
  const float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
  uint32_t q[3];
  for (int k = 0; k < 3; ++k) {
    const float bl = orderedFloat(cbounds[k]), bh = orderedFloat(cbounds[3 + k]);
    const float ext = bh - bl;
    float f = ext > 0.0f ? (c[k] - bl) / ext : 0.0f;
    f = fminf(fmaxf(f, 0.0f), 1.0f);
    q[k] = min(uint32_t(f * 1024.0f), 1023u);
  }
  const uint32_t m = (expandBits10(q[0]) << 2) | (expandBits10(q[1]) << 1) | expandBits10(q[2]);
  keys[g] = (static_cast<unsigned long long>(m) << idxBits) | g;
}

__device__ __forceinline__ int deltaKey(const unsigned long long* keys, int n, int i, int j) {
  if (j < 0 || j >= n) return -1;
  return __clzll(keys[i] ^ keys[j]);
}

// Karras 2012, Fig. 4: internal node i covers [min(i,j), max(i,j)], split at gamma.
__global__ void k_hierarchy(int n, const unsigned long long* keys, float4* nodes, int* leafParent,
                            int* nodeParent, int2* ranges) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (deltaKey(keys, n, i, i + 1) - deltaKey(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = deltaKey(keys, n, i, i - d);
  int lmax = 2;
  while (deltaKey(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
  int l = 0;
  for (int t = lmax >> 1; t >= 1; t >>= 1)
    if (deltaKey(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = deltaKey(keys, n, i, j);
  int s = 0, t = l;
  do {
    t = (t + 1) >> 1;
    if (deltaKey(keys, n, i, i + (s + t) * d) > dnode) s += t;
  } while (t > 1);
  const int gamma = i + s * d + min(d, 0);
  const int lo = min(i, j), hi = max(i, j);
  ranges[i] = make_int2(lo, hi);
  int left, right;
  if (lo == gamma) {
    left = ~gamma;
    leafParent[gamma] = (i << 1) | 0;
  } else {
    left = gamma;
    nodeParent[gamma] = (i << 1) | 0;
  }
  if (hi == gamma + 1) {
    right = ~(gamma + 1);
    leafParent[gamma + 1] = (i << 1) | 1;
  } else {
    right = gamma + 1;
    nodeParent[gamma + 1] = (i << 1) | 1;
  }
  nodes[kNodeF4 * i + 3] = make_float4(__int_as_float(left), __int_as_float(right), 0.0f, 0.0f);
  if (i == 0) nodeParent[0] = -1;
}

__device__ __forceinline__ void writeChildBox(float4* nodes, int p, int side, float3 lo, float3 hi) {
  float4* nd = nodes + kNodeF4 * p;
  if (side == 0) {
    nd[0] = make_float4(lo.x, hi.x, lo.y, hi.y);
    float* z = reinterpret_cast<float*>(&nd[2]);
    z[0] = lo.z;
    z[1] = hi.z;
  } else {
    nd[1] = make_float4(lo.x, hi.x, lo.y, hi.y);
    float* z = reinterpret_cast<float*>(&nd[2]);
    z[2] = lo.z;
    z[3] = hi.z;
  }
}

// Leaf packing + bottom-up refit.  One thread per sorted slot.
__global__ void k_refit(BuildIn in, int n, int idxBits, const unsigned long long* keys,
                        const float4* boxLo, const float4* boxHi, const float4* rcClip,
                        float4* nodes, const int* leafParent, const int* nodeParent, int* counters,
                        uint32_t* leafRef, float4* leafGeo, int refit) {
  const int sIdx = blockIdx.x * blockDim.x + threadIdx.x;
  if (sIdx >= n) return;
  const uint32_t g = uint32_t(keys[sIdx] & ((1ull << idxBits) - 1ull));
  int kind;
  uint32_t prim;
  globalToRef(in, g, kind, prim);
  leafRef[sIdx] = packRef(kind, prim);
  float4* lg = leafGeo + kLeafF4 * sIdx;
  if (kind == kMesh) {
    for (int k = 0; k < 3; ++k) {
      const uint32_t v = in.idx[3 * prim + k];
      lg[k] = make_float4(in.pos[3 * v], in.pos[3 * v + 1], in.pos[3 * v + 2], 0.0f);
    }
  } else if (kind == kSphere) {
    lg[0] = in.sph[prim];
  } else {
    const float4* V = kind == kRound ? in.rcV : in.ccV;
    const uint32_t v = kind == kRound ? in.rcIdx[prim] : in.ccIdx[prim];
    lg[0] = V[v];
    lg[1] = V[v + 1];
    if (kind == kRound) {
      lg[2] = make_float4(__uint_as_float(uint32_t(in.rcFlags[prim])), 0, 0, 0);
    } else {
      f3 a;
      float L;
      segmentAxis(f3{V[v].x, V[v].y, V[v].z}, f3{V[v + 1].x, V[v + 1].y, V[v + 1].z}, a, L);
      lg[2] = make_float4(a.x, a.y, a.z, L);
    }
  }
  if (n == 1 || !refit) return;
  const float4 bl = boxLo[g], bh = boxHi[g];
  float3 lo = make_float3(bl.x, bl.y, bl.z), hi = make_float3(bh.x, bh.y, bh.z);
  int pinfo = leafParent[sIdx];
  while (pinfo >= 0) {
    const int p = pinfo >> 1, side = pinfo & 1;
    writeChildBox(nodes, p, side, lo, hi);
    __threadfence();
    if (atomicAdd(&counters[p], 1) == 0) return;
    __threadfence();
    const float4 a = __ldcg(&nodes[kNodeF4 * p + 0]);
    const float4 b = __ldcg(&nodes[kNodeF4 * p + 1]);
    const float4 z = __ldcg(&nodes[kNodeF4 * p + 2]);
    lo = make_float3(fminf(a.x, b.x), fminf(a.z, b.z), fminf(z.x, z.z));
    hi = make_float3(fmaxf(a.y, b.y), fmaxf(a.w, b.w), fmaxf(z.y, z.w));
    pinfo = nodeParent[p];
  }
}

// Locally-ordered clustering (PLOC: Meister and Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction",
// IEEE TVCG 2018).  Clusters start as the Morton-sorted leaves; each round
// every cluster finds its nearest neighbour within kPlocRadius positions by
// the surface area of the merged box, mutual nearest pairs merge into a new
// binary node (written in the radix tree's node format, child boxes
// included, so no refit is needed) and the cluster list is compacted in
// order.  The pair with the smallest distance (ties to the lowest indices)
// is always mutual, so every round merges at least once.
constexpr int kPlocRadius = 16;
constexpr int kPlocBlock = 256;
constexpr int kPlocBatch = 4;  // merge rounds between host reads of the cluster count

__device__ __forceinline__ float unionArea(float4 alo, float4 ahi, float4 blo, float4 bhi) {
  const float ex = fmaxf(ahi.x, bhi.x) - fminf(alo.x, blo.x);
  const float ey = fmaxf(ahi.y, bhi.y) - fminf(alo.y, blo.y);
  const float ez = fmaxf(ahi.z, bhi.z) - fminf(alo.z, blo.z);
  return ex * ey + ey * ez + ez * ex;
}

__global__ void k_ploc_init(int n, int idxBits, const unsigned long long* keys, const float4* primLo,
                            const float4* primHi, int* code, float4* lo, float4* hi, int* cnt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint32_t g = uint32_t(keys[i] & ((1ull << idxBits) - 1ull));
  code[i] = ~i;
  lo[i] = primLo[g];
  hi[i] = primHi[g];
  cnt[i] = 1;
}

__global__ void __launch_bounds__(kPlocBlock) k_ploc_nn(const int* ncIn, const float4* lo, const float4* hi, int* nn) {
  __shared__ float4 sLo[kPlocBlock + 2 * kPlocRadius], sHi[kPlocBlock + 2 * kPlocRadius];
  const int nc = *ncIn;
  const int b0 = blockIdx.x * kPlocBlock - kPlocRadius;
  for (int k = threadIdx.x; k < kPlocBlock + 2 * kPlocRadius; k += kPlocBlock) {
    const int j = b0 + k;
    if (j >= 0 && j < nc) {
      sLo[k] = lo[j];
      sHi[k] = hi[j];
    }
  }
  __syncthreads();
  const int i = blockIdx.x * kPlocBlock + threadIdx.x;
  if (i >= nc) return;
  const int si = threadIdx.x + kPlocRadius;
  const float4 ilo = sLo[si], ihi = sHi[si];
  float best = __int_as_float(0x7F800000);
  int bestJ = -1;
  const int j0 = max(0, i - kPlocRadius), j1 = min(nc - 1, i + kPlocRadius);
  for (int j = j0; j <= j1; ++j) {
    if (j == i) continue;
    const float d = unionArea(ilo, ihi, sLo[j - b0], sHi[j - b0]);
    if (d < best) {
      best = d;
      bestJ = j;
    }
  }
  nn[i] = bestJ;
}

__device__ __forceinline__ void writeBinNode(float4* nodes, int node, int c0, float4 lo0, float4 hi0, int c1,
                                             float4 lo1, float4 hi1) {
  float4* nd = nodes + kNodeF4 * node;
  nd[0] = make_float4(lo0.x, hi0.x, lo0.y, hi0.y);
  nd[1] = make_float4(lo1.x, hi1.x, lo1.y, hi1.y);
  nd[2] = make_float4(lo0.z, hi0.z, lo1.z, hi1.z);
  nd[3] = make_float4(__int_as_float(c0), __int_as_float(c1), 0.0f, 0.0f);
}

__global__ void k_ploc_merge(const int* ncIn, int ncCap, const int* nn, int* code, float4* lo, float4* hi, int* cnt,
                             float4* nodes, int2* ranges, int* nodeCounter, int* valid, int* leafParent,
                             int* nodeParent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncCap) return;
  if (i >= *ncIn) {  // past the clusters of this round: nothing to keep
    valid[i] = 0;
    return;
  }
  const int j = nn[i];
  const bool mutual = j >= 0 && nn[j] == i;
  if (mutual && i < j) {
    const int node = atomicAdd(nodeCounter, 1);
    const float4 l0 = lo[i], h0 = hi[i], l1 = lo[j], h1 = hi[j];
    writeBinNode(nodes, node, code[i], l0, h0, code[j], l1, h1);
    const int c0 = code[i], c1 = code[j];
    if (c0 < 0) leafParent[~c0] = node << 1;
    else nodeParent[c0] = node << 1;
    if (c1 < 0) leafParent[~c1] = (node << 1) | 1;
    else nodeParent[c1] = (node << 1) | 1;
    const int c = cnt[i] + cnt[j];
    ranges[node] = make_int2(0, c - 1);  // only the primitive count is read
    code[i] = node;
    lo[i] = make_float4(fminf(l0.x, l1.x), fminf(l0.y, l1.y), fminf(l0.z, l1.z), 0.0f);
    hi[i] = make_float4(fmaxf(h0.x, h1.x), fmaxf(h0.y, h1.y), fmaxf(h0.z, h1.z), 0.0f);
    cnt[i] = c;
    valid[i] = 1;
  } else {
    valid[i] = (mutual && i > j) ? 0 : 1;
  }
}

__global__ void k_ploc_compact(int ncCap, const int* valid, const int* pos, const int* code, const float4* lo,
                               const float4* hi, const int* cnt, int* code2, float4* lo2, float4* hi2, int* cnt2,
                               int* newCount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncCap) return;
  if (i == ncCap - 1) *newCount = pos[i] + valid[i];
  if (!valid[i]) return;
  const int o = pos[i];
  code2[o] = code[i];
  lo2[o] = lo[i];
  hi2[o] = hi[i];
  cnt2[o] = cnt[i];
}

__device__ __forceinline__ void binChild(const float4* nodes, int node, int side, int& code, float3& lo, float3& hi) {
  const float4* nd = nodes + kNodeF4 * node;
  const float4 a = nd[side], z = nd[2], c = nd[3];
  lo = make_float3(a.x, a.z, side == 0 ? z.x : z.z);
  hi = make_float3(a.y, a.w, side == 0 ? z.y : z.w);
  code = __float_as_int(side == 0 ? c.x : c.y);
}

__device__ __forceinline__ float halfArea(float3 lo, float3 hi) {
  const float ex = hi.x - lo.x, ey = hi.y - lo.y, ez = hi.z - lo.z;
  return ex * ey + ey * ez + ez * ex;
}

// Power-of-two scale s >= ext/255 (with slack) as its biased exponent.
__device__ __forceinline__ uint32_t scaleExp(float ext) {
  float x = ext * (1.0f / 255.0f) * (1.0f + 0x1.0p-20f);
  if (!(x > 0x1.0p-126f)) x = 0x1.0p-126f;
  const uint32_t bits = __float_as_uint(x);
  uint32_t ex = bits >> 23;
  if (bits & 0x7FFFFFu) ++ex;
  return ex;
}

__device__ __forceinline__ void quantize(float lo, float hi, float p, float sc, uint32_t& qlo, uint32_t& qhi) {
  int a = int(floorf((lo - p) / sc)), b = int(ceilf((hi - p) / sc));
  a = max(0, min(255, a));
  b = max(0, min(255, b));
  while (a > 0 && fmaf(float(a), sc, p) > lo) --a;
  while (b < 255 && fmaf(float(b), sc, p) < hi) ++b;
  qlo = uint32_t(a);
  qhi = uint32_t(b);
}

// SAH-optimal collapse of the binary tree into 8-wide nodes (the dynamic
// programme of Ylitie, Karras and Laine, "Efficient Incoherent Ray Traversal
// on GPUs Through Compressed Wide BVHs", HPG 2017).  For binary node n and
// j = 1..7 child slots, C(n, j) is the least cost of covering n's subtree
// with at most j children of a wide node: C(n, 1) = min(leaf cost, internal
// cost), C(n, j) = min(best split of j slots over n's two children,
// C(n, j - 1)).  Leaf cost = area x the primitives' test costs (leaves hold
// at most kWideLeafMax primitives), internal cost = area x node cost + the
// best split of 8 slots.  Costs are per unit of node-visit work; primitive
// test weights by kind reflect the intersectors' instruction counts.
constexpr float kSahNode = 1.0f;
__device__ __forceinline__ float sahPrimCost(int kind) {
  return kind == kSphere ? 0.12f : kind == kMesh ? 0.16f : kind == kCone ? 0.25f : 0.35f;
}
constexpr float kSahInf = 3.0e38f;
constexpr int kSahStride = 8;  // per node: C(n,1..7) and the sum of primitive costs

// Cost row of a child: an internal node's stored row, or a single primitive.
__device__ __forceinline__ void sahChildRow(const float* cost, int code, float3 lo, float3 hi,
                                            const uint32_t* leafRef, float* row, float& sumC, int& cnt,
                                            const int2* brange, float primScale) {
  if (code < 0) {
    const float c = primScale * sahPrimCost(refKind(leafRef[~code]));
    const float a = halfArea(lo, hi) * c;
    for (int j = 1; j <= 7; ++j) row[j] = a;
    sumC = c;
    cnt = 1;
  } else {
    const float* r = cost + kSahStride * code;
    for (int j = 1; j <= 7; ++j) row[j] = __ldcg(r + j - 1);
    sumC = __ldcg(r + 7);
    cnt = brange[code].y - brange[code].x + 1;
  }
}

// Bottom-up: one thread per leaf walks to the root; the second child to
// arrive at a node computes the node's row (the refit pattern).
__global__ void k_sah_costs(int n, const float4* nodes, const int2* brange, const uint32_t* leafRef,
                            const int* leafParent, const int* nodeParent, int* counters, float* cost,
                            uint8_t* dec, float primScale) {
  const int sIdx = blockIdx.x * blockDim.x + threadIdx.x;
  if (sIdx >= n) return;
  int pinfo = leafParent[sIdx];
  while (pinfo >= 0) {
    const int p = pinfo >> 1;
    __threadfence();
    if (atomicAdd(&counters[p], 1) == 0) return;
    __threadfence();
    int c0, c1;
    float3 lo0, hi0, lo1, hi1;
    binChild(nodes, p, 0, c0, lo0, hi0);
    binChild(nodes, p, 1, c1, lo1, hi1);
    float r0[8], r1[8], s0, s1;
    int n0, n1;
    sahChildRow(cost, c0, lo0, hi0, leafRef, r0, s0, n0, brange, primScale);
    sahChildRow(cost, c1, lo1, hi1, leafRef, r1, s1, n1, brange, primScale);
    const float3 lo = make_float3(fminf(lo0.x, lo1.x), fminf(lo0.y, lo1.y), fminf(lo0.z, lo1.z));
    const float3 hi = make_float3(fmaxf(hi0.x, hi1.x), fmaxf(hi0.y, hi1.y), fmaxf(hi0.z, hi1.z));
    const float A = halfArea(lo, hi);
    // best split of j slots over the two children, j = 2..8
    float dist[9];
    uint8_t split[9];
    for (int j = 2; j <= 8; ++j) {
      float best = kSahInf;
      int bk = 1;
      for (int k = 1; k < j; ++k) {
        if (k > 7 || j - k > 7) continue;
        const float c = r0[k] + r1[j - k];
        if (c < best) {
          best = c;
          bk = k;
        }
      }
      dist[j] = best;
      split[j] = uint8_t(bk);
    }
    const int cnt = n0 + n1;
    const float sumC = s0 + s1;
    const float cLeaf = cnt <= kWideLeafMax ? A * sumC : kSahInf;
    const float cInt = A * kSahNode + dist[8];
    float* out = cost + kSahStride * p;
    uint8_t* d = dec + 8 * p;
    float cj = fminf(cLeaf, cInt);
    out[0] = cj;
    d[0] = cLeaf <= cInt ? 1 : 0;  // j = 1: 1 leaf, 0 wide node
    for (int j = 2; j <= 7; ++j) {
      if (dist[j] < cj) {
        cj = dist[j];
        d[j - 1] = split[j];       // split j slots: k to child 0
      } else {
        d[j - 1] = 0;              // no better than j - 1 slots
      }
      out[j - 1] = cj;
    }
    out[7] = sumC;
    d[7] = split[8];               // the split of a wide node's 8 slots
    pinfo = nodeParent[p];
  }
}

// Primitive slots of a binary subtree with at most kWideLeafMax primitives.
__device__ __forceinline__ int subtreePrims(const float4* nodes, int code, int* out) {
  int stack[kWideLeafMax + 1], sp = 0, nOut = 0;
  stack[sp++] = code;
  while (sp > 0 && nOut < kWideLeafMax) {
    const int c = stack[--sp];
    if (c < 0) {
      out[nOut++] = ~c;
    } else {
      const float4 cc = nodes[kNodeF4 * c + 3];
      if (sp + 2 > kWideLeafMax + 1) break;
      stack[sp++] = __float_as_int(cc.y);
      stack[sp++] = __float_as_int(cc.x);
    }
  }
  return nOut;
}

// Top-down collapse with the DP's decisions: a wide node made from binary
// node n takes the children the 8-slot split of n selects; a child is a
// single primitive, a leaf of up to kWideLeafMax primitives, or a binary node
// that becomes a wide node of the next level.
__global__ void k_collapse_sah(const float4* bnodes, const uint8_t* dec, const int* workCode, const int* workWide,
                               int workCount, int* nextCode, int* nextWide, int* cursors, float4* wnodes,
                               const uint32_t* srcRef, const float4* srcGeo, uint32_t* dstRef, float4* dstGeo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= workCount) return;
  const int code = workCode[i];
  const int w = workWide[i];
  int ec[8], et[8];  // child code, type: 0 leaf, 1 wide node
  float3 elo[8], ehi[8];
  int en = 0;
  // stack of (binary parent, side, slots)
  int sp = 0;
  int stP[16], stS[16], stJ[16];
  const int k8 = dec[8 * code + 7];
  stP[sp] = code; stS[sp] = 1; stJ[sp] = 8 - k8; ++sp;
  stP[sp] = code; stS[sp] = 0; stJ[sp] = k8; ++sp;
  while (sp > 0 && en < 8) {
    --sp;
    const int par = stP[sp], side = stS[sp], j = stJ[sp];
    int c;
    float3 lo, hi;
    binChild(bnodes, par, side, c, lo, hi);
    if (c < 0) {
      ec[en] = c; et[en] = 0; elo[en] = lo; ehi[en] = hi; ++en;
      continue;
    }
    int jj = j;
    while (jj > 1 && dec[8 * c + jj - 1] == 0) --jj;
    if (jj <= 1) {
      ec[en] = c; et[en] = dec[8 * c] ? 0 : 1; elo[en] = lo; ehi[en] = hi; ++en;
      continue;
    }
    const int k = dec[8 * c + jj - 1];
    if (sp + 2 > 16) break;  // cannot happen: at most 8 open entries
    stP[sp] = c; stS[sp] = 1; stJ[sp] = jj - k; ++sp;
    stP[sp] = c; stS[sp] = 0; stJ[sp] = k; ++sp;
  }
  int nInt = 0, nLeaf = 0;
  int prims[8][kWideLeafMax], pc[8];
  for (int k = 0; k < en; ++k) {
    if (et[k] == 1) {
      ++nInt;
      pc[k] = 0;
    } else {
      pc[k] = subtreePrims(bnodes, ec[k], prims[k]);
      nLeaf += pc[k];
    }
  }
  const int childBase = nInt ? atomicAdd(&cursors[0], nInt) : 0;
  const int primBase = nLeaf ? atomicAdd(&cursors[1], nLeaf) : 0;
  const int pushBase = nInt ? atomicAdd(&cursors[2], nInt) : 0;
  float3 p = elo[0], hmax = ehi[0];
  for (int k = 1; k < en; ++k) {
    p = make_float3(fminf(p.x, elo[k].x), fminf(p.y, elo[k].y), fminf(p.z, elo[k].z));
    hmax = make_float3(fmaxf(hmax.x, ehi[k].x), fmaxf(hmax.y, ehi[k].y), fmaxf(hmax.z, ehi[k].z));
  }
  const uint32_t exX = scaleExp(hmax.x - p.x), exY = scaleExp(hmax.y - p.y), exZ = scaleExp(hmax.z - p.z);
  const float scX = __uint_as_float(exX << 23), scY = __uint_as_float(exY << 23), scZ = __uint_as_float(exZ << 23);
  uint32_t meta[2] = {0u, 0u}, qlx[2] = {0u, 0u}, qly[2] = {0u, 0u}, qlz[2] = {0u, 0u};
  uint32_t qhx[2] = {0u, 0u}, qhy[2] = {0u, 0u}, qhz[2] = {0u, 0u};
  int order[8];
  {
    int o = 0;
    for (int k = 0; k < en; ++k)
      if (et[k] == 1) order[o++] = k;
    for (int k = 0; k < en; ++k)
      if (et[k] == 0) order[o++] = k;
  }
  int kInt = 0, off = 0;
  for (int slot = 0; slot < en; ++slot) {
    const int k = order[slot];
    uint32_t a, b;
    const int wd = slot >> 2, sh = (slot & 3) * 8;
    quantize(elo[k].x, ehi[k].x, p.x, scX, a, b);
    qlx[wd] |= a << sh;
    qhx[wd] |= b << sh;
    quantize(elo[k].y, ehi[k].y, p.y, scY, a, b);
    qly[wd] |= a << sh;
    qhy[wd] |= b << sh;
    quantize(elo[k].z, ehi[k].z, p.z, scZ, a, b);
    qlz[wd] |= a << sh;
    qhz[wd] |= b << sh;
    uint32_t m;
    if (et[k] == 1) {
      m = 0x80u | uint32_t(kInt);
      nextCode[pushBase + kInt] = ec[k];
      nextWide[pushBase + kInt] = childBase + kInt;
      ++kInt;
    } else {
      const int cnt = pc[k];
      m = (uint32_t(cnt) << 5) | uint32_t(off);
      for (int q = 0; q < cnt; ++q) {
        const int d = primBase + off + q, sidx = prims[k][q];
        dstRef[d] = srcRef[sidx];
        for (int f = 0; f < kLeafF4; ++f) dstGeo[kLeafF4 * d + f] = srcGeo[kLeafF4 * sidx + f];
      }
      off += cnt;
    }
    meta[wd] |= m << sh;
  }
  for (int k = en; k < 8; ++k) {
    const int wd = k >> 2, sh = (k & 3) * 8;
    qlx[wd] |= 255u << sh;
    qly[wd] |= 255u << sh;
    qlz[wd] |= 255u << sh;
  }
  float4* o = wnodes + kWideF4 * w;
  o[0] = make_float4(p.x, p.y, p.z,
                     __uint_as_float(exX | (exY << 8) | (exZ << 16) | (uint32_t(nInt) << 24) | (uint32_t(en) << 28)));
  o[1] = make_float4(__int_as_float(childBase), __int_as_float(primBase), __uint_as_float(meta[0]),
                     __uint_as_float(meta[1]));
  o[2] = make_float4(__uint_as_float(qlx[0]), __uint_as_float(qlx[1]), __uint_as_float(qly[0]),
                     __uint_as_float(qly[1]));
  o[3] = make_float4(__uint_as_float(qlz[0]), __uint_as_float(qlz[1]), __uint_as_float(qhx[0]),
                     __uint_as_float(qhx[1]));
  o[4] = make_float4(__uint_as_float(qhy[0]), __uint_as_float(qhy[1]), __uint_as_float(qhz[0]),
                     __uint_as_float(qhz[1]));
}

// Top-down collapse of the binary LBVH into 8-wide nodes, one level of wide
// nodes per launch.  A wide node starts from its binary node's two children
// and repeatedly opens the child with the largest surface area until it has
// 8 children or none is worth opening (subtrees of <= 3 primitives become
// leaves: their primitives are a contiguous run of Morton-sorted slots).
// Leaf primitives of a node are copied into one contiguous block so a wide
// node addresses them with an 8-bit offset.
__global__ void k_collapse(const float4* bnodes, const int2* brange, const float4* rootLo, const float4* rootHi,
                           const int* workCode, const int* workWide, int workCount, int leafMax, int* nextCode,
                           int* nextWide,
                           int* cursors, float4* wnodes, const uint32_t* srcRef, const float4* srcGeo,
                           uint32_t* dstRef, float4* dstGeo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= workCount) return;
  const int code = workCode[i];
  const int w = workWide[i];
  int ec[8];
  float3 elo[8], ehi[8];
  int en;
  if (code < 0) {  // single-primitive scene
    ec[0] = code;
    elo[0] = make_float3(rootLo->x, rootLo->y, rootLo->z);
    ehi[0] = make_float3(rootHi->x, rootHi->y, rootHi->z);
    en = 1;
  } else {
    binChild(bnodes, code, 0, ec[0], elo[0], ehi[0]);
    binChild(bnodes, code, 1, ec[1], elo[1], ehi[1]);
    en = 2;
  }
  auto countOf = [&](int c) { return c < 0 ? 1 : brange[c].y - brange[c].x + 1; };
  while (en < 8) {
    int best = -1;
    float bestA = -1.0f;
    for (int k = 0; k < en; ++k) {
      if (ec[k] >= 0 && countOf(ec[k]) > leafMax) {
        const float a = halfArea(elo[k], ehi[k]);
        if (a > bestA) {
          bestA = a;
          best = k;
        }
      }
    }
    if (best < 0) break;
    const int c = ec[best];
    binChild(bnodes, c, 0, ec[best], elo[best], ehi[best]);
    binChild(bnodes, c, 1, ec[en], elo[en], ehi[en]);
    ++en;
  }
  int nInt = 0, nLeaf = 0;
  for (int k = 0; k < en; ++k) {
    if (ec[k] >= 0 && countOf(ec[k]) > leafMax) ++nInt;
    else nLeaf += countOf(ec[k]);
  }
  const int childBase = nInt ? atomicAdd(&cursors[0], nInt) : 0;
  const int primBase = nLeaf ? atomicAdd(&cursors[1], nLeaf) : 0;
  const int pushBase = nInt ? atomicAdd(&cursors[2], nInt) : 0;
  float3 p = elo[0], hmax = ehi[0];
  for (int k = 1; k < en; ++k) {
    p = make_float3(fminf(p.x, elo[k].x), fminf(p.y, elo[k].y), fminf(p.z, elo[k].z));
    hmax = make_float3(fmaxf(hmax.x, ehi[k].x), fmaxf(hmax.y, ehi[k].y), fmaxf(hmax.z, ehi[k].z));
  }
  const uint32_t exX = scaleExp(hmax.x - p.x), exY = scaleExp(hmax.y - p.y), exZ = scaleExp(hmax.z - p.z);
  const float scX = __uint_as_float(exX << 23), scY = __uint_as_float(exY << 23), scZ = __uint_as_float(exZ << 23);
  uint32_t meta[2] = {0u, 0u}, qlx[2] = {0u, 0u}, qly[2] = {0u, 0u}, qlz[2] = {0u, 0u};
  uint32_t qhx[2] = {0u, 0u}, qhy[2] = {0u, 0u}, qhz[2] = {0u, 0u};
  // slot order: internal children first (slot k -> node childBase + k), then leaves
  int order[8];
  {
    int o = 0;
    for (int k = 0; k < en; ++k)
      if (ec[k] >= 0 && countOf(ec[k]) > leafMax) order[o++] = k;
    for (int k = 0; k < en; ++k)
      if (!(ec[k] >= 0 && countOf(ec[k]) > leafMax)) order[o++] = k;
  }
  int kInt = 0, off = 0;
  for (int slot = 0; slot < en; ++slot) {
    const int k = order[slot];
    uint32_t a, b;
    const int wd = slot >> 2, sh = (slot & 3) * 8;
    quantize(elo[k].x, ehi[k].x, p.x, scX, a, b);
    qlx[wd] |= a << sh;
    qhx[wd] |= b << sh;
    quantize(elo[k].y, ehi[k].y, p.y, scY, a, b);
    qly[wd] |= a << sh;
    qhy[wd] |= b << sh;
    quantize(elo[k].z, ehi[k].z, p.z, scZ, a, b);
    qlz[wd] |= a << sh;
    qhz[wd] |= b << sh;
    uint32_t m;
    if (ec[k] >= 0 && countOf(ec[k]) > leafMax) {
      m = 0x80u | uint32_t(kInt);
      nextCode[pushBase + kInt] = ec[k];
      nextWide[pushBase + kInt] = childBase + kInt;
      ++kInt;
    } else {
      const int cnt = countOf(ec[k]);
      const int first = ec[k] < 0 ? ~ec[k] : brange[ec[k]].x;
      m = (uint32_t(cnt) << 5) | uint32_t(off);
      for (int q = 0; q < cnt; ++q) {
        const int d = primBase + off + q, sidx = first + q;
        dstRef[d] = srcRef[sidx];
        for (int f = 0; f < kLeafF4; ++f) dstGeo[kLeafF4 * d + f] = srcGeo[kLeafF4 * sidx + f];
      }
      off += cnt;
    }
    meta[wd] |= m << sh;
  }
  // empty slots: qlo = 255 > qhi = 0 and meta 0 (never tested)
  for (int k = en; k < 8; ++k) {
    const int wd = k >> 2, sh = (k & 3) * 8;
    qlx[wd] |= 255u << sh;
    qly[wd] |= 255u << sh;
    qlz[wd] |= 255u << sh;
  }
  float4* o = wnodes + kWideF4 * w;
  o[0] = make_float4(p.x, p.y, p.z,
                     __uint_as_float(exX | (exY << 8) | (exZ << 16) | (uint32_t(nInt) << 24) | (uint32_t(en) << 28)));
  o[1] = make_float4(__int_as_float(childBase), __int_as_float(primBase), __uint_as_float(meta[0]),
                     __uint_as_float(meta[1]));
  o[2] = make_float4(__uint_as_float(qlx[0]), __uint_as_float(qlx[1]), __uint_as_float(qly[0]),
                     __uint_as_float(qly[1]));
  o[3] = make_float4(__uint_as_float(qlz[0]), __uint_as_float(qlz[1]), __uint_as_float(qhx[0]),
                     __uint_as_float(qhx[1]));
  o[4] = make_float4(__uint_as_float(qhy[0]), __uint_as_float(qhy[1]), __uint_as_float(qhz[0]),
                     __uint_as_float(qhz[1]));
}

template <class T>
ubr_status upload(Context* c, Scene* sc, const std::vector<T>& v, const T** out) {
  *out = nullptr;
  if (v.empty()) return UBR_OK;
  sc->bufs.emplace_back();
  DevBuf& b = sc->bufs.back();
  ubr_status st = devAlloc(c, b, v.size() * sizeof(T));
  if (st != UBR_OK) return st;
  UBR_CUDA(c, cudaMemcpyAsync(b.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
  *out = static_cast<const T*>(b.ptr);
  return UBR_OK;
}

ubr_status allocOwned(Context* c, Scene* sc, size_t bytes, void** out) {
  sc->bufs.emplace_back();
  DevBuf& b = sc->bufs.back();
  ubr_status st = devAlloc(c, b, bytes);
  *out = b.ptr;
  return st;
}

int bitsFor(uint32_t n) {
  int b = 1;
  while ((1ull << b) < n) ++b;
  return b;
}

}  // namespace

ubr_status buildScene(Context* c, const ubr_scene_desc& d, Scene** out) {
  const auto t0 = std::chrono::steady_clock::now();
  ubr_status st = validate(c, d);
  if (st != UBR_OK) return st;
  // host staging of the flattened tables, reused by this thread's next build
  // (a copy from pageable memory has left the buffer when cudaMemcpyAsync
  // returns); released after a build that needed more than 64 MB
  static thread_local HostScene staging;
  HostScene& hs = staging;
  hs.reset();
  struct Release {
    HostScene& h;
    ~Release() {
      if (h.capacityBytes() > (64u << 20)) h = HostScene();
    }
  } release{hs};
  st = flatten(c, d, hs);
  if (st != UBR_OK) return st;
  const auto tFlat = std::chrono::steady_clock::now();
  Scene* sc = new Scene();
  sc->ctx = c;
  auto fail = [&](ubr_status s) {
    for (DevBuf& b : sc->bufs) devFree(c, b);
    delete sc;
    return s;
  };
  DScene& v = sc->view;
  const uint32_t nTri = uint32_t(hs.idx.size() / 3), nSph = uint32_t(hs.sph.size()),
                 nRc = uint32_t(hs.rcIdx.size()), nCc = uint32_t(hs.ccIdx.size());
  const uint32_t n = nTri + nSph + nRc + nCc;
  sc->primCount[kMesh] = nTri;
  sc->primCount[kSphere] = nSph;
  sc->primCount[kRound] = nRc;
  sc->primCount[kCone] = nCc;
  for (int k = 0; k < 4; ++k) v.geomID[k] = hs.geomID[k];
  v.primCount = n;
  sc->opaque = hs.opaque;
  sc->principled = hs.principled;
  sc->aoReceivers = nTri > 0;
  for (int k = 1; k < 4 && !sc->aoReceivers; ++k)
    for (uint8_t fe : hs.fromEdge[k])
      if (!fe) {
        sc->aoReceivers = true;
        break;
      }
  v.baseTri = hs.baseTri;
  v.meshMat = hs.meshMat;
  cudaEventRecord(c->ev[0], c->stream);
  const float* dpos = nullptr;
  const float4* dsph = nullptr;
  const float4* drcV = nullptr;
  const uint32_t* drcIdx = nullptr;
  const uint8_t* drcFl = nullptr;
  const float4* dccV = nullptr;
  const uint32_t* dccIdx = nullptr;
  if ((st = upload(c, sc, hs.pos, &dpos)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.nrm, &v.meshNrm)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.col, &v.meshCol)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.idx, &v.meshIdx)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.triMat, &v.meshTriMat)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.triMatId, &v.meshTriMatId)) != UBR_OK) return fail(st);
  // edge G-buffer material blocks (scene_build.cpp:151-155, 104-123; curve_build.cpp:179)
  v.meshMatCount = uint32_t(d.mesh_material_count);
  v.baseSpheres = uint32_t(d.sphere_count);
  v.roundCount = uint32_t(hs.rcIdx.size());
  if ((st = upload(c, sc, hs.sph, &dsph)) != UBR_OK) return fail(st);
  v.sph = dsph;
  v.baseSph = hs.baseSph;
  if ((st = upload(c, sc, hs.rcV, &drcV)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.rcIdx, &drcIdx)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.rcFlags, &drcFl)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.rcClip, &v.rcClip)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.ccV, &dccV)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.ccIdx, &dccIdx)) != UBR_OK) return fail(st);
  if ((st = upload(c, sc, hs.mats, &v.mats)) != UBR_OK) return fail(st);
  {
    // pt2: reflection ownership flags (hit_shader.hpp:243-270) and the
    // emissive primitives sampled as lights
    for (const ubr_material& m : hs.mats) {
      if (m.model == 1u) {
        if (m.pbr_metallic > 1e-4f || m.pbr_specular > 1e-4f) {
          sc->reflective = true;
          sc->glossy = sc->glossy || m.pbr_roughness * m.pbr_roughness >= 0.015f;
        }
        if (m.pbr_anisotropy != 0.0f) sc->anisoPrincipled = true;
      } else if (m.reflection > 0.0f) {
        sc->reflective = true;
        sc->glossy = sc->glossy || m.specular > 0.0f;
      }
    }
    std::vector<f3> offs;
    for (uint64_t i = 0; i < d.instance_count; ++i) offs.push_back(ld3(d.instance_offsets, i));
    if (offs.empty()) offs.push_back(f3{0, 0, 0});
    HostEmit he;
    buildEmitters(d, offs, he);
    EmitD& em = sc->emit;
    em.n = uint32_t(he.cdf.size());
    em.triCount = he.triCount;
    em.nTriIndex = uint32_t(he.triIndex.size());
    em.nSphereIndex = uint32_t(he.sphereIndex.size());
    em.nCylIndex = uint32_t(he.cylIndex.size());
    if (em.n > 0) {
      if ((st = upload(c, sc, he.cdf, &em.cdf)) != UBR_OK) return fail(st);
      if ((st = upload(c, sc, he.pdf, &em.pdfChoose)) != UBR_OK) return fail(st);
      if ((st = upload(c, sc, he.rec, &em.rec)) != UBR_OK) return fail(st);
      if ((st = upload(c, sc, he.triIndex, &em.triIndex)) != UBR_OK) return fail(st);
      if ((st = upload(c, sc, he.sphereIndex, &em.sphereIndex)) != UBR_OK) return fail(st);
      if ((st = upload(c, sc, he.cylIndex, &em.cylIndex)) != UBR_OK) return fail(st);
    }
  }
  for (int k = 1; k < 4; ++k) {
    if ((st = upload(c, sc, hs.color[k], &v.primColor[k])) != UBR_OK) return fail(st);
    if ((st = upload(c, sc, hs.mat[k], &v.primMat[k])) != UBR_OK) return fail(st);
    if ((st = upload(c, sc, hs.fromEdge[k], &v.primFromEdge[k])) != UBR_OK) return fail(st);
    if ((st = upload(c, sc, hs.opacity1[k], &v.primOpacity1[k])) != UBR_OK) return fail(st);
    if ((st = upload(c, sc, hs.group[k], &v.primGroup[k])) != UBR_OK) return fail(st);
    if ((st = upload(c, sc, hs.axis[k], &v.primAxis[k])) != UBR_OK) return fail(st);
  }
  if ((st = upload(c, sc, hs.triGroup, &v.meshTriGroup)) != UBR_OK) return fail(st);
  const auto tUp = std::chrono::steady_clock::now();
  if (n > 0) {
    BuildIn in{dpos, v.meshIdx, dsph, drcV, drcIdx, drcFl, dccV, dccIdx, nTri, nSph, nRc, nCc};
    void *pLo, *pHi, *pKeys, *pKeys2, *pCb, *pLeafP, *pNodeP, *pCnt, *pNodes, *pRef, *pGeo;
    void *pWide, *pRef2, *pGeo2, *pRange, *pWc[2], *pWw[2], *pCur;
    const size_t nn = n > 1 ? n - 1 : 1;
    // the scene keeps the 8-wide nodes and the leaf records in wide order;
    // the binary tree and the Morton-ordered leaves are build temporaries
    if ((st = allocOwned(c, sc, sizeof(float4) * kWideF4 * nn, &pWide)) != UBR_OK) return fail(st);
    if ((st = allocOwned(c, sc, sizeof(uint32_t) * n, &pRef2)) != UBR_OK) return fail(st);
    if ((st = allocOwned(c, sc, sizeof(float4) * kLeafF4 * n, &pGeo2)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 50, sizeof(float4) * kNodeF4 * nn, &pNodes)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 51, sizeof(uint32_t) * n, &pRef)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 52, sizeof(float4) * kLeafF4 * n, &pGeo)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 53, sizeof(int2) * nn, &pRange)) != UBR_OK) return fail(st);
    for (int k = 0; k < 2; ++k) {
      if ((st = scratchGet(c, 54 + 2 * k, sizeof(int) * nn, &pWc[k])) != UBR_OK) return fail(st);
      if ((st = scratchGet(c, 55 + 2 * k, sizeof(int) * nn, &pWw[k])) != UBR_OK) return fail(st);
    }
    if ((st = scratchGet(c, 58, 64, &pCur)) != UBR_OK) return fail(st);
    // build temporaries live in context scratch slots 0..7
    if ((st = scratchGet(c, 0, sizeof(float4) * n, &pLo)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 1, sizeof(float4) * n, &pHi)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 2, sizeof(unsigned long long) * n, &pKeys)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 3, sizeof(unsigned long long) * n, &pKeys2)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 4, 64, &pCb)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 5, sizeof(int) * n, &pLeafP)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 6, sizeof(int) * nn, &pNodeP)) != UBR_OK) return fail(st);
    if ((st = scratchGet(c, 7, sizeof(int) * nn, &pCnt)) != UBR_OK) return fail(st);
    const int initB[6] = {0x7FFFFFFF, 0x7FFFFFFF, 0x7FFFFFFF, int(0x80000000), int(0x80000000), int(0x80000000)};
    UBR_CUDA(c, cudaMemcpyAsync(pCb, initB, sizeof(initB), cudaMemcpyHostToDevice, c->stream));
    UBR_CUDA(c, cudaMemsetAsync(pCnt, 0, sizeof(int) * nn, c->stream));
    // parents start at -1 so a refit walk always terminates
    UBR_CUDA(c, cudaMemsetAsync(pLeafP, 0xFF, sizeof(int) * n, c->stream));
    UBR_CUDA(c, cudaMemsetAsync(pNodeP, 0xFF, sizeof(int) * nn, c->stream));
    UBR_CUDA(c, cudaMemsetAsync(pNodes, 0, sizeof(float4) * kNodeF4 * nn, c->stream));
    const int TB = 256;
    const int grid = int((n + TB - 1) / TB);
    k_prim_bounds<<<grid, TB, 0, c->stream>>>(in, n, (float4*)pLo, (float4*)pHi, (int*)pCb);
    const int idxBits = bitsFor(n);
    k_morton<<<grid, TB, 0, c->stream>>>(n, idxBits, (const float4*)pLo, (const float4*)pHi, (const int*)pCb,
                                         (unsigned long long*)pKeys);
    size_t tmpBytes = 0;
    cub::DeviceRadixSort::SortKeys(nullptr, tmpBytes, (unsigned long long*)pKeys, (unsigned long long*)pKeys2,
                                   int(n), 0, 30 + idxBits, c->stream);
    void* pTmp;
    if ((st = scratchGet(c, 8, tmpBytes, &pTmp)) != UBR_OK) return fail(st);
    UBR_CUDA(c, cub::DeviceRadixSort::SortKeys(pTmp, tmpBytes, (unsigned long long*)pKeys,
                                               (unsigned long long*)pKeys2, int(n), 0, 30 + idxBits, c->stream));
    const bool ploc = n > 1 && c->builder == 2 && (c->leafMax == 1 || c->collapse == 2);
    if (n > 1 && !ploc)
      k_hierarchy<<<int((n - 1 + TB - 1) / TB), TB, 0, c->stream>>>(int(n), (const unsigned long long*)pKeys2,
                                                                   (float4*)pNodes, (int*)pLeafP, (int*)pNodeP,
                                                                   (int2*)pRange);
    // leaf records in Morton order (+ the radix tree's bottom-up refit)
    k_refit<<<grid, TB, 0, c->stream>>>(in, int(n), idxBits, (const unsigned long long*)pKeys2,
                                        (const float4*)pLo, (const float4*)pHi, v.rcClip, (float4*)pNodes,
                                        (const int*)pLeafP, (const int*)pNodeP, (int*)pCnt, (uint32_t*)pRef,
                                        (float4*)pGeo, ploc ? 0 : 1);
    UBR_CUDA(c, cudaGetLastError());
    int rootCodeDev = -1;  // root node of the PLOC tree (the radix tree's root is node 0)
    if (ploc) {
      void *pCode[2], *pCLo[2], *pCHi[2], *pCCnt[2], *pNn, *pValid, *pPos, *pPc;
      for (int k = 0; k < 2; ++k) {
        if ((st = scratchGet(c, 40 + 4 * k, sizeof(int) * n, &pCode[k])) != UBR_OK) return fail(st);
        if ((st = scratchGet(c, 41 + 4 * k, sizeof(float4) * n, &pCLo[k])) != UBR_OK) return fail(st);
        if ((st = scratchGet(c, 42 + 4 * k, sizeof(float4) * n, &pCHi[k])) != UBR_OK) return fail(st);
        if ((st = scratchGet(c, 43 + 4 * k, sizeof(int) * n, &pCCnt[k])) != UBR_OK) return fail(st);
      }
      if ((st = scratchGet(c, 48, sizeof(int) * n, &pNn)) != UBR_OK) return fail(st);
      if ((st = scratchGet(c, 49, sizeof(int) * n, &pValid)) != UBR_OK) return fail(st);
      if ((st = scratchGet(c, 59, sizeof(int) * n, &pPos)) != UBR_OK) return fail(st);
      if ((st = scratchGet(c, 9, 64, &pPc)) != UBR_OK) return fail(st);
      size_t scanBytes = 0;
      cub::DeviceScan::ExclusiveSum(nullptr, scanBytes, (const int*)pValid, (int*)pPos, int(n), c->stream);
      void* pScan;
      if ((st = scratchGet(c, 10, scanBytes, &pScan)) != UBR_OK) return fail(st);
      UBR_CUDA(c, cudaMemsetAsync(pPc, 0, 64, c->stream));
      k_ploc_init<<<grid, TB, 0, c->stream>>>(int(n), idxBits, (const unsigned long long*)pKeys2,
                                              (const float4*)pLo, (const float4*)pHi, (int*)pCode[0],
                                              (float4*)pCLo[0], (float4*)pCHi[0], (int*)pCCnt[0]);
      // rounds run kPlocBatch at a time between host reads of the cluster
      // count; the count of each round lives on the device (pPc[1], pPc[2])
      // and bounds the work of the next, the host's last read bounds the grid
      const int nInit = int(n);
      UBR_CUDA(c, cudaMemcpyAsync(static_cast<int*>(pPc) + 1, &nInit, sizeof(int), cudaMemcpyHostToDevice,
                                  c->stream));
      int ncCap = int(n), cur = 0, which = 0, rounds = 0;
      int* hostPc = static_cast<int*>(c->pinned);
      while (ncCap > 1) {
        const int g = (ncCap + kPlocBlock - 1) / kPlocBlock;
        for (int r = 0; r < kPlocBatch; ++r) {
          const int* ncIn = static_cast<const int*>(pPc) + 1 + which;
          int* ncOut = static_cast<int*>(pPc) + 1 + (which ^ 1);
          k_ploc_nn<<<g, kPlocBlock, 0, c->stream>>>(ncIn, (const float4*)pCLo[cur], (const float4*)pCHi[cur],
                                                     (int*)pNn);
          k_ploc_merge<<<g, kPlocBlock, 0, c->stream>>>(ncIn, ncCap, (const int*)pNn, (int*)pCode[cur],
                                                        (float4*)pCLo[cur], (float4*)pCHi[cur], (int*)pCCnt[cur],
                                                        (float4*)pNodes, (int2*)pRange, (int*)pPc, (int*)pValid,
                                                        (int*)pLeafP, (int*)pNodeP);
          UBR_CUDA(c, cub::DeviceScan::ExclusiveSum(pScan, scanBytes, (const int*)pValid, (int*)pPos, ncCap,
                                                    c->stream));
          k_ploc_compact<<<g, kPlocBlock, 0, c->stream>>>(
              ncCap, (const int*)pValid, (const int*)pPos, (const int*)pCode[cur], (const float4*)pCLo[cur],
              (const float4*)pCHi[cur], (const int*)pCCnt[cur], (int*)pCode[cur ^ 1], (float4*)pCLo[cur ^ 1],
              (float4*)pCHi[cur ^ 1], (int*)pCCnt[cur ^ 1], ncOut);
          which ^= 1;
          cur ^= 1;
        }
        UBR_CUDA(c, cudaGetLastError());
        UBR_CUDA(c, cudaMemcpyAsync(hostPc, pPc, 3 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        UBR_CUDA(c, cudaStreamSynchronize(c->stream));
        const int next = hostPc[1 + which];
        rounds += kPlocBatch;
        if (!(next < ncCap || next == 1) || rounds > (1 << 20))
          return fail(setError(c, UBR_INTERNAL, "PLOC did not converge"));
        ncCap = next;
      }
      if (hostPc[0] != int(n) - 1) return fail(setError(c, UBR_INTERNAL, "PLOC node count mismatch"));
      rootCodeDev = int(n) - 2;  // the last merge makes the root
    }
    // SAH collapse: the DP's cost rows and decisions, bottom-up
    const bool sah = n > 1 && c->collapse == 2;
    void *pCost = nullptr, *pDec = nullptr, *pSahCnt = nullptr;
    if (sah) {
      const size_t nn1 = size_t(n) - 1;
      if ((st = scratchGet(c, 11, sizeof(float) * kSahStride * nn1, &pCost)) != UBR_OK) return fail(st);
      if ((st = scratchGet(c, 12, 8 * nn1, &pDec)) != UBR_OK) return fail(st);
      if ((st = scratchGet(c, 13, sizeof(int) * nn1, &pSahCnt)) != UBR_OK) return fail(st);
      UBR_CUDA(c, cudaMemsetAsync(pSahCnt, 0, sizeof(int) * nn1, c->stream));
      k_sah_costs<<<grid, TB, 0, c->stream>>>(int(n), (const float4*)pNodes, (const int2*)pRange,
                                              (const uint32_t*)pRef, (const int*)pLeafP, (const int*)pNodeP,
                                              (int*)pSahCnt, (float*)pCost, (uint8_t*)pDec, c->sahPrimScale);
      UBR_CUDA(c, cudaGetLastError());
    }
    // collapse to 8-wide, level by level: cursors = {wide nodes, leaf prims, next work}
    {
      const int rootCode = n > 1 ? (rootCodeDev >= 0 ? rootCodeDev : 0) : ~0;
      const int zero = 0;
      const int cur0[3] = {1, 0, 0};
      UBR_CUDA(c, cudaMemcpyAsync(pCur, cur0, sizeof(cur0), cudaMemcpyHostToDevice, c->stream));
      UBR_CUDA(c, cudaMemcpyAsync(pWc[0], &rootCode, sizeof(int), cudaMemcpyHostToDevice, c->stream));
      UBR_CUDA(c, cudaMemcpyAsync(pWw[0], &zero, sizeof(int), cudaMemcpyHostToDevice, c->stream));
      int count = 1, cur = 0, levels = 0;
      int* hostCur = static_cast<int*>(c->pinned);
      while (count > 0) {
        UBR_CUDA(c, cudaMemsetAsync(static_cast<int*>(pCur) + 2, 0, sizeof(int), c->stream));
        if (sah)
          k_collapse_sah<<<(count + 127) / 128, 128, 0, c->stream>>>(
              (const float4*)pNodes, (const uint8_t*)pDec, (const int*)pWc[cur], (const int*)pWw[cur], count,
              (int*)pWc[cur ^ 1], (int*)pWw[cur ^ 1], (int*)pCur, (float4*)pWide, (const uint32_t*)pRef,
              (const float4*)pGeo, (uint32_t*)pRef2, (float4*)pGeo2);
        else
          k_collapse<<<(count + 127) / 128, 128, 0, c->stream>>>(
              (const float4*)pNodes, (const int2*)pRange, (const float4*)pLo, (const float4*)pHi,
              (const int*)pWc[cur], (const int*)pWw[cur], count, c->leafMax, (int*)pWc[cur ^ 1],
              (int*)pWw[cur ^ 1], (int*)pCur, (float4*)pWide, (const uint32_t*)pRef, (const float4*)pGeo,
              (uint32_t*)pRef2, (float4*)pGeo2);
        UBR_CUDA(c, cudaGetLastError());
        UBR_CUDA(c, cudaMemcpyAsync(hostCur, pCur, 3 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        UBR_CUDA(c, cudaStreamSynchronize(c->stream));
        count = hostCur[2];
        cur ^= 1;
        if (++levels > 64) return fail(setError(c, UBR_INTERNAL, "wide BVH collapse did not converge"));
      }
      sc->nodes = uint64_t(hostCur[0]);
      v.wideNodes = uint32_t(hostCur[0]);
      // traversal stack entries pack a node index into 24 bits
      if (sc->nodes >= (1ull << 24))
        return fail(setError(c, UBR_INVALID_ARGUMENT, "scene too large: more than 2^24 wide BVH nodes"));
    }
    v.wnodes = (const float4*)pWide;
    v.nodes = nullptr;
    v.leafRef = (const uint32_t*)pRef2;
    v.leafGeo = (const float4*)pGeo2;
    v.root = 0;
    int cb[6];
    UBR_CUDA(c, cudaMemcpyAsync(cb, pCb, sizeof(cb), cudaMemcpyDeviceToHost, c->stream));
    cudaEventRecord(c->ev[1], c->stream);
    UBR_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int k = 0; k < 3; ++k) {
      auto of = [](int i) {
        int b = i >= 0 ? i : i ^ 0x7FFFFFFF;
        float f;
        std::memcpy(&f, &b, 4);
        return f;
      };
      sc->lo[k] = of(cb[k]);
      sc->hi[k] = of(cb[3 + k]);
    }
  } else {
    cudaEventRecord(c->ev[1], c->stream);
    UBR_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  for (const DevBuf& b : sc->bufs) sc->deviceBytes += b.bytes;
  const auto t1 = std::chrono::steady_clock::now();
  sc->buildMs = std::chrono::duration<double, std::milli>(t1 - t0).count();
  sc->flattenMs = std::chrono::duration<double, std::milli>(tFlat - t0).count();
  sc->uploadMs = std::chrono::duration<double, std::milli>(tUp - tFlat).count();
  *out = sc;
  return UBR_OK;
}

void releaseScene(Scene* sc) {
  if (!sc) return;
  for (DevBuf& b : sc->bufs) devFree(sc->ctx, b);
  delete sc;
}

}  // namespace ubr

// umbreon public scene types for the GB300 drop-in library.
// Declarations match umbreon's scene.hpp (same names, field order, types and
// defaults) so code written against the reference compiles and links
// unchanged; the implementation behind them is this library's.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstdint>
#include <limits>
#include <vector>

#include "render/render_types.hpp"

namespace umbreon {

struct Vec3 {
  float x = 0.0f, y = 0.0f, z = 0.0f;
  Vec3() = default;
  Vec3(float x_, float y_, float z_) : x(x_), y(y_), z(z_) {}
};

inline Vec3 operator+(Vec3 a, Vec3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline Vec3 operator-(Vec3 a, Vec3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline Vec3 operator*(Vec3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline Vec3 operator*(float s, Vec3 a) { return a * s; }
inline float dot(Vec3 a, Vec3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline Vec3 cross(Vec3 a, Vec3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
inline float length(Vec3 a) { return std::sqrt(dot(a, a)); }
inline Vec3 normalize(Vec3 a) {
  const float l = length(a);
  return l > 0.0f ? a * (1.0f / l) : a;
}
// Normalise with the squared length floored at the smallest normal float, so
// a zero vector comes back finite (zero) rather than NaN.
inline Vec3 safeNormalize(Vec3 a) {
  const float s = 1.0f / std::sqrt(std::fmax(dot(a, a), 0x1.0p-126f));
  return a * s;
}
// Normalise, or return `fallback` when |a| < 1e-9.
inline Vec3 safeNormalize(Vec3 a, Vec3 fallback) {
  const float d = dot(a, a);
  if (d < 1.0e-18f) return fallback;
  return a * (1.0f / std::sqrt(d));
}

// Orthonormal frame with n as the local +z axis.
struct Frame {
  Vec3 t, b, n;
};
inline Frame frameFromNormal(Vec3 n) {
  const Vec3 seed0{0.0f, n.z, -n.y};
  const Vec3 seed1{-n.z, 0.0f, n.x};
  const Vec3 t = safeNormalize(std::fabs(n.x) < std::fabs(n.y) ? seed0 : seed1, Vec3{1.0f, 0.0f, 0.0f});
  return {t, cross(n, t), n};
}

inline float radians(float deg) { return deg * 0.01745329252f; }
inline float degrees(float rad) { return rad * 57.2957795131f; }

struct Vec4 {
  float x = 0.0f, y = 0.0f, z = 0.0f, w = 1.0f;
  Vec4() = default;
  Vec4(float x_, float y_, float z_, float w_) : x(x_), y(y_), z(z_), w(w_) {}
};

struct Aabb {
  Vec3 lo{1e30f, 1e30f, 1e30f};
  Vec3 hi{-1e30f, -1e30f, -1e30f};
  void extend(Vec3 p) {
    lo = {std::fmin(lo.x, p.x), std::fmin(lo.y, p.y), std::fmin(lo.z, p.z)};
    hi = {std::fmax(hi.x, p.x), std::fmax(hi.y, p.y), std::fmax(hi.z, p.z)};
  }
  bool valid() const { return lo.x <= hi.x; }
  Vec3 center() const { return (lo + hi) * 0.5f; }
  Vec3 extent() const { return hi - lo; }
  float diagonal() const { return length(extent()); }
};

enum class ShadingModel : uint8_t { Pov = 0, Principled = 1, Toon = 2 };

// POV finish plus the principled parameters.  This library shades the Pov
// and Toon models (identical lobes) and the Principled model's direct pass
// (GGX / Smith / Schlick, src/umbreon/shading/principled.hpp:139).
struct Material {
  float ambient = 0.2f;
  float diffuse = 0.8f;
  float specular = 0.0f;
  float roughness = 0.02f;
  float brilliance = 1.0f;
  float phong = 0.0f;
  float phongSize = 40.0f;
  bool metallic = false;
  float reflection = 0.0f;
  float emission = 0.0f;
  ShadingModel model = ShadingModel::Pov;
  struct Pbr {
    float metallic = 0.0f;
    float roughness = 0.5f;
    float specular = 0.5f;
    float anisotropy = 0.0f;
    float anisotropyRotation = 0.0f;
  } pbr;

  float diffuseWeight() const {
    return model == ShadingModel::Principled ? diffuse * (1.0f - pbr.metallic) : diffuse;
  }
  bool toonLike() const {
    if (model == ShadingModel::Toon) return true;
    if (model != ShadingModel::Pov) return false;
    if (specular > 1.0f || phong > 1.0f || brilliance == 0.0f) return true;
    return diffuse <= 0.0f && specular <= 0.0f && phong <= 0.0f && reflection <= 0.0f;
  }
  // ambient 1, diffuse 0, no highlight: out = pigment under unit ambient light
  static Material flatOutline() {
    Material m;
    m.ambient = 1.0f;
    m.diffuse = 0.0f;
    return m;
  }
};

struct Mesh {
  std::vector<Vec3> positions;
  std::vector<Vec3> normals;
  std::vector<Vec4> colors;
  std::vector<uint32_t> index;      // 3 per triangle, or empty = de-indexed
  std::vector<int32_t> posClass;
  int32_t posClassCount = 0;
  Material material;
  std::vector<Material> materials;
  std::vector<uint8_t> triMaterialId;
  std::vector<uint16_t> triGroupId;

  std::size_t vertexCount() const { return positions.size(); }
  std::size_t cornerCount() const { return index.empty() ? positions.size() : index.size(); }
  std::size_t triangleCount() const { return cornerCount() / 3; }
  uint32_t cornerVertex(std::size_t corner) const {
    return index.empty() ? static_cast<uint32_t>(corner) : index[corner];
  }
  const Material& materialForTri(std::size_t triIdx) const {
    return triMaterialId.empty() ? material : materials[triMaterialId[triIdx]];
  }
  uint16_t groupForTri(std::size_t triIdx) const { return triGroupId.empty() ? 0 : triGroupId[triIdx]; }
  Aabb bounds() const {
    Aabb b;
    for (const Vec3& p : positions) b.extend(p);
    return b;
  }
  Mesh toDeindexed() const {
    if (index.empty()) return *this;
    Mesh m;
    const bool haveNrm = normals.size() == positions.size();
    const bool haveCol = colors.size() == positions.size();
    for (uint32_t v : index) {
      m.positions.push_back(positions[v]);
      if (haveNrm) m.normals.push_back(normals[v]);
      if (haveCol) m.colors.push_back(colors[v]);
    }
    m.material = material;
    m.materials = materials;
    m.triMaterialId = triMaterialId;
    m.triGroupId = triGroupId;
    return m;
  }
};

struct Sphere {
  Vec3 center;
  float radius = 1.0f;
  Vec4 color{0.0f, 0.0f, 0.0f, 1.0f};
  Material material = Material::flatOutline();
  uint16_t group = 0;
  bool fromEdgeMacro = false;
};

struct Cylinder {
  Vec3 p0, p1;
  float radius = 1.0f;
  Vec4 color{0.0f, 0.0f, 0.0f, 1.0f};
  Material material = Material::flatOutline();
  uint16_t group = 0;
  float opacity1 = -1.0f;
  bool open = false;
  bool fromEdgeMacro = false;
};

struct GroupBlend {
  uint16_t group = 0;
  float alpha = 1.0f;
};

struct Camera {
  Vec3 position{0.0f, 0.0f, 1.0f};
  Vec3 direction{0.0f, 0.0f, -1.0f};
  Vec3 up{0.0f, 1.0f, 0.0f};
  float fovy = 40.0f;
  bool orthographic = false;
  float height = 1.0f;
};

struct DistantLight {
  Vec3 direction{0.0f, -0.3f, -1.0f};
  Vec3 color{1.0f, 1.0f, 1.0f};
  float intensity = 1.0f;
  bool castsHighlight = true;
  float angularRadius = 0.0f;
};

struct Fog {
  bool enabled = false;
  Vec3 color{0.0f, 0.0f, 0.0f};
  float start = 0.0f;
  float end = 0.0f;
  float distance = 1.0e30f;
  int type = 1;
  float offset = 0.0f;
  float alt = 0.0f;
  Vec3 up{0.0f, 1.0f, 0.0f};
};

struct Scene {
  Mesh mesh;
  std::vector<Sphere> spheres;
  std::vector<Cylinder> cylinders;
  std::vector<Vec3> instanceOffsets;
  Camera camera;
  std::vector<DistantLight> lights;
  float ambientIntensity = 0.25f;
  Vec3 ambientColor{1.0f, 1.0f, 1.0f};
  Vec3 background{0.0f, 0.0f, 0.0f};
  Fog fog;
  float aoDistance = 1.0e20f;
  float assumedGamma = 1.0f;
  float clipNear = -std::numeric_limits<float>::infinity();
  float clipFar = std::numeric_limits<float>::infinity();
  bool clipEnabled() const {
    return clipNear > -std::numeric_limits<float>::infinity() ||
           clipFar < std::numeric_limits<float>::infinity();
  }
  std::vector<GroupBlend> groupBlend;
  std::vector<EdgeStyle> groupEdgeStyle;

  std::size_t instanceCount() const { return instanceOffsets.size(); }
  std::size_t effectiveTriangles() const {
    return mesh.triangleCount() * (instanceOffsets.empty() ? 1 : instanceOffsets.size());
  }
};

}  // namespace umbreon

// pov_dump -- print what the POV readers recover, one field per line with
// floats in hex, so two builds of this program (against this library's
// readers, and against the reference's) can be compared byte for byte.
//
//   pov_dump scene FILE.pov [WIDTH HEIGHT [name=value ...]]
//   pov_dump geom FILE.inc [name=value ...]
#include <cstdio>
#include <cstdlib>
#include <exception>
#include <string>

#include "geom/mesh2_reader.hpp"
#include "pov/pov_scene_reader.hpp"

namespace {

void f(const char* k, float v) { std::printf("%s %a\n", k, static_cast<double>(v)); }
void v3(const char* k, const umbreon::Vec3& v) {
  std::printf("%s %a %a %a\n", k, static_cast<double>(v.x), static_cast<double>(v.y), static_cast<double>(v.z));
}
void v4(const char* k, const umbreon::Vec4& v) {
  std::printf("%s %a %a %a %a\n", k, static_cast<double>(v.x), static_cast<double>(v.y), static_cast<double>(v.z),
              static_cast<double>(v.w));
}
void material(const umbreon::Material& m) {
  std::printf("material %a %a %a %a %a %a %a %d %a %a\n", m.ambient, m.diffuse, m.specular, m.roughness,
              m.brilliance, m.phong, m.phongSize, m.metallic ? 1 : 0, m.reflection, m.emission);
}

int scene(int argc, char** argv) {
  umbreon::PovParseOptions o;
  int k = 3;
  if (argc > 4) {
    o.imageWidth = std::atoi(argv[3]);
    o.imageHeight = std::atoi(argv[4]);
    k = 5;
  }
  for (; k < argc; ++k) {
    const std::string a = argv[k];
    const std::size_t eq = a.find('=');
    if (eq != std::string::npos) o.predefined[a.substr(0, eq)] = std::atof(a.c_str() + eq + 1);
  }
  const umbreon::PovSceneResult r = umbreon::readPovScene(argv[2], o);
  v3("camera.position", r.camera.position);
  v3("camera.direction", r.camera.direction);
  v3("camera.up", r.camera.up);
  f("camera.fovy", r.camera.fovy);
  std::printf("camera.orthographic %d\n", r.camera.orthographic ? 1 : 0);
  f("camera.height", r.camera.height);
  for (const auto& L : r.lights) {
    v3("light.direction", L.direction);
    v3("light.color", L.color);
    f("light.intensity", L.intensity);
    std::printf("light.highlight %d\n", L.castsHighlight ? 1 : 0);
    f("light.angularRadius", L.angularRadius);
  }
  v3("background", r.background);
  std::printf("fog.enabled %d type %d\n", r.fog.enabled ? 1 : 0, r.fog.type);
  v3("fog.color", r.fog.color);
  f("fog.start", r.fog.start);
  f("fog.end", r.fog.end);
  f("fog.distance", r.fog.distance);
  f("fog.offset", r.fog.offset);
  f("fog.alt", r.fog.alt);
  v3("fog.up", r.fog.up);
  f("assumedGamma", r.assumedGamma);
  for (const auto& kv : r.declares) {
    std::printf("declare %s", kv.first.c_str());
    for (double x : kv.second) std::printf(" %a", x);
    std::printf("\n");
  }
  std::printf("include %s\nradiosity %d\n", r.includePath.c_str(), r.radiosity ? 1 : 0);
  return 0;
}

int geom(int argc, char** argv) {
  umbreon::SymbolTable seed;
  for (int k = 3; k < argc; ++k) {
    const std::string a = argv[k];
    const std::size_t eq = a.find('=');
    if (eq != std::string::npos) seed[a.substr(0, eq)] = {std::atof(a.c_str() + eq + 1)};
  }
  const umbreon::SceneGeometry g = umbreon::readGeometryFromFile(argv[2], seed);
  const umbreon::Mesh& m = g.mesh;
  std::printf("vertices %zu triangles %zu classes %d\n", m.vertexCount(), m.triangleCount(), m.posClassCount);
  for (std::size_t i = 0; i < m.positions.size(); ++i) {
    v3("p", m.positions[i]);
    v3("n", m.normals[i]);
    v4("c", m.colors[i]);
    std::printf("class %d\n", m.posClass[i]);
  }
  for (std::size_t i = 0; i < m.index.size(); ++i) std::printf("i %u\n", m.index[i]);
  for (std::size_t t = 0; t < m.triMaterialId.size(); ++t)
    std::printf("tri %u group %u\n", m.triMaterialId[t], static_cast<unsigned>(m.triGroupId[t]));
  material(m.material);
  for (const auto& mm : m.materials) material(mm);
  for (const auto& s : g.spheres) {
    v3("sphere", s.center);
    f("radius", s.radius);
    v4("color", s.color);
    material(s.material);
    std::printf("group %u edge %d\n", static_cast<unsigned>(s.group), s.fromEdgeMacro ? 1 : 0);
  }
  for (const auto& c : g.cylinders) {
    v3("cylinder.p0", c.p0);
    v3("cylinder.p1", c.p1);
    f("radius", c.radius);
    v4("color", c.color);
    f("opacity1", c.opacity1);
    material(c.material);
    std::printf("group %u open %d edge %d\n", static_cast<unsigned>(c.group), c.open ? 1 : 0,
                c.fromEdgeMacro ? 1 : 0);
  }
  for (const auto& n : g.groupNames) std::printf("groupName '%s'\n", n.c_str());
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: pov_dump scene|geom FILE [...]\n");
    return 2;
  }
  try {
    const std::string mode = argv[1];
    return mode == "scene" ? scene(argc, argv) : geom(argc, argv);
  } catch (const std::exception& e) {
    std::printf("error %s\n", e.what());
    return 1;
  }
}

// umbreon::render through the GB300 library: the reference's own render
// known answers (tests/test_render_shading.cpp, test_render_transparency.cpp,
// test_render_shadows_gi.cpp), group-alpha blending and async/cancel, written
// against the unchanged public API.
#include <chrono>
#include <cmath>
#include <stdexcept>
#include <vector>

#include "check.hpp"
#include "postprocess/image_ops.hpp"
#include "umbreon.hpp"

using umbreon::Vec3;
using umbreon::Vec4;

namespace {
constexpr std::size_t kC = (2 * 5 + 2) * 4;

umbreon::Mesh quad(Vec4 col, float z = 0.0f) {
  umbreon::Mesh m;
  const Vec3 p[6] = {{-2, -2, z}, {2, -2, z}, {2, 2, z}, {-2, -2, z}, {2, 2, z}, {-2, 2, z}};
  for (const Vec3& v : p) {
    m.positions.push_back(v);
    m.normals.push_back({0, 0, 1});
    m.colors.push_back(col);
  }
  m.material.ambient = 0.2f;
  m.material.diffuse = 0.8f;
  return m;
}
umbreon::Camera cam() {
  umbreon::Camera c;
  c.position = {0, 0, 10};
  c.direction = {0, 0, -1};
  c.orthographic = true;
  c.height = 4.0f;
  return c;
}
umbreon::DistantLight key() {
  umbreon::DistantLight l;
  l.direction = {0, 0, -1};
  l.intensity = 0.5f;
  return l;
}
umbreon::RenderOptions o5() {
  umbreon::RenderOptions o;
  o.width = 5;
  o.height = 5;
  return o;
}
void addQuad(umbreon::Mesh& m, Vec4 col, float z, uint16_t g) {
  const umbreon::Mesh q = quad(col, z);
  m.positions.insert(m.positions.end(), q.positions.begin(), q.positions.end());
  m.normals.insert(m.normals.end(), q.normals.begin(), q.normals.end());
  m.colors.insert(m.colors.end(), q.colors.begin(), q.colors.end());
  m.triGroupId.push_back(g);
  m.triGroupId.push_back(g);
}
}  // namespace

int main() {
  Checks c;
  {  // mesh direct shading: C * (0.2 + 0.8 * 0.5)
    umbreon::Scene sc;
    sc.mesh = quad({0.5f, 0.6f, 0.7f, 1.0f});
    sc.camera = cam();
    sc.lights.push_back(key());
    umbreon::FrameResult f = umbreon::render(sc, o5());
    c("mesh centre = C*0.6", near(f.color[kC], 0.30f, 1e-4f) && near(f.color[kC + 1], 0.36f, 1e-4f) &&
                                 near(f.color[kC + 2], 0.42f, 1e-4f));
    c("mesh depth = 10", near(f.depth[12], 10.0f, 1e-3f));
    c("frame size", f.width == 5 && f.height == 5 && f.color.size() == 100);
  }
  {  // supersample keeps the final size and the uniform value
    umbreon::Scene sc;
    sc.mesh = quad({0.5f, 0.6f, 0.7f, 1.0f});
    sc.camera = cam();
    sc.lights.push_back(key());
    umbreon::RenderOptions o = o5();
    o.supersample = 2;
    umbreon::FrameResult f = umbreon::render(sc, o);
    c("ss2 final 5x5, depth on the 10x10 grid", f.width == 5 && f.depth.size() == 100);
    c("ss2 value", near(f.color[kC], 0.30f, 1e-4f));
  }
  {  // fragment over, F2 order dependence
    umbreon::Mesh m;
    addQuad(m, {1, 0, 0, 1.0f}, 0.0f, 0);
    addQuad(m, {0, 0, 1, 0.5f}, 0.5f, 2);
    addQuad(m, {0, 1, 0, 0.5f}, 1.0f, 1);
    m.material = umbreon::Material::flatOutline();
    umbreon::Scene sc;
    sc.mesh = m;
    sc.camera = cam();
    umbreon::FrameResult f = umbreon::render(sc, o5());
    c("F2 green front G=0.5 B=0.25", near(f.color[kC + 1], 0.5f, 1e-4f) && near(f.color[kC + 2], 0.25f, 1e-4f));
  }
  {  // group-alpha T1: 0.6 * blue + 0.4 * red in the display domain
    umbreon::Mesh m;
    addQuad(m, {1, 0, 0, 1.0f}, 0.0f, 0);
    addQuad(m, {0, 0, 1, 1.0f}, 1.0f, 1);
    m.material = umbreon::Material::flatOutline();
    umbreon::Scene sc;
    sc.mesh = m;
    sc.camera = cam();
    sc.groupBlend.push_back({1, 0.6f});
    umbreon::FrameResult f = umbreon::render(sc, o5());
    c("T1 blend R=0.4 B=0.6 (sRGB domain)", near(umbreon::srgbEncodeF(f.color[kC]), 0.4f, 1e-4f) &&
                                                near(umbreon::srgbEncodeF(f.color[kC + 2]), 0.6f, 1e-4f));
  }
  {  // hard shadow from a slab
    umbreon::Scene sc;
    sc.mesh = quad({1, 1, 1, 1});
    const umbreon::Mesh slab = quad({0, 0, 0, 1}, 0.4f);
    for (int i = 0; i < 6; ++i) {
      Vec3 p = slab.positions[i];
      p.x = p.x < 0 ? 0.1f : 4.0f;
      sc.mesh.positions.push_back(p);
      sc.mesh.normals.push_back({0, 0, -1});
      sc.mesh.colors.push_back({0, 0, 0, 1});
    }
    sc.camera = cam();
    umbreon::DistantLight l;
    l.direction = {-0.6f, 0.0f, -0.8f};
    sc.lights.push_back(l);
    umbreon::RenderOptions off = o5(), on = o5();
    on.shadows = true;
    const float a = umbreon::render(sc, off).color[kC], b = umbreon::render(sc, on).color[kC];
    c("shadow off ~0.84, on ~0.2", near(a, 0.84f, 0.03f) && near(b, 0.2f, 0.03f));
  }
  {  // AO AOVs (aoWriteAov): mesh first hit carries albedo = C, normal = N and an
     // open quad's contact / shape openness 1; empty when not requested
    umbreon::Scene sc;
    sc.mesh = quad({0.5f, 0.6f, 0.7f, 1.0f});
    sc.camera = cam();
    sc.lights.push_back(key());
    umbreon::RenderOptions o = o5();
    o.aoSamples = 8;
    o.aoDistance = 2.0f;
    umbreon::FrameResult plain = umbreon::render(sc, o);
    c("no AOVs unless asked", plain.albedo.empty() && plain.contactAo.empty());
    o.aoWriteAov = true;
    umbreon::FrameResult f = umbreon::render(sc, o);
    const std::size_t p = 12;
    c("AOV sizes", f.albedo.size() == 75 && f.normal.size() == 75 && f.bentNormal.size() == 75 &&
                       f.contactAo.size() == 25 && f.shapeAo.size() == 25 && f.avgHitDist.size() == 25);
    c("albedo = vertex colour", near(f.albedo[3 * p], 0.5f, 1e-6f) && near(f.albedo[3 * p + 2], 0.7f, 1e-6f));
    c("normal = +z", near(f.normal[3 * p + 2], 1.0f, 1e-6f));
    c("open quad: contact = shape = 1, no occluder", near(f.contactAo[p], 1.0f, 1e-6f) &&
                                                         near(f.shapeAo[p], 1.0f, 1e-6f) &&
                                                         near(f.avgHitDist[p], 2.0f, 1e-6f));
    c("colour unchanged by the AOVs", near(f.color[kC], plain.color[kC], 0.0f));
  }
  {  // adaptive AA: a flat quad flags nothing and replicates its centres; the
     // mask is returned at the output resolution only with aaDebug
    umbreon::Scene sc;
    sc.mesh = quad({0.5f, 0.6f, 0.7f, 1.0f});
    sc.camera = cam();
    sc.lights.push_back(key());
    umbreon::RenderOptions o = o5();
    o.supersample = 2;
    const umbreon::FrameResult grid = umbreon::render(sc, o);
    o.aaMode = 1;
    c("no mask without aaDebug", umbreon::render(sc, o).aaMask.empty());
    o.aaDebug = true;
    const umbreon::FrameResult f = umbreon::render(sc, o);
    bool none = f.aaMask.size() == 25;
    for (float v : f.aaMask) none = none && v == 0.0f;
    c("flat quad: mask of 25 zeros", none);
    c("adaptive centre = grid colour", near(f.color[kC], grid.color[kC], 1e-6f));
  }
  {  // principled materials render through the drop-in: metallic = 0 and
     // specular = 0 is the POV diffuse-only image bitwise; a metal differs
    umbreon::Scene pov;
    pov.mesh = quad({0.5f, 0.6f, 0.7f, 1.0f});
    pov.mesh.material.specular = 0.0f;
    pov.camera = cam();
    pov.lights.push_back(key());
    umbreon::Scene pbr = pov;
    pbr.mesh.material.model = umbreon::ShadingModel::Principled;
    pbr.mesh.material.pbr.metallic = 0.0f;
    pbr.mesh.material.pbr.specular = 0.0f;
    const umbreon::FrameResult a = umbreon::render(pov, o5()), b = umbreon::render(pbr, o5());
    bool same = a.color.size() == b.color.size();
    for (std::size_t i = 0; same && i < a.color.size(); ++i) same = a.color[i] == b.color[i];
    c("principled diffuse-only == POV diffuse-only (bitwise)", same);
    umbreon::Scene metal = pbr;
    metal.mesh.material.pbr.metallic = 1.0f;
    metal.mesh.material.pbr.specular = 0.5f;
    metal.mesh.material.pbr.roughness = 0.3f;
    const umbreon::FrameResult m = umbreon::render(metal, o5());
    c("principled metal differs and stays finite", m.color[kC] != a.color[kC] && std::isfinite(m.color[kC]));
  }
  {  // coarse-grid AO through the drop-in: the fallback mask is hi-res
    umbreon::Scene sc;
    sc.mesh = quad({0.8f, 0.8f, 0.8f, 1.0f});
    sc.camera = cam();
    sc.lights.push_back(key());
    umbreon::RenderOptions o = o5();
    o.supersample = 2;
    o.aoSamples = 8;
    o.aoDistance = 2.0f;
    o.aoResDiv = -1;
    o.aoResDebug = true;
    const umbreon::FrameResult f = umbreon::render(sc, o);
    c("coarse AO: patch mask at render resolution", f.aoPatchMask.size() == 100);
    c("coarse AO: open quad stays lit", f.color[kC] > 0.3f);
  }
  {  // pt1 GI at its defaults renders (reduced gather grid, denoise, upsample,
     // edge patch), pt2 with and without ReSTIR rounds; the irradiance cache
     // is not built and throws
    umbreon::Scene sc;
    sc.mesh = quad({1, 1, 1, 1});
    sc.camera = cam();
    sc.lights.push_back(key());
    umbreon::RenderOptions o = o5();
    o.supersample = 2;
    o.gi = true;
    o.giIntegrator = 1;
    const umbreon::FrameResult f = umbreon::render(sc, o);
    c("pt1 defaults: frame rendered", f.color.size() == 100 && f.color[kC] > 0.0f);
    c("pt1 defaults: gather rays counted", f.pt1Rays.gatherRays > 0 && f.pt1Rays.gbufferRays > 0);
    c("pt1 defaults: a-trous denoise of E reported", f.pt1DenoiserUsed == 1);
    o.giIntegrator = 2;  // the reference's default integrator, every option at its default
    const umbreon::FrameResult f2 = umbreon::render(sc, o);
    c("pt2 defaults: frame rendered", f2.color.size() == 100 && f2.color[kC] > 0.0f);
    c("pt2 defaults: gather rays counted", f2.pt1Rays.gatherRays > 0);
    o.pt2Rounds = 2;  // ReSTIR spatial rounds on top of the defaults
    const umbreon::FrameResult f3 = umbreon::render(sc, o);
    c("pt2 ReSTIR rounds: frame rendered", f3.color.size() == 100 && f3.color[kC] > 0.0f);
    o.pt2Rounds = 0;
    o.giIntegrator = 0;
    bool threw = false;
    try {
      umbreon::render(sc, o);
    } catch (const std::runtime_error&) {
      threw = true;
    }
    c("irradiance-cache GI request throws std::runtime_error", threw);
  }
  {  // async == blocking; cancel before start yields a cancelled frame
    umbreon::Scene sc;
    sc.mesh = quad({0.5f, 0.6f, 0.7f, 1.0f});
    sc.camera = cam();
    sc.lights.push_back(key());
    umbreon::RenderOptions o = o5();
    o.aoSamples = 8;
    o.aoDistance = 10.0f;
    const umbreon::FrameResult blocking = umbreon::render(sc, o);
    umbreon::RenderTask t = umbreon::renderAsync(sc, o);
    t.wait();
    const umbreon::FrameResult async = t.get();
    c("async result == blocking result", async.color == blocking.color);
    umbreon::RenderProgress p;
    p.requestCancel();
    const umbreon::FrameResult cf = umbreon::render(sc, o, p);
    c("pre-cancelled render reports cancelled", cf.cancelled);
  }
  return c.report("host_render");
}

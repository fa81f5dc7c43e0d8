// mesh2_reader.cpp -- the geometry of a CueMol .inc (geom/mesh2_reader.hpp).
// One scan of the token stream: #declare values and textures are recorded,
// mesh2 / sphere / cylinder blocks and edge_line / edge_line2 calls become
// geometry, `#if (_show_<id>)` wrappers set the transparency group.  Unlike
// the scene reader, conditionals are not evaluated: every branch is scanned
// (CueMol toggles whole objects with them), and function calls evaluate to
// nothing.  Behaviour follows the reference reader (src/bench/geom/
// mesh2_reader.cpp, mesh2_texture_parse.cpp, mesh2_block_parser.cpp,
// mesh2_build.cpp): which finish a block adopts, how pigments become colours,
// the edge_line argument layout, cylinder caps, and the two welds of
// mesh2_build.cpp:53-160.
#include "geom/mesh2_reader.hpp"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>
#include <unordered_map>
#include <utility>

#include "sdl.hpp"

namespace umbreon {
namespace {

using sdl::Kind;
using sdl::Val;

Vec3 vec3Of(const Val& v) {
  return Vec3{static_cast<float>(v.at(0)), static_cast<float>(v.at(1)), static_cast<float>(v.at(2))};
}

float srgbToLinear(float c) { return c <= 0.04045f ? c / 12.92f : std::pow((c + 0.055f) / 1.055f, 2.4f); }

// A colour `kind expr`: rgb / rgbf / rgbt / rgbft, optionally sRGB-encoded;
// a scalar is grey, nothing is white; filter / transmit (the 4th component
// of the transparent kinds) gives opacity 1 - t.
Vec4 colorOf(const Val& v, const std::string& kind) {
  float r = 1.0f, g = 1.0f, b = 1.0f;
  if (v.n >= 3) {
    r = static_cast<float>(v.v[0]);
    g = static_cast<float>(v.v[1]);
    b = static_cast<float>(v.v[2]);
  } else if (v.n >= 1) {
    r = g = b = static_cast<float>(v.v[0]);
  }
  const bool transparent = kind != "rgb" && kind != "srgb";
  const float opacity = transparent && v.n >= 4 ? 1.0f - static_cast<float>(v.v[3]) : 1.0f;
  if (kind.compare(0, 4, "srgb") == 0) {
    r = srgbToLinear(r);
    g = srgbToLinear(g);
    b = srgbToLinear(b);
  }
  return Vec4{r, g, b, opacity};
}

// The metallic finishes of POV-Ray's standard metals.inc (F_MetalA..E),
// which CueMol names but does not define in its files: ambient,
// brilliance, diffuse, specular, roughness, reflection; metallic, no phong.
bool namedFinish(const std::string& name, Material& out) {
  struct Preset {
    const char* name;
    float ambient, brilliance, diffuse, specular, roughness, reflection;
  };
  static const Preset kMetals[] = {
      {"F_MetalA", 0.35f, 2.0f, 0.3f, 0.80f, 1.0f / 20.0f, 0.10f},
      {"F_MetalB", 0.30f, 3.0f, 0.4f, 0.70f, 1.0f / 60.0f, 0.25f},
      {"F_MetalC", 0.25f, 4.0f, 0.5f, 0.80f, 1.0f / 80.0f, 0.50f},
      {"F_MetalD", 0.15f, 5.0f, 0.6f, 0.80f, 1.0f / 100.0f, 0.65f},
      {"F_MetalE", 0.10f, 6.0f, 0.7f, 0.80f, 1.0f / 120.0f, 0.80f},
  };
  for (const Preset& p : kMetals) {
    if (name != p.name) continue;
    out = Material{};
    out.ambient = p.ambient;
    out.brilliance = p.brilliance;
    out.diffuse = p.diffuse;
    out.specular = p.specular;
    out.roughness = p.roughness;
    out.reflection = p.reflection;
    out.metallic = true;
    out.phong = 0.0f;
    return true;
  }
  return false;
}

// Render-vertex key: the bits of (position, normal, colour).
struct CornerKey {
  uint32_t w[10];
  bool operator==(const CornerKey& o) const { return std::memcmp(w, o.w, sizeof(w)) == 0; }
};
struct CornerHash {
  std::size_t operator()(const CornerKey& k) const {
    uint64_t h = 0x9E3779B97F4A7C15ull;
    for (uint32_t x : k.w) h = (h ^ x) * 0xFF51AFD7ED558CCDull + (h >> 29);
    return static_cast<std::size_t>(h);
  }
};
// Position-class key: the position on a 1e-4 grid (lround of p * 1e4).
struct CellKey {
  long x, y, z;
  bool operator==(const CellKey& o) const { return x == o.x && y == o.y && z == o.z; }
};
struct CellHash {
  std::size_t operator()(const CellKey& k) const {
    return static_cast<std::size_t>(k.x) * 73856093u ^ static_cast<std::size_t>(k.y) * 19349663u ^
           static_cast<std::size_t>(k.z) * 83492791u;
  }
};
constexpr float kCellsPerUnit = 1.0e4f;

struct Texture {
  Vec4 color{1.0f, 1.0f, 1.0f, 1.0f};
  Material finish;
  bool hasFinish = false;
};

struct Face {
  int v[3] = {0, 0, 0};
  int tex[3] = {0, 0, 0};
  bool hasTex = false;
};

class Mesh2Scan {
 public:
  Mesh2Scan(std::vector<sdl::Tok> toks, const SymbolTable& seed) : s_(std::move(toks)) {
    for (const auto& kv : seed) {
      Val v;
      v.n = static_cast<int>(std::min<std::size_t>(4, kv.second.size()));
      for (int i = 0; i < v.n; ++i) v.v[i] = kv.second[static_cast<std::size_t>(i)];
      vars_[kv.first] = v;
    }
  }

  SceneGeometry read() {
    while (!s_.done()) {
      if (s_.sym('#')) {
        s_.next();
        directive();
        continue;
      }
      const std::string w = s_.name() ? s_.cur().text : std::string();
      if (w == "mesh2") {
        s_.next();
        mesh2();
      } else if (w == "sphere" && s_.isSym(s_.pos + 1, '{')) {
        s_.next();
        sphere();
      } else if (w == "cylinder" && s_.isSym(s_.pos + 1, '{')) {
        s_.next();
        cylinder();
      } else if ((w == "edge_line" || w == "edge_line2") && s_.isSym(s_.pos + 1, '(')) {
        s_.next();
        edgeLine(w == "edge_line2");
      } else {
        s_.next();
      }
    }
    if (!haveMesh_ && out_.spheres.empty() && out_.cylinders.empty())
      throw Mesh2ReadError("no geometry (mesh2/sphere/edge_line) found in input");
    if (!blockMaterials_.empty()) {
      out_.mesh.materials = std::move(blockMaterials_);
      out_.mesh.material = out_.mesh.materials[0];
    }
    out_.groupNames = std::move(groups_);
    return std::move(out_);
  }

 private:
  Val expr() { return s_.expr(vars_, false); }
  std::size_t closing(std::size_t open) const {
    const std::size_t c = s_.closing(open);
    if (c == std::string::npos) throw Mesh2ReadError("unbalanced '{' near line " + std::to_string(s_.at(open).line));
    return c;
  }
  bool blockAt(std::size_t k, const char* word) const {
    return s_.isName(k) && s_.at(k).text == word && s_.isSym(k + 1, '{');
  }

  // ---- directives (cursor on the word after '#') ----
  void directive() {
    if (!s_.name()) return;
    const std::string d = s_.cur().text;
    if (d == "macro") {
      s_.skipMacro();
      return;
    }
    s_.next();
    if (d == "declare" || d == "local") {
      declare();
    } else if (d == "if" || d == "ifdef" || d == "ifndef") {
      // CueMol wraps each rendering object in `#if (_show_<id>)`: its
      // primitives form transparency group <id> (created on first use)
      groupStack_.push_back(group_);
      const std::string show = showVariable();
      if (!show.empty()) group_ = groupOf(show.size() > 5 ? show.substr(5) : show);
    } else if (d == "end") {
      if (!groupStack_.empty()) {
        group_ = groupStack_.back();
        groupStack_.pop_back();
      }
    }
  }
  // a `_show*` name inside the parenthesised condition at the cursor
  std::string showVariable() const {
    if (!s_.sym('(')) return std::string();
    int depth = 0;
    for (std::size_t k = s_.pos; k < s_.size() && s_.at(k).kind != Kind::Eof; ++k) {
      if (s_.isSym(k, '(')) {
        ++depth;
      } else if (s_.isSym(k, ')')) {
        if (--depth == 0) break;
      } else if (s_.isName(k) && s_.at(k).text.compare(0, 5, "_show") == 0) {
        return s_.at(k).text;
      }
    }
    return std::string();
  }
  int groupOf(const std::string& id) {
    const auto it = groupIndex_.find(id);
    if (it != groupIndex_.end()) return it->second;
    const int g = static_cast<int>(groups_.size());
    groups_.push_back(id);
    groupIndex_.emplace(id, g);
    return g;
  }

  void declare() {
    if (!s_.name()) return;
    const std::string id = s_.cur().text;
    s_.next();
    if (!s_.sym('=')) return;
    s_.next();
    if (s_.name()) {
      const std::string& w = s_.cur().text;
      if (w == "texture") {
        s_.next();
        if (!s_.sym('{')) return;
        const std::size_t open = s_.pos, close = closing(open);
        const Texture t = textureBody(open + 1, close);
        textures_[id] = t;
        adopt(t);
        s_.pos = close + 1;
        return;
      }
      if (w == "pigment" || w == "finish" || w == "normal" || w == "material") {
        s_.next();
        if (s_.sym('{')) s_.pos = closing(s_.pos) + 1;
        return;
      }
    }
    const Val v = expr();
    if (v.n > 0) vars_[id] = v;
    s_.skipStatement();
  }

  // ---- textures ----
  // The first finish seen while a mesh2 block is open (from a declared
  // texture or its texture_list) becomes that block's material.
  void adopt(const Texture& t) {
    if (t.hasFinish && !haveBlockMaterial_) {
      blockMaterial_ = t.finish;
      haveBlockMaterial_ = true;
    }
  }

  // texture { [name] [pigment { ... }] [finish { ... }] } over tokens
  // [begin, end); a leading name refers to a declared texture whose colour
  // and finish fill what the block does not set
  Texture textureBody(std::size_t begin, std::size_t end) {
    Texture t;
    bool haveColor = false;
    std::string base;
    std::size_t k = begin;
    while (k < end) {
      if (blockAt(k, "pigment")) {
        const std::size_t c = closing(k + 1);
        Vec4 col;
        if (pigmentColor(k + 2, c, col)) {
          t.color = col;
          haveColor = true;
        }
        k = c + 1;
      } else if (blockAt(k, "finish")) {
        const std::size_t c = closing(k + 1);
        t.finish = finish(k + 2, c);
        t.hasFinish = true;
        k = c + 1;
      } else if (s_.isName(k)) {
        if (base.empty() && !haveColor && s_.at(k).text != "pigment" && s_.at(k).text != "finish")
          base = s_.at(k).text;
        ++k;
      } else if (s_.isSym(k, '{')) {
        k = closing(k) + 1;
      } else {
        ++k;
      }
    }
    if (!base.empty()) {
      const auto it = textures_.find(base);
      if (it != textures_.end()) {
        if (!haveColor) t.color = it->second.color;
        if (!t.hasFinish && it->second.hasFinish) {
          t.finish = it->second.finish;
          t.hasFinish = true;
        }
      }
    }
    return t;
  }

  bool pigmentColor(std::size_t begin, std::size_t end, Vec4& out) {
    for (std::size_t k = begin; k < end; ++k) {
      if (!s_.isName(k)) continue;
      const std::string& w = s_.at(k).text;
      std::string kind;
      std::size_t at;
      if (w == "color" || w == "colour") {
        kind = "rgb";
        at = k + 1;
        if (at < end && s_.isName(at) && sdl::isColorKeyword(s_.at(at).text)) kind = s_.at(at++).text;
      } else if (sdl::isColorKeyword(w)) {
        kind = w;
        at = k + 1;
      } else {
        continue;
      }
      s_.pos = at;
      out = colorOf(expr(), kind);
      return true;
    }
    return false;
  }

  Material finish(std::size_t begin, std::size_t end) {
    Material m;
    std::size_t k = begin;
    while (k < end) {
      if (s_.isSym(k, '{')) {  // nested block, e.g. reflection { ... }
        k = closing(k) + 1;
        continue;
      }
      if (!s_.isName(k)) {
        ++k;
        continue;
      }
      const std::string& w = s_.at(k).text;
      float* field = w == "ambient"      ? &m.ambient
                     : w == "diffuse"    ? &m.diffuse
                     : w == "specular"   ? &m.specular
                     : w == "roughness"  ? &m.roughness
                     : w == "brilliance" ? &m.brilliance
                     : w == "phong"      ? &m.phong
                     : w == "phong_size" ? &m.phongSize
                     : w == "reflection" ? &m.reflection
                     : w == "emission"   ? &m.emission
                                         : nullptr;
      if (field) {
        s_.pos = k + 1;
        const Val v = expr();
        *field = v.n > 0 ? static_cast<float>(v.v[0]) : 0.0f;
        k = s_.pos;
      } else if (w == "metallic") {
        // an optional amount; at or below 0 turns it off
        m.metallic = true;
        const std::size_t n = k + 1;
        if (n < end && (s_.at(n).kind == Kind::Number || s_.isSym(n, '-') || s_.isSym(n, '+'))) {
          s_.pos = n;
          const Val v = expr();
          m.metallic = (v.n > 0 ? static_cast<float>(v.v[0]) : 1.0f) > 0.0f;
          k = s_.pos;
        } else {
          k = n;
        }
      } else {
        Material preset;
        if (namedFinish(w, preset)) m = preset;  // later keywords still override
        ++k;
      }
    }
    return m;
  }

  // the first texture { } in [begin, end), or black without a finish
  Texture firstTexture(std::size_t begin, std::size_t end) {
    for (std::size_t k = begin; k < end; ++k)
      if (blockAt(k, "texture")) return textureBody(k + 2, closing(k + 1));
    Texture t;
    t.color = Vec4{0.0f, 0.0f, 0.0f, 1.0f};
    return t;
  }

  // ---- geometry ----
  void mesh2() {
    if (!s_.sym('{')) return;
    const std::size_t open = s_.pos, close = closing(open);
    std::size_t k = open + 1;
    while (k < close) {
      if (s_.isName(k) && s_.isSym(k + 1, '{')) {
        const std::size_t c = closing(k + 1);
        const std::string& w = s_.at(k).text;
        if (w == "vertex_vectors") vectorList(k + 2, c, verts_);
        else if (w == "normal_vectors") vectorList(k + 2, c, norms_);
        else if (w == "texture_list") textureList(k + 2, c);
        else if (w == "face_indices") faceList(k + 2, c);
        k = c + 1;  // uv_vectors, normal_indices, uv_indices: not used
      } else if (s_.isSym(k, '{')) {
        k = closing(k) + 1;
      } else {
        ++k;
      }
    }
    haveMesh_ = true;
    weldBlock();
    haveBlockMaterial_ = false;
    s_.pos = close + 1;
  }

  // sphere { <centre>, radius texture { ... } }; a texture named *_sl_tex
  // marks CueMol's silhouette joint dots (baked edges)
  void sphere() {
    if (!s_.sym('{')) return;
    const std::size_t open = s_.pos, close = closing(open);
    s_.pos = open + 1;
    const Val c = expr();
    if (s_.sym(',')) s_.next();
    const Val r = expr();
    Sphere sp;
    sp.center = vec3Of(c);
    sp.radius = static_cast<float>(r.at(0));
    const Texture t = firstTexture(s_.pos, close);
    sp.color = t.color;
    if (t.hasFinish) sp.material = t.finish;
    sp.group = static_cast<uint16_t>(group_);
    for (std::size_t k = open + 1; k < close; ++k) {
      const std::string& w = s_.at(k).text;
      if (s_.isName(k) && w.size() >= 7 && w.compare(w.size() - 7, 7, "_sl_tex") == 0) {
        sp.fromEdgeMacro = true;
        break;
      }
    }
    if (sp.radius > 0.0f) out_.spheres.push_back(sp);
    s_.pos = close + 1;
  }

  // cylinder { <p0>, <p1>, radius [open] texture { ... } }: capped unless
  // `open` precedes the first nested block
  void cylinder() {
    if (!s_.sym('{')) return;
    const std::size_t open = s_.pos, close = closing(open);
    s_.pos = open + 1;
    const Val a = expr();
    if (s_.sym(',')) s_.next();
    const Val b = expr();
    if (s_.sym(',')) s_.next();
    const Val r = expr();
    const std::size_t afterRadius = s_.pos;
    Cylinder cy;
    cy.p0 = vec3Of(a);
    cy.p1 = vec3Of(b);
    cy.radius = static_cast<float>(r.at(0));
    const Texture t = firstTexture(s_.pos, close);
    cy.color = t.color;
    if (t.hasFinish) cy.material = t.finish;
    cy.group = static_cast<uint16_t>(group_);
    cy.open = openKeyword(afterRadius, close);
    if (cy.radius > 0.0f) out_.cylinders.push_back(cy);
    s_.pos = close + 1;
  }
  bool openKeyword(std::size_t begin, std::size_t end) const {
    int depth = 0;
    for (std::size_t k = begin; k < end; ++k) {
      if (s_.isSym(k, '{')) {
        ++depth;
      } else if (s_.isSym(k, '}')) {
        if (depth > 0) --depth;
      } else if (depth == 0 && s_.isName(k)) {
        const std::string& w = s_.at(k).text;
        if (w == "open") return true;
        if (w == "texture" || w == "pigment" || w == "finish" || w == "normal" || w == "material") break;
      }
    }
    return false;
  }

  // edge_line(v1, n1, v2, n2, raise, w, tex, col) and
  // edge_line2(v1, n1, t1, v2, n2, t2, raise, w, tex, col): an open cylinder
  // from v1 + raise n1 to v2 + raise n2 of radius w and colour col;
  // edge_line2's transmits give the end opacities 1 - t (clamped to [0, 1])
  void edgeLine(bool two) {
    const std::vector<Val> a = s_.arguments(vars_, false);
    if (a.size() < (two ? 10u : 8u)) return;
    const std::size_t v1 = 0, n1 = 1, v2 = two ? 3 : 2, n2 = two ? 4 : 3, rs = two ? 6 : 4, w = two ? 7 : 5,
                      col = two ? 9 : 7;
    const float raise = static_cast<float>(a[rs].at(0));
    Cylinder cy;
    cy.p0 = vec3Of(a[v1]) + vec3Of(a[n1]) * raise;
    cy.p1 = vec3Of(a[v2]) + vec3Of(a[n2]) * raise;
    cy.radius = static_cast<float>(a[w].at(0));
    cy.color = colorOf(a[col], "rgb");
    if (two) {
      auto opacity = [](double t) { return std::min(1.0f, std::max(0.0f, 1.0f - static_cast<float>(t))); };
      cy.color.w = opacity(a[2].at(0));
      cy.opacity1 = opacity(a[5].at(0));
    }
    cy.group = static_cast<uint16_t>(group_);
    cy.open = true;
    cy.fromEdgeMacro = true;
    if (cy.radius > 0.0f) out_.cylinders.push_back(cy);
  }

  // ---- mesh2 lists ----
  float signedNumber() {
    float sign = 1.0f;
    for (; s_.sym('-') || s_.sym('+'); s_.next())
      if (s_.sym('-')) sign = -sign;
    if (!s_.number()) return 0.0f;
    const float v = static_cast<float>(s_.cur().number);
    s_.next();
    return sign * v;
  }
  // < a, b, c [, ...] > of literal numbers
  Vec3 literalVector() {
    float c[3] = {0.0f, 0.0f, 0.0f};
    if (!s_.sym('<')) return Vec3{};
    s_.next();
    for (int i = 0; i < 3; ++i) {
      c[i] = signedNumber();
      if (!s_.sym(',')) break;
      s_.next();
    }
    while (!s_.sym('>') && !s_.done()) s_.next();
    if (s_.sym('>')) s_.next();
    return Vec3{c[0], c[1], c[2]};
  }
  // [count ,] <v>, <v>, ...
  void vectorList(std::size_t begin, std::size_t end, std::vector<Vec3>& dst) {
    s_.pos = begin;
    if (s_.number()) {
      const std::size_t at = s_.pos;
      s_.next();
      if (s_.sym(',')) s_.next();
      else s_.pos = at;
    }
    while (s_.pos < end && !s_.done()) {
      if (s_.sym('<')) {
        dst.push_back(literalVector());
        if (s_.sym(',')) s_.next();
      } else if (s_.sym(',')) {
        s_.next();
      } else {
        break;
      }
    }
  }
  void textureList(std::size_t begin, std::size_t end) {
    std::size_t k = begin;
    if (k < end && s_.at(k).kind == Kind::Number) {
      ++k;
      if (k < end && s_.isSym(k, ',')) ++k;
    }
    while (k < end) {
      if (!blockAt(k, "texture")) {
        ++k;
        continue;
      }
      const std::size_t c = closing(k + 1);
      const Texture t = textureBody(k + 2, c);
      texColors_.push_back(t.color);
      adopt(t);
      k = c + 1;
      if (k < end && s_.isSym(k, ',')) ++k;
    }
  }
  // [count ,] <a, b, c> [, t | , ta, tb, tc], ...
  void faceList(std::size_t begin, std::size_t end) {
    s_.pos = begin;
    if (s_.number()) {
      s_.next();
      if (s_.sym(',')) s_.next();
    }
    while (s_.pos < end && !s_.done()) {
      if (s_.sym(',')) {
        s_.next();
        continue;
      }
      if (!s_.sym('<')) break;
      s_.next();
      Face f;
      for (int i = 0; i < 3; ++i) {
        f.v[i] = static_cast<int>(signedNumber());
        if (i < 2 && s_.sym(',')) s_.next();
      }
      while (!s_.sym('>') && !s_.done() && s_.pos < end) s_.next();
      if (s_.sym('>')) s_.next();
      std::vector<int> tex;
      while (s_.sym(',') && s_.pos < end) {
        s_.next();
        if (!s_.number()) break;
        tex.push_back(static_cast<int>(s_.cur().number));
        s_.next();
      }
      if (tex.size() == 1 || tex.size() >= 3) {
        for (int i = 0; i < 3; ++i) f.tex[i] = tex[tex.size() == 1 ? 0 : static_cast<std::size_t>(i)];
        f.hasTex = true;
      }
      faces_.push_back(f);
    }
  }

  // The open block's faces into the indexed mesh.  Corners share a render
  // vertex only when position, normal and colour match bit for bit (within
  // this block: a vertex stays in one transparency group), so hard edges and
  // colour seams keep their own vertices; positions also get a class id on
  // a 1e-4 grid across all blocks (the ribbon topology that face_indices do
  // not encode), numbered in first-seen corner order.  A block without
  // normals gets flat ones.  The block's material (its adopted finish, else
  // the default) and group are per triangle.
  void weldBlock() {
    const std::size_t nf = faces_.size();
    if (nf == 0) return;
    Mesh& m = out_.mesh;
    std::vector<Vec3> pos(nf * 3), nrm(nf * 3);
    std::vector<Vec4> col(nf * 3);
    for (std::size_t f = 0; f < nf; ++f) {
      for (int i = 0; i < 3; ++i) {
        const std::size_t c = f * 3 + static_cast<std::size_t>(i);
        const int vi = faces_[f].v[i];
        if (vi < 0 || static_cast<std::size_t>(vi) >= verts_.size())
          throw Mesh2ReadError("face vertex index out of range: " + std::to_string(vi));
        const std::size_t u = static_cast<std::size_t>(vi);
        pos[c] = verts_[u];
        nrm[c] = u < norms_.size() ? norms_[u] : Vec3{0.0f, 0.0f, 0.0f};
        col[c] = Vec4{1.0f, 1.0f, 1.0f, 1.0f};
        if (faces_[f].hasTex && !texColors_.empty()) {
          const int ti = std::min(std::max(faces_[f].tex[i], 0), static_cast<int>(texColors_.size()) - 1);
          col[c] = texColors_[static_cast<std::size_t>(ti)];
        }
      }
    }
    if (norms_.empty()) {
      for (std::size_t f = 0; f < nf; ++f) {
        const std::size_t c = f * 3;
        const Vec3 n = normalize(cross(pos[c + 1] - pos[c], pos[c + 2] - pos[c]));
        nrm[c] = nrm[c + 1] = nrm[c + 2] = n;
      }
    }
    std::unordered_map<CornerKey, uint32_t, CornerHash> vertexOf;
    vertexOf.reserve(nf * 3);
    for (std::size_t c = 0; c < nf * 3; ++c) {
      CornerKey key;
      const float f[10] = {pos[c].x, pos[c].y, pos[c].z, nrm[c].x, nrm[c].y, nrm[c].z,
                           col[c].x, col[c].y, col[c].z, col[c].w};
      std::memcpy(key.w, f, sizeof(key.w));
      auto ins = vertexOf.emplace(key, static_cast<uint32_t>(m.positions.size()));
      if (ins.second) {
        m.positions.push_back(pos[c]);
        m.normals.push_back(nrm[c]);
        m.colors.push_back(col[c]);
        const CellKey cell{std::lround(pos[c].x * kCellsPerUnit), std::lround(pos[c].y * kCellsPerUnit),
                           std::lround(pos[c].z * kCellsPerUnit)};
        auto cls = classOf_.emplace(cell, classCount_);
        if (cls.second) ++classCount_;
        m.posClass.push_back(cls.first->second);
      }
      m.index.push_back(ins.first->second);
    }
    m.posClassCount = classCount_;
    const uint8_t mat = static_cast<uint8_t>(blockMaterials_.size());
    blockMaterials_.push_back(haveBlockMaterial_ ? blockMaterial_ : Material{});
    m.triMaterialId.resize(m.triangleCount(), mat);
    m.triGroupId.resize(m.triangleCount(), static_cast<uint16_t>(group_));
    verts_.clear();
    norms_.clear();
    texColors_.clear();
    faces_.clear();
  }

  sdl::Stream s_;
  sdl::Vars vars_;
  std::map<std::string, Texture> textures_;
  // the open mesh2 block
  std::vector<Vec3> verts_, norms_;
  std::vector<Vec4> texColors_;
  std::vector<Face> faces_;
  Material blockMaterial_;
  bool haveBlockMaterial_ = false;
  bool haveMesh_ = false;
  std::vector<Material> blockMaterials_;
  std::unordered_map<CellKey, int32_t, CellHash> classOf_;
  int32_t classCount_ = 0;
  // transparency groups: [0] is the geometry outside any `#if (_show_*)`
  std::vector<std::string> groups_{std::string()};
  std::map<std::string, int> groupIndex_;
  int group_ = 0;
  std::vector<int> groupStack_;
  SceneGeometry out_;
};

}  // namespace

SceneGeometry readGeometryFromString(const std::string& text, const SymbolTable& seedSymbols) {
  return Mesh2Scan(sdl::lex(text), seedSymbols).read();
}

SceneGeometry readGeometryFromFile(const std::string& path, const SymbolTable& seedSymbols) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Mesh2ReadError("cannot open file: " + path);
  std::ostringstream ss;
  ss << f.rdbuf();
  return readGeometryFromString(ss.str(), seedSymbols);
}

Mesh readMesh2FromString(const std::string& text) { return readGeometryFromString(text).mesh; }

Mesh readMesh2FromFile(const std::string& path) { return readGeometryFromFile(path).mesh; }

}  // namespace umbreon

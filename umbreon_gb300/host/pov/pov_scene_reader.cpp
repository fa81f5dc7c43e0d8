// pov_scene_reader.cpp -- the viewing setup of a CueMol .pov scene
// (pov/pov_scene_reader.hpp).  One pass over the token stream: directives
// are evaluated on a conditional stack, statements in an active scope are
// dispatched by keyword.  Behaviour follows the reference reader
// (src/bench/pov/pov_scene_reader.cpp): the camera model (:464-490), the
// colour and fog blocks (:493-588), CueMol's two lighting macros
// (:590-640) and the restoration of CueMol's OpenGL linear fog from its POV
// ground fog (:71-88).
#include "pov/pov_scene_reader.hpp"

#include <cmath>
#include <fstream>
#include <sstream>
#include <utility>

#include "sdl.hpp"

namespace umbreon {
namespace {

using sdl::Kind;
using sdl::Val;

Vec3 vec3Of(const Val& v) {
  return Vec3{static_cast<float>(v.at(0)), static_cast<float>(v.at(1)), static_cast<float>(v.at(2))};
}

class PovScene {
 public:
  PovScene(std::vector<sdl::Tok> toks, const PovParseOptions& opt) : s_(std::move(toks)) {
    vars_["image_width"] = Val::scalar(opt.imageWidth);
    vars_["image_height"] = Val::scalar(opt.imageHeight);
    for (const auto& kv : opt.predefined) vars_[kv.first] = Val::scalar(kv.second);
  }

  PovSceneResult read() {
    while (!s_.done()) {
      if (cam_.open && s_.pos >= cam_.end) {
        finishCamera();
        s_.next();  // the camera's '}'
      } else if (s_.sym('#')) {
        s_.next();
        directive();
      } else if (active() && s_.name()) {
        statement();
      } else {
        s_.next();
      }
    }
    if (res_.fog.enabled) restoreLinearFog();
    for (const auto& kv : vars_) {
      const Val& v = kv.second;
      res_.declares.emplace(kv.first, std::vector<double>(v.v, v.v + (v.n > 1 ? v.n : 1)));
    }
    res_.radiosity = vars_.count("_radiosity") > 0;
    return std::move(res_);
  }

 private:
  struct Frame {
    bool enclosing, cond, inElse;
  };
  struct CameraBlock {
    bool open = false;
    std::size_t end = 0;
    bool ortho = false;
    bool hasUp = false, hasRight = false, hasLocation = false, hasLookAt = false, hasAngle = false;
    Val direction, up, right, location, lookAt;
    double angle = 0.0;
  };

  bool active() const {
    if (stack_.empty()) return true;
    const Frame& f = stack_.back();
    return f.enclosing && (f.inElse ? !f.cond : f.cond);
  }
  Val expr() { return s_.expr(vars_, true); }
  Val parenthesised() {
    if (!s_.sym('(')) return expr();
    s_.next();
    Val v = expr();
    if (s_.sym(')')) s_.next();
    return v;
  }
  std::size_t closing(std::size_t open) const {
    const std::size_t c = s_.closing(open);
    if (c == std::string::npos) throw PovSceneError("unbalanced '{' near line " + std::to_string(s_.at(open).line));
    return c;
  }
  double scalarVar(const char* name, double dflt) const {
    const auto it = vars_.find(name);
    return it != vars_.end() ? it->second.at(0) : dflt;
  }

  // ---- directives (cursor on the word after '#') ----
  void directive() {
    if (!s_.name()) return;
    const std::string d = s_.cur().text;
    if (d == "macro") {
      s_.skipMacro();
    } else if (d == "declare" || d == "local") {
      s_.next();
      declare();
    } else if (d == "ifdef" || d == "ifndef") {
      s_.next();
      std::string id;
      if (s_.sym('(')) s_.next();
      if (s_.name()) {
        id = s_.cur().text;
        s_.next();
      }
      if (s_.sym(')')) s_.next();
      const bool defined = vars_.count(id) > 0;
      stack_.push_back(Frame{active(), d == "ifdef" ? defined : !defined, false});
    } else if (d == "if" || d == "while" || d == "switch") {
      s_.next();
      const bool c = parenthesised().at(0) != 0.0;
      stack_.push_back(Frame{active(), c, false});
    } else if (d == "else" || d == "elseif") {
      if (!stack_.empty()) stack_.back().inElse = true;
      s_.next();
      if (d == "elseif" && s_.sym('(')) parenthesised();
    } else if (d == "end" || d == "break") {
      if (d == "end" && !stack_.empty()) stack_.pop_back();
      s_.next();
    } else if (d == "version") {
      s_.next();
      s_.skipStatement();
    } else if (d == "include") {
      s_.next();
      if (s_.cur().kind == Kind::Text) s_.next();
    } else {
      s_.next();
    }
  }

  void declare() {
    if (!s_.name()) return;
    const std::string id = s_.cur().text;
    s_.next();
    if (!s_.sym('=')) return;
    s_.next();
    if (s_.sym('#')) {  // #declare _scene = #include "geometry.inc"
      s_.next();
      if (s_.name() && s_.cur().text == "include") {
        s_.next();
        if (s_.cur().kind == Kind::Text) {
          if (active() && id == "_scene") res_.includePath = s_.cur().text;
          s_.next();
        }
      }
      return;
    }
    if (s_.name()) {
      const std::string& w = s_.cur().text;
      if (w == "texture" || w == "pigment" || w == "finish" || w == "normal" || w == "material") {
        s_.next();
        if (s_.sym('{')) s_.pos = closing(s_.pos) + 1;
        return;
      }
    }
    const Val v = expr();
    if (active() && v.n > 0) vars_[id] = v;
    s_.skipStatement();
  }

  // ---- statements in an active scope (cursor on the keyword) ----
  void statement() {
    const std::string w = s_.cur().text;
    if (cam_.open) {
      cameraKeyword(w);
      return;
    }
    s_.next();
    if (w == "camera") {
      if (s_.sym('{')) {
        cam_ = CameraBlock{};
        cam_.open = true;
        cam_.end = closing(s_.pos);
        cam_.direction.n = 3;
        cam_.direction.v[2] = -1.0;
        s_.next();
      }
    } else if (w == "background") {
      background();
    } else if (w == "SpecLighting") {
      specLighting(s_.arguments(vars_, true));
    } else if (w == "FlashLighting") {
      flashLighting(s_.arguments(vars_, true));
    } else if (w == "fog") {
      fog();
    } else if (w == "global_settings") {
      globalSettings();
    } else if (s_.sym('{')) {
      s_.pos = closing(s_.pos) + 1;  // any other block
    } else if (s_.sym('(')) {
      s_.skipParens();
    }
  }

  void cameraKeyword(const std::string& w) {
    s_.next();
    if (w == "orthographic") cam_.ortho = true;  // (`perspective` is the default)
    else if (w == "direction") cam_.direction = expr();
    else if (w == "up") cam_.up = expr(), cam_.hasUp = true;
    else if (w == "right") cam_.right = expr(), cam_.hasRight = true;
    else if (w == "location") cam_.location = expr(), cam_.hasLocation = true;
    else if (w == "look_at") cam_.lookAt = expr(), cam_.hasLookAt = true;
    else if (w == "angle") cam_.angle = expr().at(0), cam_.hasAngle = true;
    else if (w == "sky") expr();
  }

  // POV camera -> umbreon Camera: view direction toward look_at (else the
  // direction vector), up normalised; orthographic height = |up|;
  // perspective: `angle` is the horizontal field of view of the `right`
  // vector, the vertical one follows from |up| / |right|.
  void finishCamera() {
    cam_.open = false;
    Camera& c = res_.camera;
    const Vec3 loc = cam_.hasLocation ? vec3Of(cam_.location) : Vec3{0.0f, 0.0f, 1.0f};
    c.position = loc;
    c.direction = cam_.hasLookAt ? normalize(vec3Of(cam_.lookAt) - loc) : normalize(vec3Of(cam_.direction));
    c.up = cam_.hasUp ? normalize(vec3Of(cam_.up)) : Vec3{0.0f, 1.0f, 0.0f};
    if (cam_.ortho) {
      c.orthographic = true;
      c.height = cam_.hasUp ? length(vec3Of(cam_.up)) : 1.0f;
      return;
    }
    c.orthographic = false;
    const double rightLen = cam_.hasRight ? length(vec3Of(cam_.right)) : 1.0;
    const double upLen = cam_.hasUp ? length(vec3Of(cam_.up)) : 1.0;
    const float halfX = radians(static_cast<float>(cam_.hasAngle ? cam_.angle : 40.0)) * 0.5f;
    const float halfY = static_cast<float>(std::atan(std::tan(halfX) * (upLen / rightLen)));
    c.fovy = degrees(2.0f * halfY);
  }

  // first colour of a block [open, close): `color [kw] expr`, or `kw expr`
  bool colorIn(std::size_t open, std::size_t close, Vec3& out) {
    for (std::size_t k = open + 1; k < close; ++k) {
      if (!s_.isName(k)) continue;
      const std::string& w = s_.at(k).text;
      std::size_t at;
      if (w == "color" || w == "colour") {
        at = k + 1;
        if (at < close && s_.isName(at) && sdl::isColorKeyword(s_.at(at).text)) ++at;
      } else if (sdl::isColorKeyword(w)) {
        at = k + 1;
      } else {
        continue;
      }
      s_.pos = at;
      out = vec3Of(expr());
      return true;
    }
    return false;
  }

  void background() {
    if (!s_.sym('{')) return;
    const std::size_t open = s_.pos, close = closing(open);
    colorIn(open, close, res_.background);
    s_.pos = close + 1;
  }

  void globalSettings() {
    if (!s_.sym('{')) return;
    const std::size_t open = s_.pos, close = closing(open);
    for (std::size_t k = open + 1; k < close; ++k) {
      if (s_.isName(k) && s_.at(k).text == "assumed_gamma") {
        s_.pos = k + 1;
        res_.assumedGamma = static_cast<float>(expr().at(0));
        break;
      }
    }
    s_.pos = close + 1;
  }

  void fog() {
    if (!s_.sym('{')) return;
    const std::size_t open = s_.pos, close = closing(open);
    Fog& f = res_.fog;
    f.enabled = true;
    s_.pos = open + 1;
    while (s_.pos < close && !s_.done()) {
      if (!s_.name()) {
        s_.next();
        continue;
      }
      const std::string w = s_.cur().text;
      s_.next();
      if (w == "distance") {
        f.distance = static_cast<float>(expr().at(0));
      } else if (w == "fog_type") {
        f.type = static_cast<int>(expr().at(0));
      } else if (w == "fog_offset") {
        f.offset = static_cast<float>(expr().at(0));
      } else if (w == "fog_alt") {
        f.alt = static_cast<float>(expr().at(0));
      } else if (w == "up") {
        f.up = vec3Of(expr());
      } else if (w == "color" || w == "colour") {
        if (s_.name() && sdl::isColorKeyword(s_.cur().text)) s_.next();
        f.color = vec3Of(expr());
      } else if (sdl::isColorKeyword(w)) {
        f.color = vec3Of(expr());
      }
    }
    s_.pos = close + 1;
  }

  // SpecLighting(spread, distance, intensity, shadow): CueMol's key light at
  // vnormalize(<1,1,1>) * distance * 2 aimed at the origin, a distant light
  // along -<1,1,1>.  It casts highlights unless it is the shadowless
  // parallel form (spread <= 1 and shadow == 0); spread > 1 is an area light
  // of angular half-radius atan(spread / 40) (side distance * spread / 10 at
  // distance 2 * distance).
  void specLighting(const std::vector<Val>& a) {
    if (a.size() < 3) return;
    DistantLight L;
    L.direction = normalize(Vec3{0.0f, 0.0f, 0.0f} - normalize(Vec3{1.0f, 1.0f, 1.0f}));
    L.color = Vec3{1.0f, 1.0f, 1.0f};
    L.intensity = static_cast<float>(a[2].at(0));
    const double spread = a[0].at(0);
    const double shadow = a.size() > 3 ? a[3].at(0) : 0.0;
    L.castsHighlight = spread > 1.0 || shadow != 0.0;
    if (spread > 1.0) L.angularRadius = static_cast<float>(std::atan(spread / 40.0));
    res_.lights.push_back(L);
  }

  // FlashLighting(intensity): a shadowless head light at the eye
  // (<_stereo * _distance * _iod, 0, _distance>) aimed at the origin: a fill
  // light (diffuse only) along origin - eye.
  void flashLighting(const std::vector<Val>& a) {
    if (a.empty()) return;
    const double stereo = scalarVar("_stereo", 0.0), dist = scalarVar("_distance", 200.0),
                 iod = scalarVar("_iod", 0.03);
    const Vec3 eye{static_cast<float>(stereo * dist * iod), 0.0f, static_cast<float>(dist)};
    DistantLight L;
    L.direction = normalize(Vec3{0.0f, 0.0f, 0.0f} - eye);
    L.color = Vec3{1.0f, 1.0f, 1.0f};
    L.intensity = static_cast<float>(a[0].at(0));
    L.castsHighlight = false;
    res_.lights.push_back(L);
  }

  // CueMol writes POV fog `distance` = slab depth / 3 for an OpenGL linear
  // fog from the view distance over half the slab: start = _distance (else
  // |look_at - location|, else 200), at least 1; end = start + 1.5 distance.
  void restoreLinearFog() {
    double dist;
    const auto it = vars_.find("_distance");
    if (it != vars_.end()) dist = it->second.at(0);
    else if (cam_.hasLocation && cam_.hasLookAt) dist = length(vec3Of(cam_.lookAt) - vec3Of(cam_.location));
    else dist = 200.0;
    if (dist < 1.0) dist = 1.0;
    res_.fog.start = static_cast<float>(dist);
    res_.fog.end = static_cast<float>(dist + 1.5 * res_.fog.distance);
  }

  sdl::Stream s_;
  sdl::Vars vars_;
  std::vector<Frame> stack_;
  CameraBlock cam_;
  PovSceneResult res_;
};

}  // namespace

PovSceneResult readPovSceneFromString(const std::string& text, const PovParseOptions& opt) {
  return PovScene(sdl::lex(text), opt).read();
}

PovSceneResult readPovScene(const std::string& path, const PovParseOptions& opt) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw PovSceneError("cannot open file: " + path);
  std::ostringstream ss;
  ss << f.rdbuf();
  return readPovSceneFromString(ss.str(), opt);
}

}  // namespace umbreon

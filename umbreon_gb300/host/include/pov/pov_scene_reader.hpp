// Reader of the viewing setup in a CueMol POV-Ray scene file (.pov).
// Declarations match umbreon's src/bench/pov/pov_scene_reader.hpp (same
// names, fields and defaults) so a caller of the reference reader compiles
// unchanged; the implementation (pov/pov_scene_reader.cpp) is this
// library's.
//
// Recovered: the camera (orthographic / perspective), the two lights of
// CueMol's SpecLighting / FlashLighting macros, the background colour, the
// fog block, global_settings' assumed_gamma, every scalar / vector #declare
// (to seed the geometry reader) and the .inc named by
// `#declare _scene = #include "..."`.  #if / #ifdef / #ifndef / #else / #end
// are evaluated; macro definitions and all other blocks are skipped.
#pragma once

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "scene.hpp"

namespace umbreon {
// Resolved scalar/vector constants (name -> components).
using PovSymbols = std::map<std::string, std::vector<double>>;
}  // namespace umbreon

namespace umbreon {

// Thrown when the input cannot be read as a CueMol .pov scene.
struct PovSceneError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct PovParseOptions {
  int imageWidth = 300;
  int imageHeight = 300;
  // Constants predefined on the command line (POV "Declare=name=value"),
  // seeded before the file is read.
  std::map<std::string, double> predefined;
};

struct PovSceneResult {
  Camera camera;
  std::vector<DistantLight> lights;
  Vec3 background{0.0f, 0.0f, 0.0f};
  Fog fog;
  float assumedGamma = 1.0f;
  PovSymbols declares;
  std::string includePath;
  bool radiosity = false;
};

PovSceneResult readPovSceneFromString(const std::string& text, const PovParseOptions& opt);
PovSceneResult readPovScene(const std::string& path, const PovParseOptions& opt);

}  // namespace umbreon

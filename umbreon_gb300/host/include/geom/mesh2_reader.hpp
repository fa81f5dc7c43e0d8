// Reader of the geometry in a CueMol POV-Ray include file (.inc).
// Declarations match umbreon's src/bench/geom/mesh2_reader.hpp (same names,
// fields and defaults) so a caller of the reference reader compiles
// unchanged; the implementation (pov/mesh2_reader.cpp) is this library's.
//
// Recovered: every mesh2 block (merged into one indexed Mesh with per-block
// materials and transparency groups), sphere { } primitives, cylinder { }
// primitives and CueMol's edge_line / edge_line2 macro calls (cylinders);
// groups come from the `#if (_show_<id>)` wrappers CueMol writes around each
// rendering object.
#pragma once

#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "scene.hpp"

namespace umbreon {

// Thrown when the input cannot be read as CueMol geometry.
struct Mesh2ReadError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

struct SceneGeometry {
  Mesh mesh;
  std::vector<Sphere> spheres;
  std::vector<Cylinder> cylinders;
  // group index -> CueMol section id ("" for group 0, geometry outside any
  // `#if (_show_*)` block)
  std::vector<std::string> groupNames;
};

// Scalar/vector constants the .pov declares before including the geometry.
using SymbolTable = std::map<std::string, std::vector<double>>;

SceneGeometry readGeometryFromString(const std::string& text, const SymbolTable& seedSymbols = {});
SceneGeometry readGeometryFromFile(const std::string& path, const SymbolTable& seedSymbols = {});

// The merged mesh alone.
Mesh readMesh2FromString(const std::string& text);
Mesh readMesh2FromFile(const std::string& path);

}  // namespace umbreon

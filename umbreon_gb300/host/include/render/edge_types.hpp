// Edge option types of the umbreon API.  The stroke / object-space edge
// passes are not part of this library; the types exist so RenderOptions and
// Scene keep their shape, and render() rejects a request that enables them.
#pragma once

#include <cstdint>

namespace umbreon {

enum class EdgeClass : uint8_t { Silhouette = 0, Disconnected = 1, Object = 2, Material = 3, Crease = 4, Count = 5 };

struct EdgeClassStyle {
  bool enabled = false;
  float color[3] = {0.0f, 0.0f, 0.0f};
  float opacity = 1.0f;
  float width = 2.0f;
};

enum class SilhouetteMode : uint8_t { Full = 0, Outline = 1 };
enum class StrokeAlign : uint8_t { Center = 0, Outside = 1 };

struct EdgeStyle {
  EdgeClassStyle cls[static_cast<int>(EdgeClass::Count)];
  SilhouetteMode silhouetteMode = SilhouetteMode::Full;
  StrokeAlign align = StrokeAlign::Outside;
};

struct StrokeEdgeOptions {
  bool enable = false;
  float screenDepthGapPx = 12.0f;
  float screenSlopeClampPx = 300.0f;
  float screenSimplifyPx = 0.4f;
  int screenSmoothIters = 2;
  float screenMinLenPx = 4.0f;
  int screenClassMergeLen = 2;
  float screenGrazeK = 1.0f;
  bool silhouette = true;
  bool crease = false;
  bool border = true;
  bool contact = false;
  float raise = 0.0f;
  bool analytic = true;
  int analyticSegments = 48;
  float meshHardEdgeDeg = 40.0f;
  float creaseAngleDeg = 30.0f;
  float meshCreaseSmoothVetoDeg = 35.0f;
  bool meshCreaseConvexOnly = true;
  float meshBorderCoplanarVetoDeg = 35.0f;
  int meshCreaseMaxDegree = 4;
  bool meshGeomSilhouette = false;
  bool rejectConcaveEdges = true;
  int selfExcludeRings = 6;
  int thickness = 2;
  int resampleStepPx = 2;
  float color[3] = {0.0f, 0.0f, 0.0f};
  float opacity = 1.0f;
  bool taper = false;
  bool smooth = false;
  bool roundCap = false;
  bool roundJoin = false;
  StrokeAlign align = StrokeAlign::Outside;
  bool edgesOnly = false;
  EdgeStyle defaultStyle;
  bool debugQiDots = false;
  bool debugNodeDots = false;
  bool debugQiVertexDots = false;
  float debugQiVertexDelta = 0.0f;
  float qiNormalLift = 0.0f;
  bool qiSplit = false;
};

struct ObjectSpaceEdgeOptions {
  bool enable = false;
  float width = 0.03f;
  float raise = 0.0f;
  int segments = 48;
  float color[3] = {0.0f, 0.0f, 0.0f};
  bool clip = true;
  bool meshSilhouette = true;
  bool meshCrease = true;
  bool meshBorder = true;
  bool visibilityClip = false;
  float meshHardEdgeDeg = 40.0f;
  float creaseAngleDeg = 30.0f;
  float meshCreaseSmoothVetoDeg = 0.0f;
  bool meshCreaseConvexOnly = false;
  float meshBorderCoplanarVetoDeg = 0.0f;
  int meshCreaseMaxDegree = 0;
};

}  // namespace umbreon

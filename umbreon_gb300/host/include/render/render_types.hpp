// Umbrella header for the render option / result / progress types.
#pragma once

#include "render/edge_types.hpp"
#include "render/frame_result.hpp"
#include "render/render_options.hpp"
#include "render/render_progress.hpp"

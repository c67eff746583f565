// bd_surface.h -- host side of the surface panels: the derived geometry of a
// panel and the coarse grid of panel lists the step kernels walk.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gpusmoldyn.h"
#include "bd_layout.h"

namespace bd {

// Checks a panel as given and derives the geometry a step uses (unit
// normals, squared radius, rectangle bounds).  BD_ERR_INVALID_ARGUMENT with
// a message for a malformed panel.
bd_status derive_panel(const bd_panel& in, int surface, bd_panel_info* out, std::string* msg);

// Panel lists over a grid of at most 32 boxes per axis spanning [lo, hi]:
// every panel is listed in each box its bounding box (padded by 1e-3 of a
// box edge) touches, so the panels a segment can cross are among those
// listed in the boxes its own bounding box touches.
struct PanelGrid {
  float lo[3], inv[3];
  uint32_t dims[3];
  std::vector<uint32_t> start;  // [n_boxes + 1]
  std::vector<uint32_t> list;
};
void build_panel_grid(const std::vector<bd_panel_info>& panels, const float lo[3], const float hi[3], PanelGrid* g);

}  // namespace bd

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

// Panel lists over a grid of at most 32 boxes per axis spanning [lo, hi]
// (the edge boxes extend to infinity): every panel is listed in each box,
// grown by 1e-3 of a box edge, that its bounding box touches and that the
// panel itself can pass through (spheres and hemispheres by their surface,
// cylinders not in boxes they contain, triangles by their plane), so the
// panels a segment can cross are among those listed in the boxes its own
// bounding box touches.
struct PanelGrid {
  float lo[3], inv[3];
  uint32_t dims[3];
  std::vector<uint32_t> start;  // [n_boxes + 1]
  std::vector<uint32_t> list;
};
void build_panel_grid(const std::vector<bd_panel_info>& panels, const float lo[3], const float hi[3], PanelGrid* g);

// Species bit of the per-cell masks: species s < 7 has bit s, every species
// from 7 on shares bit 7.
inline uint32_t species_bit(int s) { return s < 7 ? (uint32_t)s : 7u; }

// Per-cell species masks of one instance's uniform grid (dims cells of edge
// `cell` from lo): bit species_bit(s) of cell c is set when some panel that
// a step of species s may meet (panel_species[id], same bits: s itself or a
// product of its first-order reactions sees it) passes within `reach` of
// the cell.  A molecule whose step starts in a cell without its bit can meet
// no panel it sees on that step, nor with the products it places at the
// step's end, when `reach` bounds how far both go from the start.
void build_cell_masks(const std::vector<bd_panel_info>& panels, const std::vector<uint8_t>& panel_species,
                      const PanelGrid& g, const float lo[3], const float cell[3], const uint32_t dims[3],
                      double reach, uint8_t* out);

}  // namespace bd

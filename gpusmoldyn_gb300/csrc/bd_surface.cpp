// bd_surface.cpp -- surface panels on the host: checks, derived geometry and
// the coarse grid of panel lists (the reference's draft keeps a per-cell
// panel range, getSurfaceGridIndex in particles_kernel.cu:426-431, but never
// builds it).
#include "bd_surface.h"

#include <math.h>

#include <algorithm>
#include <cmath>
#include <thread>

namespace bd {

namespace {

bool finite_all(const float* p, int n) {
  for (int k = 0; k < n; k++)
    if (!std::isfinite(p[k])) return false;
  return true;
}

// Unit vector of (x, y, z) in float, computed in double; false for zero.
bool unit(double x, double y, double z, float out[3], double* norm = nullptr) {
  const double L = std::sqrt(x * x + y * y + z * z);
  if (!(L > 0.0) || !std::isfinite(L)) return false;
  out[0] = (float)(x / L);
  out[1] = (float)(y / L);
  out[2] = (float)(z / L);
  if (norm) *norm = L;
  return true;
}

bd_status bad(std::string* msg, const char* why) {
  if (msg) *msg = why;
  return BD_ERR_INVALID_ARGUMENT;
}

}  // namespace

bd_status derive_panel(const bd_panel& in, int surface, bd_panel_info* out, std::string* msg) {
  bd_panel_info P{};
  P.shape = in.shape;
  P.surface = surface;
  P.front = 1.0f;
  const float* p = in.p;
  const bool sided = in.shape == BD_PANEL_RECT || in.shape == BD_PANEL_SPH || in.shape == BD_PANEL_CYL ||
                     in.shape == BD_PANEL_HEMI;
  if (sided) {
    if (in.front != 1 && in.front != -1) return bad(msg, "panel front must be +1 or -1");
    P.front = (float)in.front;
  }
  switch (in.shape) {
    case BD_PANEL_RECT: {
      if (!finite_all(p, 5)) return bad(msg, "rect: non-finite parameter");
      if (in.axis < 0 || in.axis > 2) return bad(msg, "rect: axis must be 0, 1 or 2");
      if (p[3] == 0.0f || p[4] == 0.0f) return bad(msg, "rect: zero side");
      P.axis = in.axis;
      for (int k = 0; k < 3; k++) P.a[k] = p[k];
      const int u = in.axis == 0 ? 1 : 0, v = in.axis == 2 ? 1 : 2;
      const float eu = p[u] + p[3], ev = p[v] + p[4];
      P.bounds[0] = std::min(p[u], eu);
      P.bounds[1] = std::max(p[u], eu);
      P.bounds[2] = std::min(p[v], ev);
      P.bounds[3] = std::max(p[v], ev);
      break;
    }
    case BD_PANEL_TRI: {
      if (!finite_all(p, 9)) return bad(msg, "tri: non-finite parameter");
      const double e1[3] = {(double)p[3] - p[0], (double)p[4] - p[1], (double)p[5] - p[2]};
      const double e2[3] = {(double)p[6] - p[0], (double)p[7] - p[1], (double)p[8] - p[2]};
      const double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2],
                           e1[0] * e2[1] - e1[1] * e2[0]};
      if (!unit(c[0], c[1], c[2], P.n)) return bad(msg, "tri: degenerate triangle");
      for (int k = 0; k < 3; k++) {
        P.a[k] = p[k];
        P.v1[k] = p[3 + k];
        P.v2[k] = p[6 + k];
      }
      break;
    }
    case BD_PANEL_SPH:
    case BD_PANEL_HEMI:
    case BD_PANEL_DISK: {
      const int np = in.shape == BD_PANEL_SPH ? 4 : 7;
      if (!finite_all(p, np)) return bad(msg, "panel: non-finite parameter");
      if (!(p[3] > 0.0f)) return bad(msg, "panel: radius must be positive");
      for (int k = 0; k < 3; k++) P.a[k] = p[k];
      P.r = p[3];
      P.r2 = p[3] * p[3];
      if (in.shape != BD_PANEL_SPH && !unit(p[4], p[5], p[6], P.n)) return bad(msg, "panel: zero direction vector");
      break;
    }
    case BD_PANEL_CYL: {
      if (!finite_all(p, 7)) return bad(msg, "cyl: non-finite parameter");
      if (!(p[6] > 0.0f)) return bad(msg, "cyl: radius must be positive");
      double L = 0.0;
      if (!unit((double)p[3] - p[0], (double)p[4] - p[1], (double)p[5] - p[2], P.n, &L))
        return bad(msg, "cyl: the two ends coincide");
      for (int k = 0; k < 3; k++) P.a[k] = p[k];
      P.len = (float)L;
      P.r = p[6];
      P.r2 = p[6] * p[6];
      break;
    }
    default:
      return bad(msg, "unknown panel shape");
  }
  *out = P;
  return BD_OK;
}

namespace {

// Bounding box of one panel in double.
void panel_aabb(const bd_panel_info& P, double lo[3], double hi[3]) {
  switch (P.shape) {
    case BD_PANEL_RECT: {
      const int u = P.axis == 0 ? 1 : 0, v = P.axis == 2 ? 1 : 2;
      lo[P.axis] = hi[P.axis] = P.a[P.axis];
      lo[u] = P.bounds[0];
      hi[u] = P.bounds[1];
      lo[v] = P.bounds[2];
      hi[v] = P.bounds[3];
      return;
    }
    case BD_PANEL_TRI:
      for (int k = 0; k < 3; k++) {
        lo[k] = std::min({(double)P.a[k], (double)P.v1[k], (double)P.v2[k]});
        hi[k] = std::max({(double)P.a[k], (double)P.v1[k], (double)P.v2[k]});
      }
      return;
    case BD_PANEL_CYL:
      for (int k = 0; k < 3; k++) {
        const double e = (double)P.a[k] + (double)P.n[k] * P.len;
        lo[k] = std::min((double)P.a[k], e) - P.r;
        hi[k] = std::max((double)P.a[k], e) + P.r;
      }
      return;
    default:  // sphere, hemisphere, disk
      for (int k = 0; k < 3; k++) {
        lo[k] = (double)P.a[k] - P.r;
        hi[k] = (double)P.a[k] + P.r;
      }
  }
}

// False when the panel cannot pass through the box [lo, hi] grown by pad:
// a sphere or hemisphere whose surface misses it (box inside, or wholly
// outside, the sphere), a cylinder that contains the box, a triangle whose
// plane leaves every corner on one side.  Panels are kept in doubt.
bool panel_meets_box(const bd_panel_info& P, const double lo[3], const double hi[3], double pad) {
  double c[8][3];
  for (int k = 0; k < 8; k++)
    for (int a = 0; a < 3; a++) c[k][a] = ((k >> a) & 1) ? hi[a] + pad : lo[a] - pad;
  switch (P.shape) {
    case BD_PANEL_SPH:
    case BD_PANEL_HEMI: {
      double near2 = 0.0, far2 = 0.0;
      for (int a = 0; a < 3; a++) {
        const double l = lo[a] - pad - P.a[a], h = hi[a] + pad - P.a[a];
        const double n = l > 0 ? l : (h < 0 ? -h : 0.0);
        near2 += n * n;
        far2 += std::max(l * l, h * h);
      }
      const double r = P.r;
      return near2 <= r * r && far2 >= r * r;
    }
    case BD_PANEL_CYL: {
      for (int k = 0; k < 8; k++) {
        double w[3], t = 0.0, q = 0.0;
        for (int a = 0; a < 3; a++) {
          w[a] = c[k][a] - P.a[a];
          t += w[a] * P.n[a];
        }
        for (int a = 0; a < 3; a++) {
          const double d = w[a] - t * P.n[a];
          q += d * d;
        }
        if (q >= (double)P.r * P.r) return true;  // a corner outside the infinite cylinder
      }
      return false;
    }
    case BD_PANEL_TRI: {
      bool pos = false, neg = false;
      for (int k = 0; k < 8; k++) {
        double s = 0.0;
        for (int a = 0; a < 3; a++) s += (c[k][a] - P.a[a]) * P.n[a];
        pos |= s >= 0.0;
        neg |= s <= 0.0;
      }
      return pos && neg;
    }
    default:
      return true;
  }
}

}  // namespace

void build_panel_grid(const std::vector<bd_panel_info>& panels, const float lo[3], const float hi[3], PanelGrid* g) {
  double ext[3], emax = 0.0;
  for (int k = 0; k < 3; k++) {
    ext[k] = std::max((double)hi[k] - lo[k], 1e-30);
    emax = std::max(emax, ext[k]);
  }
  // about 8 boxes per panel, at most 32 per axis
  const double per_axis = std::ceil(std::cbrt(8.0 * (double)std::max<size_t>(panels.size(), 1)));
  for (int k = 0; k < 3; k++) {
    const double n = std::ceil(per_axis * ext[k] / emax);
    g->dims[k] = (uint32_t)std::min(32.0, std::max(1.0, n));
    g->lo[k] = lo[k];
    g->inv[k] = (float)(g->dims[k] / ext[k]);
  }
  const uint32_t nb = g->dims[0] * g->dims[1] * g->dims[2];
  std::vector<std::vector<uint32_t>> boxes(nb);
  for (size_t id = 0; id < panels.size(); id++) {
    double a[3], b[3];
    panel_aabb(panels[id], a, b);
    int r0[3], r1[3];
    double edge[3], pad_all = 0.0;
    for (int k = 0; k < 3; k++) {
      edge[k] = ext[k] / g->dims[k];
      const double pad = 1e-3 * edge[k] + 1e-6 * (std::fabs(a[k]) + std::fabs(b[k]) + 1.0);
      pad_all = std::max(pad_all, pad);
      const double f0 = std::floor((a[k] - pad - lo[k]) / edge[k]), f1 = std::floor((b[k] + pad - lo[k]) / edge[k]);
      r0[k] = (int)std::min<double>(std::max<double>(f0, 0.0), g->dims[k] - 1.0);
      r1[k] = (int)std::min<double>(std::max<double>(f1, 0.0), g->dims[k] - 1.0);
    }
    for (int z = r0[2]; z <= r1[2]; z++)
      for (int y = r0[1]; y <= r1[1]; y++)
        for (int x = r0[0]; x <= r1[0]; x++) {
          // the edge boxes take every position beyond the grid as well
          const int i3[3] = {x, y, z};
          double blo[3], bhi[3];
          for (int k = 0; k < 3; k++) {
            blo[k] = i3[k] == 0 ? -1e30 : lo[k] + i3[k] * edge[k];
            bhi[k] = i3[k] == (int)g->dims[k] - 1 ? 1e30 : lo[k] + (i3[k] + 1) * edge[k];
          }
          if (!panel_meets_box(panels[id], blo, bhi, pad_all)) continue;
          boxes[((uint32_t)z * g->dims[1] + (uint32_t)y) * g->dims[0] + (uint32_t)x].push_back((uint32_t)id);
        }
  }
  g->start.assign(nb + 1, 0);
  g->list.clear();
  for (uint32_t b = 0; b < nb; b++) {
    g->start[b] = (uint32_t)g->list.size();
    g->list.insert(g->list.end(), boxes[b].begin(), boxes[b].end());
  }
  g->start[nb] = (uint32_t)g->list.size();
}

void build_cell_masks(const std::vector<bd_panel_info>& panels, const std::vector<uint8_t>& panel_species,
                      const PanelGrid& g, const float lo[3], const float cell[3], const uint32_t dims[3],
                      double reach, uint8_t* out) {
  std::vector<double> plo(panels.size() * 3), phi(panels.size() * 3);
  for (size_t id = 0; id < panels.size(); id++) panel_aabb(panels[id], &plo[3 * id], &phi[3 * id]);
  double pedge[3];
  for (int k = 0; k < 3; k++) pedge[k] = 1.0 / g.inv[k];
  const double pad = 1e-4 * std::min({(double)cell[0], (double)cell[1], (double)cell[2]}) +
                     1e-6 * (std::fabs(lo[0]) + std::fabs(lo[1]) + std::fabs(lo[2]) + 1.0);
  auto slab = [&](uint32_t z0, uint32_t z1) {
    for (uint32_t z = z0; z < z1; z++)
      for (uint32_t y = 0; y < dims[1]; y++)
        for (uint32_t x = 0; x < dims[0]; x++) {
          const uint32_t c3[3] = {x, y, z};
          double blo[3], bhi[3];
          int r0[3], r1[3];
          for (int k = 0; k < 3; k++) {
            blo[k] = (double)lo[k] + (double)c3[k] * cell[k] - reach;
            bhi[k] = (double)lo[k] + (double)(c3[k] + 1) * cell[k] + reach;
            const double f0 = std::floor((blo[k] - pad - g.lo[k]) / pedge[k]);
            const double f1 = std::floor((bhi[k] + pad - g.lo[k]) / pedge[k]);
            r0[k] = (int)std::min<double>(std::max<double>(f0, 0.0), g.dims[k] - 1.0);
            r1[k] = (int)std::min<double>(std::max<double>(f1, 0.0), g.dims[k] - 1.0);
          }
          uint8_t m = 0;
          for (int bz = r0[2]; bz <= r1[2] && m != 0xFF; bz++)
            for (int by = r0[1]; by <= r1[1] && m != 0xFF; by++)
              for (int bx = r0[0]; bx <= r1[0] && m != 0xFF; bx++) {
                const uint32_t box = ((uint32_t)bz * g.dims[1] + (uint32_t)by) * g.dims[0] + (uint32_t)bx;
                for (uint32_t e = g.start[box]; e < g.start[box + 1]; e++) {
                  const uint32_t id = g.list[e];
                  if (!(panel_species[id] & ~m)) continue;
                  bool apart = false;
                  for (int k = 0; k < 3; k++)
                    apart |= plo[3 * id + k] > bhi[k] + pad || phi[3 * id + k] < blo[k] - pad;
                  if (!apart && panel_meets_box(panels[id], blo, bhi, pad)) m |= panel_species[id];
                }
              }
          out[((size_t)z * dims[1] + y) * dims[0] + x] = m;
        }
  };
  const uint32_t nt = std::max(1u, std::min<uint32_t>(std::thread::hardware_concurrency(), dims[2]));
  std::vector<std::thread> pool;
  for (uint32_t t = 0; t < nt; t++)
    pool.emplace_back(slab, (uint32_t)((uint64_t)dims[2] * t / nt), (uint32_t)((uint64_t)dims[2] * (t + 1) / nt));
  for (std::thread& th : pool) th.join();
}

}  // namespace bd

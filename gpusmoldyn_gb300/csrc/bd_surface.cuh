// bd_surface.cuh -- surface panels on the step's displacement segments.
//
// The reference drafts Smoldyn's surfaces (panelside, lineXpanel in
// surfaces_kernel.cuh:97-248; checkSurfaceCollisions, particles_kernel.cu:
// 414-440) but never compiles or launches them.  This is a GPU design of the
// same model: a molecule's move from x0 to x1 is walked against the panels
// near the segment, the first crossing along it is found, and the action of
// the panel's surface for the molecule's species on the face it arrives
// from is applied (absorb, transmit, reflect), repeating on what is left of
// the move.
//
// Every float operation is explicitly rounded (as in bd_device.cuh), so a
// CPU program doing the same IEEE operations in the same order reproduces
// each crossing, reflection and nudge bit for bit.  The order of
// operations is part of the contract:
//   dot(a, b)        = (ax*bx + ay*by) + az*bz
//   side, rect       = +-(x[axis] - a[axis])
//   side, tri/disk   = dot(x - a, n)
//   side, sph/hemi   = +-(dot(w, w) - r2), w = x - a
//   side, cyl        = +-(dot(q, q) - r2), q = w - dot(w, n) n (per component)
//   crossing, flat   t = s0 / (s0 - s1), c = fma(t, x1 - x0, x0)
//   crossing, curved A, B, C of |w + t d|^2 = r2 (perpendicular parts for
//                    cyl), disc = B*B - A*C, t = (-B -+ sqrt(disc)) / A,
//                    clamped to [0, 1]
// A point exactly on a panel is on its back face.
#pragma once
#include "bd_device.cuh"
#include "bd_kernels.h"

namespace bd {

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ float comp(const V3& v, uint32_t k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }
__device__ __forceinline__ V3 sub3(const V3& a, const V3& b) {
  return V3{__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)};
}
__device__ __forceinline__ float dot3(const V3& a, const V3& b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
// a + t b, one rounding per component
__device__ __forceinline__ V3 axpy3(float t, const V3& b, const V3& a) {
  return V3{__fmaf_rn(t, b.x, a.x), __fmaf_rn(t, b.y, a.y), __fmaf_rn(t, b.z, a.z)};
}
__device__ __forceinline__ V3 ld3(const float* p) { return V3{p[0], p[1], p[2]}; }

// Component of w perpendicular to the unit axis n.
__device__ __forceinline__ V3 perp3(const V3& w, const V3& n) {
  const float t = dot3(w, n);
  return V3{__fsub_rn(w.x, __fmul_rn(t, n.x)), __fsub_rn(w.y, __fmul_rn(t, n.y)), __fsub_rn(w.z, __fmul_rn(t, n.z))};
}

// Signed side value of x for panel P: > 0 on the front face.
__device__ __forceinline__ float panel_side(const DevPanel& P, const V3& x) {
  const V3 a = ld3(P.a);
  float s;
  switch (P.shape) {
    case kPanelRect:
      s = __fsub_rn(comp(x, P.axis), comp(a, P.axis));
      return P.front > 0.0f ? s : -s;
    case kPanelTri:
    case kPanelDisk:
      return dot3(sub3(x, a), ld3(P.n));
    case kPanelCyl: {
      const V3 q = perp3(sub3(x, a), ld3(P.n));
      s = __fsub_rn(dot3(q, q), P.r2);
      return P.front > 0.0f ? s : -s;
    }
    default: {  // sphere, hemisphere
      const V3 w = sub3(x, a);
      s = __fsub_rn(dot3(w, w), P.r2);
      return P.front > 0.0f ? s : -s;
    }
  }
}

// Explicit selects (not fminf / fmaxf): the sign of a zero is kept.
__device__ __forceinline__ float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

// (e x w) . n
__device__ __forceinline__ float edge_test(const V3& e, const V3& w, const V3& n) {
  const V3 c{__fsub_rn(__fmul_rn(e.y, w.z), __fmul_rn(e.z, w.y)),
             __fsub_rn(__fmul_rn(e.z, w.x), __fmul_rn(e.x, w.z)),
             __fsub_rn(__fmul_rn(e.x, w.y), __fmul_rn(e.y, w.x))};
  return dot3(c, n);
}

// Does the crossing point c of a curved panel lie on the panel?
__device__ __forceinline__ bool curved_on_panel(const DevPanel& P, const V3& c) {
  if (P.shape == kPanelSph) return true;
  const float h = dot3(sub3(c, ld3(P.a)), ld3(P.n));
  if (P.shape == kPanelHemi) return h <= 0.0f;
  return h >= 0.0f && h <= P.len;  // cylinder between its ends
}

// First crossing of the segment x0 -> x1 (side values s0, s1) with P.
// Returns true with the fraction t in [0, 1] and the face the segment
// arrives from (true = front).
__device__ __forceinline__ bool panel_cross(const DevPanel& P, const V3& x0, const V3& x1, float s0, float s1,
                                            float& t, bool& face_front) {
  const bool f0 = s0 > 0.0f, f1 = s1 > 0.0f;
  const V3 d = sub3(x1, x0);
  if (P.shape == kPanelRect || P.shape == kPanelTri || P.shape == kPanelDisk) {
    if (f0 == f1) return false;
    t = __fdiv_rn(s0, __fsub_rn(s0, s1));
    const V3 c = axpy3(t, d, x0);
    face_front = f0;
    if (P.shape == kPanelRect) {
      const uint32_t u = P.axis == 0 ? 1u : 0u, v = P.axis == 2 ? 1u : 2u;
      const float cu = comp(c, u), cv = comp(c, v);
      return P.bounds[0] <= cu && cu <= P.bounds[1] && P.bounds[2] <= cv && cv <= P.bounds[3];
    }
    const V3 a = ld3(P.a), n = ld3(P.n);
    if (P.shape == kPanelDisk) {
      const V3 w = sub3(c, a);
      return dot3(w, w) <= P.r2;
    }
    const V3 b = ld3(P.v1), e = ld3(P.v2);
    return edge_test(sub3(b, a), sub3(c, a), n) >= 0.0f && edge_test(sub3(e, b), sub3(c, b), n) >= 0.0f &&
           edge_test(sub3(a, e), sub3(c, e), n) >= 0.0f;
  }
  // sphere, hemisphere, cylinder: "inside" is the face on the centre's side
  const bool out_front = P.front > 0.0f;
  const bool in0 = f0 != out_front, in1 = f1 != out_front;
  if (in0 && in1) return false;
  const V3 w = sub3(x0, ld3(P.a));
  float A, B, C;
  if (P.shape == kPanelCyl) {
    const V3 n = ld3(P.n);
    const V3 dp = perp3(d, n), wp = perp3(w, n);
    A = dot3(dp, dp);
    B = dot3(dp, wp);
    C = __fsub_rn(dot3(wp, wp), P.r2);
  } else {
    A = dot3(d, d);
    B = dot3(d, w);
    C = __fsub_rn(dot3(w, w), P.r2);
  }
  if (!(A > 0.0f)) return false;
  const float disc = __fsub_rn(__fmul_rn(B, B), __fmul_rn(A, C));
  if (!in0 && !in1 && !(disc > 0.0f)) return false;
  const float sq = __fsqrt_rn(disc > 0.0f ? disc : 0.0f);
  const float raw1 = __fdiv_rn(__fsub_rn(-B, sq), A);
  const float t1 = clamp01(raw1);
  const float t2 = clamp01(__fdiv_rn(__fadd_rn(-B, sq), A));
  if (in0) {  // leaving: the far root
    t = t2;
    face_front = f0;
    return curved_on_panel(P, axpy3(t2, d, x0));
  }
  if (in1) {  // entering: the near root
    t = t1;
    face_front = f0;
    return curved_on_panel(P, axpy3(t1, d, x0));
  }
  // both ends outside: through the object only if the near root is on the
  // segment; the far root (leaving) counts where the near one misses the panel
  if (!(raw1 >= 0.0f && raw1 <= 1.0f)) return false;
  if (curved_on_panel(P, axpy3(t1, d, x0))) {
    t = t1;
    face_front = f0;
    return true;
  }
  if (P.shape == kPanelSph) return false;
  t = t2;
  face_front = !f0;
  return curved_on_panel(P, axpy3(t2, d, x0));
}

// Unit normal of P at the crossing point c, pointing to the front face; false
// where it is undefined (c on a curved panel's axis or centre).
__device__ __forceinline__ bool front_normal(const DevPanel& P, const V3& c, V3& m) {
  switch (P.shape) {
    case kPanelRect:
      m = V3{P.axis == 0 ? P.front : 0.0f, P.axis == 1 ? P.front : 0.0f, P.axis == 2 ? P.front : 0.0f};
      return true;
    case kPanelTri:
    case kPanelDisk:
      m = ld3(P.n);
      return true;
    default: {
      V3 w = sub3(c, ld3(P.a));
      if (P.shape == kPanelCyl) w = perp3(w, ld3(P.n));
      const float L = __fsqrt_rn(dot3(w, w));
      if (!(L > 0.0f)) return false;
      const float k = __fdiv_rn(P.front, L);
      m = V3{__fmul_rn(w.x, k), __fmul_rn(w.y, k), __fmul_rn(w.z, k)};
      return true;
    }
  }
}

// Mirror x1 in the tangent plane of P at c.
__device__ __forceinline__ V3 panel_reflect(const DevPanel& P, const V3& c, const V3& x1) {
  if (P.shape == kPanelRect) {
    const float m = __fsub_rn(__fmul_rn(2.0f, comp(ld3(P.a), P.axis)), comp(x1, P.axis));
    return V3{P.axis == 0 ? m : x1.x, P.axis == 1 ? m : x1.y, P.axis == 2 ? m : x1.z};
  }
  V3 m;
  if (!front_normal(P, c, m)) return x1;
  const float delta = dot3(sub3(x1, c), m);
  return axpy3(__fmul_rn(-2.0f, delta), m, x1);
}

// A point on face `want` (true = front) of P close to the crossing point c:
// c itself, else c moved along the front normal by 2^-21 (|c|_1 + 1) times
// 1, 4, 16, ... (8 tries).  Returns false when none of them is.
__device__ __forceinline__ bool panel_nudge(const DevPanel& P, const V3& c, bool want, V3& q) {
  q = c;
  if ((panel_side(P, c) > 0.0f) == want) return true;
  V3 m;
  if (!front_normal(P, c, m)) return false;
  const float eps0 =
      __fmul_rn(__fadd_rn(__fadd_rn(__fadd_rn(fabsf(c.x), fabsf(c.y)), fabsf(c.z)), 1.0f), 4.76837158203125e-07f);
  float e = want ? eps0 : -eps0;
#pragma unroll 1
  for (int k = 0; k < 8; ++k) {
    q = axpy3(e, m, c);
    if ((panel_side(P, q) > 0.0f) == want) return true;
    e = __fmul_rn(e, 4.0f);
  }
  q = c;
  return false;
}

// What the walk reads: the surface fields of the kernel parameters.
struct SurfView {
  const DevPanel* panels;
  const uint8_t* act;
  const uint32_t* start;
  const uint32_t* list;
  float lo[3], inv[3];
  uint32_t dims[3];
  uint32_t S;
};

__device__ __forceinline__ SurfView surf_view(const KParams& p) {
  SurfView v;
  v.panels = p.panels;
  v.act = p.surf_act;
  v.start = p.pbox_start;
  v.list = p.pbox_list;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    v.lo[k] = p.pbox_lo[k];
    v.inv[k] = p.pbox_inv[k];
    v.dims[k] = p.pbox_dims[k];
  }
  v.S = p.S;
  return v;
}

__device__ __forceinline__ uint32_t pbox_coord(float x, float lo, float inv, uint32_t n) {
  const float f = __fmul_rn(__fsub_rn(x, lo), inv);
  int c = (int)floorf(f);
  c = c < 0 ? 0 : c;
  c = c > (int)n - 1 ? (int)n - 1 : c;
  return (uint32_t)c;
}

// Move a molecule of species sp from x0 to x1 through the surfaces.  On
// return x1 holds where it ends; false = absorbed.
__device__ __forceinline__ bool surface_move(const SurfView& p, uint32_t sp, V3 x0, V3& x1) {
  constexpr uint32_t kNone = 0xFFFFFFFFu;
#pragma unroll 1
  for (int hit = 0; hit < kMaxSurfaceHits; ++hit) {
    uint32_t lo[3], hi[3];
    const V3 mn{fminf(x0.x, x1.x), fminf(x0.y, x1.y), fminf(x0.z, x1.z)};
    const V3 mx{fmaxf(x0.x, x1.x), fmaxf(x0.y, x1.y), fmaxf(x0.z, x1.z)};
    lo[0] = pbox_coord(mn.x, p.lo[0], p.inv[0], p.dims[0]);
    lo[1] = pbox_coord(mn.y, p.lo[1], p.inv[1], p.dims[1]);
    lo[2] = pbox_coord(mn.z, p.lo[2], p.inv[2], p.dims[2]);
    hi[0] = pbox_coord(mx.x, p.lo[0], p.inv[0], p.dims[0]);
    hi[1] = pbox_coord(mx.y, p.lo[1], p.inv[1], p.dims[1]);
    hi[2] = pbox_coord(mx.z, p.lo[2], p.inv[2], p.dims[2]);
    float best_t = 2.0f;
    uint32_t best = kNone;
    bool best_front = false;
#pragma unroll 1
    for (uint32_t bz = lo[2]; bz <= hi[2]; ++bz)
#pragma unroll 1
      for (uint32_t by = lo[1]; by <= hi[1]; ++by)
#pragma unroll 1
        for (uint32_t bx = lo[0]; bx <= hi[0]; ++bx) {
          const uint32_t box = (bz * p.dims[1] + by) * p.dims[0] + bx;
          const uint32_t e = __ldg(&p.start[box + 1]);
#pragma unroll 1
          for (uint32_t k = __ldg(&p.start[box]); k < e; ++k) {
            const uint32_t id = __ldg(&p.list[k]);
            const DevPanel& P = p.panels[id];
            const uint8_t* act = &p.act[((size_t)P.surface * p.S + sp) * 2u];
            if (act[0] == kActTransmit && act[1] == kActTransmit) continue;  // invisible to sp
            float t;
            bool ff;
            if (panel_cross(P, x0, x1, panel_side(P, x0), panel_side(P, x1), t, ff) &&
                (t < best_t || (t == best_t && id < best))) {
              best_t = t;
              best = id;
              best_front = ff;
            }
          }
        }
    if (best == kNone) return true;
    const DevPanel& P = p.panels[best];
    const uint8_t action = p.act[((size_t)P.surface * p.S + sp) * 2u + (best_front ? 0u : 1u)];
    const V3 c = axpy3(best_t, sub3(x1, x0), x0);
    if (action == kActAbsorb) return false;
    V3 q;
    if (action == kActTransmit) {
      panel_nudge(P, c, !best_front, q);
    } else {
      const bool x0_on_face = (panel_side(P, x0) > 0.0f) == best_front;
      x1 = panel_reflect(P, c, x1);
      if (!panel_nudge(P, c, best_front, q) && x0_on_face) q = x0;
    }
    x0 = q;
  }
  x1 = x0;  // too many crossings: stay at the last one
  return true;
}

}  // namespace bd

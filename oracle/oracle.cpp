// oracle.cpp -- TEST INFRASTRUCTURE: CPU restatement of one Smoldyn
// Brownian-dynamics timestep, used only to check the GPU library (tests,
// smoke) and to time a CPU baseline (bench.py).  Written independently of
// the library's kernels; compiled with -ffp-contract=off so each float
// operation below is one IEEE operation.
//
// Step semantics (reference call stack particleSystem.cpp:829-1001):
//  1. every live record diffuses, x += sqrt(2 D dt) g per axis
//     (diffuse, particles_kernel.cu:127-166), reflects at the walls
//     (replacing adjustPositions' clamp, particles_kernel.cu:61-95) and tries
//     its species' first-order reactions in list order, the first success
//     winning (uniReact, reaction_kernel.cuh:263-342);
//  2. zeroth-order reactions add Poisson-many particles uniformly in the box
//     (zeroReact, reaction_cpu.cpp:36-63);
//  3. if anything but diffusion can happen, records are sorted by uniform-grid
//     cell (calcHashD + RadixSort + reorderDataAndFindCellStartD,
//     particles_kernel.cu:170-272) and, inside a cell, by their bits;
//  4. every pair closer than its reaction's binding radius is a candidate
//     (collideD / collideCell, particles_kernel.cu:318-497), subject to a coin
//     when the reaction probability is below 1; candidates are accepted
//     greedily in (lower slot, upper slot) order, one reaction per particle;
//  5. accepted pairs become their products at the D-weighted reaction point
//     (bimReact, reaction_kernel.cuh:202-258); reactants without a product
//     leave an empty slot.
// Random numbers come from Philox4x32-10 keyed by (seed, step, slot, tag).
#include "oracle.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const uint32_t DEAD = 0xFFFFFFFFu;
const uint32_t T_DIFF = 1u << 24, T_UNI = 2u << 24, T_UNIDIR = 3u << 24, T_ZCOUNT = 4u << 24, T_ZPOS = 5u << 24,
               T_BIM = 6u << 24, T_BIMDIR = 7u << 24, T_BIMCHAN = 8u << 24;

struct Rec {
  float x, y, z;
  uint32_t w;
};

inline uint32_t fbits(float f) {
  uint32_t u;
  memcpy(&u, &f, 4);
  return u;
}
inline float bitsf(uint32_t u) {
  float f;
  memcpy(&f, &u, 4);
  return f;
}

// Philox4x32-10, Salmon et al. (SC'11): round function
// (c0,c1,c2,c3) -> (hi(M1*c2)^c1^k0, lo(M1*c2), hi(M0*c0)^c3^k1, lo(M0*c0)).
void philox10(const uint32_t in[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  uint32_t c0 = in[0], c1 = in[1], c2 = in[2], c3 = in[3];
  for (int r = 0; r < 10; r++) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    const uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n1 = (uint32_t)p1;
    const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    const uint32_t n3 = (uint32_t)p0;
    c0 = n0;
    c1 = n1;
    c2 = n2;
    c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

struct Rng {
  uint32_t k0, k1;
  void block(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t o[4]) const {
    const uint32_t in[4] = {a, b, c, d};
    philox10(in, k0, k1, o);
  }
};

// float(v) * 2^-32 (the reference's randReal)
inline float unit32(uint32_t v) { return (float)v * 2.3283064365386963e-10f; }
inline float unit24(uint32_t v) { return (float)(v >> 8) * 5.9604644775390625e-08f; }
inline double unit53(uint32_t a, uint32_t b) {
  const uint64_t m = ((uint64_t)(a >> 5) << 26) | (uint64_t)(b >> 6);
  return (double)m * 1.1102230246251565e-16;
}

float wall(float x, float lo, float hi) {
  for (int k = 0; k < 8; k++) {
    if (x > hi) x = 2.0f * hi - x;
    else if (x < lo) x = 2.0f * lo - x;
    else return x;
  }
  return std::min(std::max(x, lo), hi);
}

void direction(const Rng& g, uint32_t a, uint32_t b, uint32_t tag, uint32_t d, float v[3]) {
  for (uint32_t att = 0; att < 8; att++) {
    uint32_t o[4];
    g.block(a, b, tag | att, d, o);
    for (int h = 0; h < 2; h++) {
      const float u = (float)(o[2 * h] >> 8) * 1.1920928955078125e-07f - 1.0f;
      const float w = (float)(o[2 * h + 1] >> 8) * 1.1920928955078125e-07f - 1.0f;
      const float s = u * u + w * w;
      if (s < 1.0f && s > 0.0f) {
        const float q = 2.0f * std::sqrt(1.0f - s);
        v[0] = u * q;
        v[1] = w * q;
        v[2] = 1.0f - 2.0f * s;
        return;
      }
    }
  }
  v[0] = 0.0f;
  v[1] = 0.0f;
  v[2] = 1.0f;
}

// ---- surfaces -------------------------------------------------------------
// Smoldyn's surface panels (the reference drafts panelside / lineXpanel in
// surfaces_kernel.cuh:97-248 and a per-molecule walk in
// checkSurfaceCollisions, particles_kernel.cu:414-440, neither of which is
// ever compiled).  A molecule's move x0 -> x1 is tested against every
// panel; the first crossing along it (lowest fraction, then lowest panel id)
// is acted on with the action of the panel's surface for the species on the
// face the move arrives from: absorb ends the walk, transmit continues just
// past the crossing, reflect mirrors the end in the tangent plane at the
// crossing point and continues just before it; at most 8 crossings, after
// which the molecule stays at its last crossing.  A surface that transmits
// a species on both faces is invisible to it.  A point exactly on a panel
// is on its back face.
enum { P_RECT = 0, P_TRI = 1, P_SPH = 2, P_CYL = 3, P_HEMI = 4, P_DISK = 5 };

inline float dot3(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
inline void diff3(const float a[3], const float b[3], float out[3]) {
  for (int k = 0; k < 3; k++) out[k] = a[k] - b[k];
}
// component of w across the unit axis n
inline void across(const float w[3], const float n[3], float out[3]) {
  const float t = dot3(w, n);
  for (int k = 0; k < 3; k++) out[k] = w[k] - t * n[k];
}
inline float clamp01(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }

float side(const or_panel& P, const float x[3]) {
  float w[3];
  diff3(x, P.a, w);
  float s;
  if (P.shape == P_RECT) {
    s = x[P.axis] - P.a[P.axis];
    return P.front > 0.0f ? s : -s;
  }
  if (P.shape == P_TRI || P.shape == P_DISK) return dot3(w, P.n);
  if (P.shape == P_CYL) {
    float q[3];
    across(w, P.n, q);
    s = dot3(q, q) - P.r2;
  } else {
    s = dot3(w, w) - P.r2;
  }
  return P.front > 0.0f ? s : -s;
}

// ((e x w) . n)
float edge(const float e[3], const float w[3], const float n[3]) {
  const float c[3] = {e[1] * w[2] - e[2] * w[1], e[2] * w[0] - e[0] * w[2], e[0] * w[1] - e[1] * w[0]};
  return dot3(c, n);
}

bool on_curved(const or_panel& P, const float c[3]) {
  if (P.shape == P_SPH) return true;
  float w[3];
  diff3(c, P.a, w);
  const float h = dot3(w, P.n);
  return P.shape == P_HEMI ? h <= 0.0f : (h >= 0.0f && h <= P.len);
}

bool crossing(const or_panel& P, const float x0[3], const float x1[3], float s0, float s1, float* t, bool* ff) {
  const bool f0 = s0 > 0.0f, f1 = s1 > 0.0f;
  float d[3], c[3];
  diff3(x1, x0, d);
  auto at = [&](float tt) {
    for (int k = 0; k < 3; k++) c[k] = std::fmaf(tt, d[k], x0[k]);
  };
  if (P.shape == P_RECT || P.shape == P_TRI || P.shape == P_DISK) {
    if (f0 == f1) return false;
    *t = s0 / (s0 - s1);
    *ff = f0;
    at(*t);
    if (P.shape == P_RECT) {
      const int u = P.axis == 0 ? 1 : 0, v = P.axis == 2 ? 1 : 2;
      return P.bounds[0] <= c[u] && c[u] <= P.bounds[1] && P.bounds[2] <= c[v] && c[v] <= P.bounds[3];
    }
    float w[3];
    if (P.shape == P_DISK) {
      diff3(c, P.a, w);
      return dot3(w, w) <= P.r2;
    }
    float e[3];
    diff3(P.v1, P.a, e);
    diff3(c, P.a, w);
    if (!(edge(e, w, P.n) >= 0.0f)) return false;
    diff3(P.v2, P.v1, e);
    diff3(c, P.v1, w);
    if (!(edge(e, w, P.n) >= 0.0f)) return false;
    diff3(P.a, P.v2, e);
    diff3(c, P.v2, w);
    return edge(e, w, P.n) >= 0.0f;
  }
  const bool outward = P.front > 0.0f;
  const bool in0 = f0 != outward, in1 = f1 != outward;
  if (in0 && in1) return false;
  float w[3], A, B, C;
  diff3(x0, P.a, w);
  if (P.shape == P_CYL) {
    float dq[3], wq[3];
    across(d, P.n, dq);
    across(w, P.n, wq);
    A = dot3(dq, dq);
    B = dot3(dq, wq);
    C = dot3(wq, wq) - P.r2;
  } else {
    A = dot3(d, d);
    B = dot3(d, w);
    C = dot3(w, w) - P.r2;
  }
  if (!(A > 0.0f)) return false;
  const float disc = B * B - A * C;
  if (!in0 && !in1 && !(disc > 0.0f)) return false;
  const float sq = std::sqrt(disc > 0.0f ? disc : 0.0f);
  const float near = (-B - sq) / A, far = (-B + sq) / A;
  if (in0 || in1) {
    // one end inside: leaving through the far root or entering through the near one
    *t = clamp01(in0 ? far : near);
    *ff = f0;
    at(*t);
    return on_curved(P, c);
  }
  if (!(near >= 0.0f && near <= 1.0f)) return false;
  *t = near;
  *ff = f0;
  at(near);
  if (on_curved(P, c)) return true;
  if (P.shape == P_SPH) return false;
  *t = clamp01(far);
  *ff = !f0;
  at(*t);
  return on_curved(P, c);
}

// unit normal toward the front face at c
bool normal_at(const or_panel& P, const float c[3], float m[3]) {
  if (P.shape == P_RECT) {
    for (int k = 0; k < 3; k++) m[k] = k == P.axis ? P.front : 0.0f;
    return true;
  }
  if (P.shape == P_TRI || P.shape == P_DISK) {
    for (int k = 0; k < 3; k++) m[k] = P.n[k];
    return true;
  }
  float w[3];
  diff3(c, P.a, w);
  if (P.shape == P_CYL) {
    float q[3];
    across(w, P.n, q);
    for (int k = 0; k < 3; k++) w[k] = q[k];
  }
  const float L = std::sqrt(dot3(w, w));
  if (!(L > 0.0f)) return false;
  const float inv = P.front / L;
  for (int k = 0; k < 3; k++) m[k] = w[k] * inv;
  return true;
}

void mirror(const or_panel& P, const float c[3], float x1[3]) {
  if (P.shape == P_RECT) {
    x1[P.axis] = 2.0f * P.a[P.axis] - x1[P.axis];
    return;
  }
  float m[3], v[3];
  if (!normal_at(P, c, m)) return;
  diff3(x1, c, v);
  const float k2 = -2.0f * dot3(v, m);
  for (int k = 0; k < 3; k++) x1[k] = std::fmaf(k2, m[k], x1[k]);
}

// a point on face `front` near c: c, else c pushed along the normal by
// 2^-21 (|c|_1 + 1) x 1, 4, 16, ...; false if 8 pushes do not get there
bool onto_face(const or_panel& P, const float c[3], bool front, float q[3]) {
  for (int k = 0; k < 3; k++) q[k] = c[k];
  if ((side(P, c) > 0.0f) == front) return true;
  float m[3];
  if (!normal_at(P, c, m)) return false;
  float e = (((std::fabs(c[0]) + std::fabs(c[1])) + std::fabs(c[2])) + 1.0f) * 4.76837158203125e-07f;
  if (!front) e = -e;
  for (int it = 0; it < 8; it++) {
    for (int k = 0; k < 3; k++) q[k] = std::fmaf(e, m[k], c[k]);
    if ((side(P, q) > 0.0f) == front) return true;
    e = e * 4.0f;
  }
  for (int k = 0; k < 3; k++) q[k] = c[k];
  return false;
}

// the walk of one move; false = absorbed, x1 = where the molecule ends
bool walk(const or_system* s, int sp, const float start[3], float x1[3]) {
  float x0[3] = {start[0], start[1], start[2]};
  for (int hit = 0; hit < 8; hit++) {
    int best = -1;
    float best_t = 2.0f;
    bool best_front = false;
    for (int id = 0; id < s->n_panels; id++) {
      const or_panel& P = s->panels[id];
      const uint8_t* act = s->surf_act + ((size_t)P.surface * s->S + sp) * 2;
      if (act[0] == 0 && act[1] == 0) continue;
      float t;
      bool ff;
      if (crossing(P, x0, x1, side(P, x0), side(P, x1), &t, &ff) && t < best_t) {
        best = id;
        best_t = t;
        best_front = ff;
      }
    }
    if (best < 0) return true;
    const or_panel& P = s->panels[best];
    const uint8_t action = s->surf_act[((size_t)P.surface * s->S + sp) * 2 + (best_front ? 0 : 1)];
    if (action == 2) return false;
    float c[3], q[3];
    for (int k = 0; k < 3; k++) c[k] = std::fmaf(best_t, x1[k] - x0[k], x0[k]);
    if (action == 0) {
      onto_face(P, c, !best_front, q);
    } else {
      const bool start_on_face = (side(P, x0) > 0.0f) == best_front;
      mirror(P, c, x1);
      if (!onto_face(P, c, best_front, q) && start_on_face)
        for (int k = 0; k < 3; k++) q[k] = x0[k];
    }
    for (int k = 0; k < 3; k++) x0[k] = q[k];
  }
  for (int k = 0; k < 3; k++) x1[k] = x0[k];
  return true;
}

// the walls reflect first (the move's chord stays in the box, so a panel
// that reaches a wall cannot be passed by way of the wall) and once more
// after the walk, whose reflections can leave the box
bool walk_in_box(const or_system* s, int sp, const float start[3], float x1[3]) {
  if (!walk(s, sp, start, x1)) return false;
  for (int a = 0; a < 3; a++) x1[a] = wall(x1[a], s->lo[a], s->hi[a]);
  return true;
}

struct Model {
  const or_system* s;
  Rng rng;
  std::vector<float> sigma;
  std::vector<std::vector<int>> uni;  // per species, reaction ids in index order
  std::vector<int> table;             // S*S -> reaction id or -1
  std::vector<int> next;              // competing reactions: next reaction of the pair, -1 = last
  std::vector<float> r2;              // per reaction
  std::vector<int> zero;              // order-0 reaction ids in index order
  float max_r = 0.0f;
};

void build_model(const or_system* s, Model* m) {
  m->s = s;
  m->rng = Rng{s->key_lo, s->key_hi};
  const int S = s->S, R = s->R;
  m->sigma.resize(S);
  for (int i = 0; i < S; i++) m->sigma[i] = sqrtf(2.0f * s->D[i] * s->dt);
  m->uni.assign(S, std::vector<int>());
  m->table.assign((size_t)S * S, -1);
  m->r2.assign(R, 0.0f);
  m->next.assign(R, -1);
  for (int r = 0; r < R; r++) {
    if (s->order[r] == 1) m->uni[s->react0[r]].push_back(r);
    if (s->order[r] == 0) m->zero.push_back(r);
    if (s->order[r] == 2) {
      m->r2[r] = s->bind_radius[r] * s->bind_radius[r];
      int& e0 = m->table[(size_t)s->react0[r] * S + s->react1[r]];
      int& e1 = m->table[(size_t)s->react1[r] * S + s->react0[r]];
      if (!s->channels) {
        // the last reaction listed for a pair is the pair's reaction
        e0 = e1 = m->r2[r] > 0.0f ? r : -1;
      } else if (m->r2[r] > 0.0f) {
        // competing reactions: the pair's first reaction starts the chain
        if (e0 < 0) {
          e0 = e1 = r;
        } else {
          int last = e0;
          while (m->next[last] >= 0) last = m->next[last];
          m->next[last] = r;
        }
      }
    }
  }
  for (int r = 0; r < R; r++)
    if (s->order[r] == 2 && m->r2[r] > 0.0f) m->max_r = std::max(m->max_r, s->bind_radius[r]);
}

inline uint32_t pack(uint32_t inst, int sp) { return (inst << 16) | ((uint32_t)sp & 0x7FFFu); }

// born in this step (uni second product, zeroth order): sorted with the
// mark, excluded from this step's pair search, cleared in the output
const uint32_t NEWBORN = 0x8000u;

// Step 1 for slot i: returns the number of records written to out.
int advance(const Model& m, uint32_t t, uint32_t i, const Rec& in, Rec out[2], uint64_t* ev) {
  const or_system* s = m.s;
  if (in.w == DEAD) return 0;
  const int sp = (int)(in.w & 0x7FFFu);
  uint32_t o[4];
  m.rng.block(i, t, T_DIFF, 0, o);
  float g[3];
  if (s->normal_mode == 1) {
    for (int a = 0; a < 3; a++) g[a] = s->gauss[o[a] >> 20];
  } else {
    const float ua = unit24(o[0]) + 2.98023223876953125e-08f, uc = unit24(o[2]) + 2.98023223876953125e-08f;
    const float ra = sqrtf(-2.0f * logf(ua)), rc = sqrtf(-2.0f * logf(uc));
    const uint32_t low = ((o[0] & 0xFFu) << 24) | ((o[1] & 0xFFu) << 16) | ((o[2] & 0xFFu) << 8);
    const float pa = 6.283185307179586f * unit24(o[1]), pc = 6.283185307179586f * unit24(low);
    g[0] = ra * cosf(pa);
    g[1] = ra * sinf(pa);
    g[2] = rc * cosf(pc);
  }
  float p[3] = {in.x, in.y, in.z};
  float to[3];
  for (int a = 0; a < 3; a++) to[a] = wall(std::fmaf(m.sigma[sp], g[a], p[a]), s->lo[a], s->hi[a]);
  if (s->n_panels > 0 && !walk_in_box(s, sp, p, to)) return 0;  // absorbed
  for (int a = 0; a < 3; a++) p[a] = to[a];
  int species = sp;
  int n = 1;
  const std::vector<int>& list = m.uni[sp];
  // the first coin is the diffusion block's fourth word, the others come
  // four per block of the first-order stream
  uint32_t coin[4] = {0, 0, 0, 0};
  for (size_t k = 0; k < list.size(); k++) {
    if (k > 0 && (k - 1) % 4 == 0) m.rng.block(i, t, T_UNI | (uint32_t)((k - 1) / 4), 0, coin);
    const int r = list[k];
    const uint32_t word = k == 0 ? o[3] : coin[(k - 1) % 4];
    if (unit32(word) < s->prob[r]) {
      if (ev) ev[r]++;
      if (s->prod0[r] < 0) return 0;
      species = s->prod0[r];
      if (s->prod1[r] >= 0) {
        float b[3] = {p[0], p[1], p[2]};
        bool alive0 = true, alive1 = true;
        if (s->off0[r] != 0.0f || s->off1[r] != 0.0f) {
          float d[3], a0[3];
          direction(m.rng, i, t, T_UNIDIR, 0, d);
          for (int a = 0; a < 3; a++) {
            b[a] = wall(std::fmaf(s->off1[r], d[a], p[a]), s->lo[a], s->hi[a]);
            a0[a] = wall(std::fmaf(s->off0[r], d[a], p[a]), s->lo[a], s->hi[a]);
          }
          if (s->n_panels > 0) {
            alive1 = walk_in_box(s, s->prod1[r], p, b);
            alive0 = walk_in_box(s, s->prod0[r], p, a0);
          }
          for (int a = 0; a < 3; a++) p[a] = a0[a];
        }
        const Rec born{b[0], b[1], b[2], pack(s->inst, s->prod1[r]) | NEWBORN};
        if (!alive0) {
          // the first product was absorbed on its way out: only the second is left
          if (!alive1) return 0;
          out[0] = born;
          return 1;
        }
        if (alive1) {
          out[1] = born;
          n = 2;
        }
      }
      break;
    }
  }
  out[0] = Rec{p[0], p[1], p[2], pack(s->inst, species)};
  return n;
}

int cell_axis(float x, float lo, float inv, uint32_t n) {
  const float f = (x - lo) * inv;
  int c = (int)floorf(f);
  if (c < 0) c = 0;
  if (c > (int)n - 1) c = (int)n - 1;
  return c;
}

uint32_t cell_of(const or_system* s, const Rec& r) {
  const int cx = cell_axis(r.x, s->lo[0], s->inv[0], s->dims[0]);
  const int cy = cell_axis(r.y, s->lo[1], s->inv[1], s->dims[1]);
  const int cz = cell_axis(r.z, s->lo[2], s->inv[2], s->dims[2]);
  return ((uint32_t)cz * s->dims[1] + (uint32_t)cy) * s->dims[0] + (uint32_t)cx;
}

bool rec_before(const Rec& a, const Rec& b) {
  const uint32_t ka[4] = {fbits(a.x), fbits(a.y), fbits(a.z), a.w};
  const uint32_t kb[4] = {fbits(b.x), fbits(b.y), fbits(b.z), b.w};
  for (int k = 0; k < 4; k++)
    if (ka[k] != kb[k]) return ka[k] < kb[k];
  return false;
}

struct Cand {
  uint32_t i, j;
  int r;
};

}  // namespace

extern "C" void or_philox(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
  philox10(ctr, k0, k1, out);
}

extern "C" int or_step(const or_system* s, uint32_t t, const uint32_t* in, uint32_t n, uint32_t* out, uint32_t cap,
                       uint32_t* n_out, uint32_t* cells, uint64_t cells_cap, uint32_t* pairs, uint32_t pairs_cap,
                       uint32_t* n_pairs, uint64_t* events) {
#ifdef _OPENMP
  if (s->threads > 0) omp_set_num_threads(s->threads);
#endif
  Model m;
  build_model(s, &m);
  const int R = s->R;
  std::vector<Rec> src(n);
  for (uint32_t i = 0; i < n; i++) src[i] = Rec{bitsf(in[4 * i]), bitsf(in[4 * i + 1]), bitsf(in[4 * i + 2]), in[4 * i + 3]};

  // 1. diffusion, walls, first order (2 output places per slot)
  std::vector<Rec> adv((size_t)2 * n);
  std::vector<uint8_t> cnt(n);
  std::vector<uint64_t> ev_total(std::max(R, 1), 0);
#pragma omp parallel
  {
    std::vector<uint64_t> ev(std::max(R, 1), 0);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
      Rec o2[2];
      cnt[i] = (uint8_t)advance(m, t, (uint32_t)i, src[i], o2, ev.data());
      adv[2 * i] = o2[0];
      adv[2 * i + 1] = o2[1];
    }
#pragma omp critical
    for (int r = 0; r < R; r++) ev_total[r] += ev[r];
  }

  // 2. zeroth-order births, reaction by reaction
  std::vector<Rec> born;
  uint32_t k_local = 0;
  for (size_t zi = 0; zi < m.zero.size(); zi++) {
    const int r = m.zero[zi];
    uint32_t o[4];
    m.rng.block((uint32_t)zi, t, T_ZCOUNT, 0, o);
    const double u = unit53(o[0], o[1]);
    const double* cdf = s->cdf + s->cdf_off[r];
    int idx = 0;
    while (idx < s->cdf_len[r] - 1 && !(cdf[idx] > u)) idx++;
    const uint32_t c = (uint32_t)(s->cdf_kmin[r] + idx);
    ev_total[r] += c;
    for (uint32_t k = 0; k < c; k++, k_local++) {
      m.rng.block(k_local, t, T_ZPOS, 0, o);
      float p[3];
      for (int a = 0; a < 3; a++)
        p[a] = std::min(std::fmaf(unit24(o[a]), s->hi[a] - s->lo[a], s->lo[a]), s->hi[a]);
      const uint32_t mark = s->sorted ? NEWBORN : 0u;
      born.push_back(Rec{p[0], p[1], p[2], pack(s->inst, s->prod0[r]) | mark});
      if (s->prod1[r] >= 0) born.push_back(Rec{p[0], p[1], p[2], pack(s->inst, s->prod1[r]) | mark});
    }
  }

  std::vector<Rec> res;
  uint32_t npairs = 0;
  if (!s->sorted) {
    // in place: every slot keeps its place (diffusion only), births appended
    res.resize(n);
    for (uint32_t i = 0; i < n; i++) res[i] = cnt[i] ? adv[2 * i] : src[i];
    res.insert(res.end(), born.begin(), born.end());
  } else {
    for (uint32_t i = 0; i < n; i++)
      for (int k = 0; k < cnt[i]; k++) res.push_back(adv[2 * i + k]);
    res.insert(res.end(), born.begin(), born.end());
    // 3. sort by cell, then by record bits
    const uint64_t ncell = (uint64_t)s->dims[0] * s->dims[1] * s->dims[2];
    std::vector<uint32_t> key(res.size());
    std::vector<uint32_t> start(ncell + 1, 0);
    for (size_t q = 0; q < res.size(); q++) {
      key[q] = cell_of(s, res[q]);
      start[key[q] + 1]++;
    }
    for (uint64_t c = 0; c < ncell; c++) start[c + 1] += start[c];
    std::vector<Rec> sorted(res.size());
    {
      std::vector<uint32_t> fill(start.begin(), start.end() - 1);
      for (size_t q = 0; q < res.size(); q++) sorted[fill[key[q]]++] = res[q];
    }
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t c = 0; c < (int64_t)ncell; c++)
      if (start[c + 1] - start[c] > 1) std::sort(sorted.begin() + start[c], sorted.begin() + start[c + 1], rec_before);
    res.swap(sorted);
    if (cells) {
      for (uint64_t c = 0; c <= ncell && c < cells_cap; c++) cells[c] = start[c];
    }

    // 4. candidate pairs over the 27 neighbour cells
    std::vector<Cand> cand;
    if (m.max_r > 0.0f) {
#pragma omp parallel
      {
        std::vector<Cand> mine;
#pragma omp for schedule(dynamic, 1024)
        for (int64_t ii = 0; ii < (int64_t)res.size(); ii++) {
          const uint32_t i = (uint32_t)ii;
          const Rec& a = res[i];
          if (a.w & NEWBORN) continue;
          const int sa = (int)(a.w & 0x7FFFu);
          const int cx = cell_axis(a.x, s->lo[0], s->inv[0], s->dims[0]);
          const int cy = cell_axis(a.y, s->lo[1], s->inv[1], s->dims[1]);
          const int cz = cell_axis(a.z, s->lo[2], s->inv[2], s->dims[2]);
          for (int dz = -1; dz <= 1; dz++)
            for (int dy = -1; dy <= 1; dy++)
              for (int dx = -1; dx <= 1; dx++) {
                const int x = cx + dx, y = cy + dy, z = cz + dz;
                if (x < 0 || y < 0 || z < 0 || x >= (int)s->dims[0] || y >= (int)s->dims[1] || z >= (int)s->dims[2])
                  continue;
                const uint32_t c = ((uint32_t)z * s->dims[1] + (uint32_t)y) * s->dims[0] + (uint32_t)x;
                for (uint32_t j = start[c]; j < start[c + 1]; j++) {
                  if (j <= i) continue;
                  const Rec& b = res[j];
                  if (b.w & NEWBORN) continue;
                  const int r = m.table[(size_t)sa * s->S + (b.w & 0x7FFFu)];
                  if (r < 0) continue;
                  const float ex = a.x - b.x, ey = a.y - b.y, ez = a.z - b.z;
                  const float d2 = (ex * ex + ey * ey) + ez * ez;
                  if (d2 > m.r2[r]) continue;
                  if (s->prob[r] < 1.0f) {
                    uint32_t o[4];
                    m.rng.block(i, t, T_BIM, j, o);
                    if (!(unit32(o[0]) < s->prob[r])) continue;
                  }
                  mine.push_back(Cand{i, j, r});
                }
              }
        }
#pragma omp critical
        cand.insert(cand.end(), mine.begin(), mine.end());
      }
    }
    std::sort(cand.begin(), cand.end(),
              [](const Cand& a, const Cand& b) { return a.i != b.i ? a.i < b.i : a.j < b.j; });
    // greedy matching in pair order
    std::vector<uint8_t> used(res.size(), 0);
    std::vector<uint8_t> acc(cand.size(), 0);
    for (size_t k = 0; k < cand.size(); k++) {
      if (used[cand[k].i] || used[cand[k].j]) continue;
      used[cand[k].i] = used[cand[k].j] = 1;
      acc[k] = 1;
    }
    // 5. products
    for (size_t k = 0; k < cand.size(); k++) {
      if (!acc[k]) continue;
      const Cand& q = cand[k];
      int r = q.r;
      if (s->channels && m.next[r] >= 0) {
        // which competing reaction: the one whose share holds the coin
        uint32_t o[4];
        m.rng.block(q.i, t, T_BIMCHAN, q.j, o);
        const float coin = unit24(o[0]);
        while (!(coin < s->thresh[r]) && m.next[r] >= 0) r = m.next[r];
      }
      const Rec ri = res[q.i], rj = res[q.j];
      const bool i_first = (int)(ri.w & 0x7FFFu) == s->react0[r];
      const uint32_t m1 = i_first ? q.i : q.j, m2 = i_first ? q.j : q.i;
      const Rec& p1 = i_first ? ri : rj;
      const Rec& p2 = i_first ? rj : ri;
      const float D1 = s->D[s->react0[r]], D2 = s->D[s->react1[r]];
      const float x = (D1 == 0.0f && D2 == 0.0f) ? 0.5f : D2 / (D1 + D2);
      const float omx = 1.0f - x;
      const float rp[3] = {std::fmaf(x, p1.x, omx * p2.x), std::fmaf(x, p1.y, omx * p2.y),
                           std::fmaf(x, p1.z, omx * p2.z)};
      float d[3] = {0.0f, 0.0f, 0.0f};
      if (s->off0[r] != 0.0f || s->off1[r] != 0.0f) direction(m.rng, q.i, t, T_BIMDIR, q.j, d);
      const Rec dead{0.0f, 0.0f, 0.0f, DEAD};
      // a product moves from the reaction point by its offset (through the
      // surfaces), then the walls reflect it
      auto product = [&](int sp, float off) {
        if (sp < 0) return dead;
        float e[3];
        for (int a = 0; a < 3; a++) e[a] = wall(std::fmaf(off, d[a], rp[a]), s->lo[a], s->hi[a]);
        if (s->n_panels > 0 && off != 0.0f && !walk_in_box(s, sp, rp, e)) return dead;
        return Rec{e[0], e[1], e[2], pack(s->inst, sp)};
      };
      const Rec n1 = product(s->prod0[r], s->off0[r]);
      const Rec n2 = product(s->prod1[r], s->off1[r]);
      res[m1] = n1;
      res[m2] = n2;
      ev_total[r]++;
    }
    for (Rec& q : res)
      if (q.w != DEAD) q.w &= ~NEWBORN;
    npairs = (uint32_t)cand.size();
    if (pairs)
      for (size_t k = 0; k < cand.size() && k < pairs_cap; k++) {
        pairs[4 * k] = cand[k].i;
        pairs[4 * k + 1] = cand[k].j;
        pairs[4 * k + 2] = (uint32_t)cand[k].r;
        pairs[4 * k + 3] = acc[k];
      }
  }
  if (n_pairs) *n_pairs = npairs;
  *n_out = (uint32_t)res.size();
  if (events)
    for (int r = 0; r < R; r++) events[r] += ev_total[r];
  if (res.size() > cap) return -1;
  for (size_t q = 0; q < res.size(); q++) {
    out[4 * q] = fbits(res[q].x);
    out[4 * q + 1] = fbits(res[q].y);
    out[4 * q + 2] = fbits(res[q].z);
    out[4 * q + 3] = res[q].w;
  }
  return 0;
}

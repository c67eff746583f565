// sanitize_main.cpp -- TEST INFRASTRUCTURE, not part of the product.
//
// Runs the oracle's step (oracle.cpp) on small systems that reach every
// branch the tests rely on -- zeroth-, first- and second-order reactions,
// a decay, two products placed with offsets, a reflecting sphere and an
// absorbing plane, the cell-sorted and the in-place pipeline -- so that
// tests/test_oracle_sanitizers.py can build it with AddressSanitizer and
// UndefinedBehaviorSanitizer and check that the oracle itself is clean.
// Exit status 0 when every step returned 0 and every count stayed in
// bounds.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "oracle.h"

namespace {

uint32_t fbits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, sizeof u);
  return u;
}

// Poisson(mean) CDF over [0, kmax]; the last value is 1.
std::vector<double> poisson_cdf(double mean, int kmax) {
  std::vector<double> c;
  double acc = 0, term = std::exp(-mean);
  for (int k = 0; k <= kmax; ++k) {
    acc += term;
    c.push_back(acc < 1.0 ? acc : 1.0);
    term *= mean / (k + 1);
  }
  c.back() = 1.0;
  return c;
}

std::vector<uint32_t> uniform_records(uint32_t n, int species_mod, uint32_t seed) {
  std::mt19937 g(seed);
  std::uniform_real_distribution<float> u(0.0f, 4.0f);
  std::vector<uint32_t> r(4 * (size_t)n);
  for (uint32_t i = 0; i < n; ++i) {
    r[4 * i] = fbits(u(g));
    r[4 * i + 1] = fbits(u(g));
    r[4 * i + 2] = fbits(u(g));
    r[4 * i + 3] = (uint32_t)(i % (uint32_t)species_mod);
  }
  return r;
}

int run(or_system& s, uint32_t n0, int steps, const char* name) {
  std::vector<uint32_t> cur = uniform_records(n0, s.S, 7u);
  uint32_t n = n0;
  const uint32_t cap = 4 * n0 + 1024;
  const uint64_t ncells = (uint64_t)s.dims[0] * s.dims[1] * s.dims[2];
  std::vector<uint32_t> out(4 * (size_t)cap), cells(ncells + 1), pairs(4 * 4096);
  std::vector<uint64_t> events(s.R > 0 ? s.R : 1, 0);
  for (int t = 0; t < steps; ++t) {
    uint32_t n_out = 0, n_pairs = 0;
    const int rc = or_step(&s, (uint32_t)t, cur.data(), n, out.data(), cap, &n_out, cells.data(), ncells + 1,
                           pairs.data(), 4096, &n_pairs, events.data());
    if (rc != 0 || n_out > cap || n_pairs > 4096) {
      std::fprintf(stderr, "%s: step %d returned %d (n_out %u, n_pairs %u)\n", name, t, rc, n_out, n_pairs);
      return 1;
    }
    cur.assign(out.begin(), out.begin() + 4 * (size_t)n_out);
    n = n_out;
  }
  std::printf("%s: %d steps, %u records\n", name, steps, n);
  return 0;
}

}  // namespace

int main() {
  // box [0, 4]^3 of unit cells
  or_system s;
  std::memset(&s, 0, sizeof s);
  for (int k = 0; k < 3; ++k) {
    s.lo[k] = 0.0f;
    s.hi[k] = 4.0f;
    s.inv[k] = 1.0f;
    s.cell[k] = 1.0f;
    s.dims[k] = 4;
  }
  s.key_lo = 11;
  s.key_hi = 12;
  s.normal_mode = 0;
  std::vector<float> gauss(4096);
  for (int i = 0; i < 4096; ++i) gauss[i] = (float)(((i + 0.5) / 4096.0 - 0.5) * 6.0);
  s.gauss = gauss.data();
  // species A, B, C
  const float D[3] = {1.0f, 1.0f, 0.5f};
  s.S = 3;
  s.D = D;
  s.dt = 1e-3f;
  // A + B -> C; C -> A + B with offsets; -> A (zeroth order); B -> 0
  const int order[4] = {2, 1, 0, 1}, react0[4] = {0, 2, -1, 1}, react1[4] = {1, -1, -1, -1};
  const int prod0[4] = {2, 0, 0, -1}, prod1[4] = {-1, 1, -1, -1};
  const float prob[4] = {0.5f, 0.02f, 2.0f, 0.01f}, bind[4] = {0.2f, 0.0f, 0.0f, 0.0f};
  const float off0[4] = {0.0f, 0.05f, 0.0f, 0.0f}, off1[4] = {0.0f, 0.05f, 0.0f, 0.0f};
  const float thresh[4] = {1.0f, 1.0f, 1.0f, 1.0f};
  const std::vector<double> cdf = poisson_cdf(2.0, 40);
  const int cdf_off[4] = {0, 0, 0, 0}, cdf_len[4] = {0, 0, (int)cdf.size(), 0}, cdf_kmin[4] = {0, 0, 0, 0};
  s.R = 4;
  s.order = order;
  s.react0 = react0;
  s.react1 = react1;
  s.prod0 = prod0;
  s.prod1 = prod1;
  s.prob = prob;
  s.bind_radius = bind;
  s.off0 = off0;
  s.off1 = off1;
  s.cdf = cdf.data();
  s.cdf_off = cdf_off;
  s.cdf_len = cdf_len;
  s.cdf_kmin = cdf_kmin;
  s.thresh = thresh;
  s.sorted = 1;
  s.threads = 1;
  // surface 0: a reflecting sphere (centre (2, 2, 2), radius 1, front
  // outside); surface 1: a plane x = 3.5 that absorbs B from its front
  or_panel p[2];
  std::memset(p, 0, sizeof p);
  p[0].shape = 2;
  p[0].surface = 0;
  p[0].front = 1.0f;
  p[0].a[0] = p[0].a[1] = p[0].a[2] = 2.0f;
  p[0].r = 1.0f;
  p[0].r2 = 1.0f;
  p[1].shape = 0;
  p[1].surface = 1;
  p[1].axis = 0;
  p[1].front = -1.0f;
  p[1].a[0] = 3.5f;
  p[1].n[0] = 1.0f;
  p[1].bounds[0] = 0.0f;
  p[1].bounds[1] = 4.0f;
  p[1].bounds[2] = 0.0f;
  p[1].bounds[3] = 4.0f;
  uint8_t act[2 * 3 * 2];
  for (int sp = 0; sp < 3; ++sp) {
    act[(0 * 3 + sp) * 2 + 0] = act[(0 * 3 + sp) * 2 + 1] = 1;  // reflect
    act[(1 * 3 + sp) * 2 + 0] = sp == 1 ? 2 : 0;                 // B absorbed from the front
    act[(1 * 3 + sp) * 2 + 1] = 0;
  }
  int bad = 0;
  bad |= run(s, 3000, 25, "reacting, no panels");
  s.n_panels = 2;
  s.panels = p;
  s.surf_act = act;
  bad |= run(s, 3000, 25, "reacting, sphere and plane");
  s.channels = 1;
  bad |= run(s, 3000, 10, "reacting, competing channels");
  // diffusion only, in place
  or_system d = s;
  d.R = 0;
  d.sorted = 0;
  d.n_panels = 0;
  d.panels = nullptr;
  d.surf_act = nullptr;
  d.channels = 0;
  bad |= run(d, 2000, 10, "diffusion only");
  return bad;
}

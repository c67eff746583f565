// bd_params.cpp -- reaction-parameter derivation on the host.
//
// rxnparam part: the Andrews-Bray lookup functions (S. S. Andrews and
// D. Bray, Phys. Biol. 1:137, 2004), restated from the published method and
// evaluated on tables regenerated by rate_tables_gen.py.  The interpolation
// (cubic Lagrange in ln(step/a), then in b/a or ln(b/a)), the stencil rules
// at the table edges and the bisection searches follow the reference
// (rxnparam.cpp:42-308) operation for operation, so binding and unbinding
// radii come out with the same bits.
//
// Reaction part: rxnsetrate / rxnsetproduct (smolreact.cpp:283-483) with
// Smoldyn's intended treatment of reversible reactions -- the binding radius
// is calibrated with the actual unbinding radius b, which is solved from the
// geminate-recombination probability -- instead of the reference's literal
// code, which computes b from a probability it never sets and always uses
// the irreversible radius.
#include "bd_params.h"

#include <math.h>

#include <algorithm>
#include <cmath>

#include "../../include/gpusmoldyn.h"
#include "rate_tables.h"

namespace bd {
namespace {

constexpr double kPi = 3.14159265358979323846;

// Weights of the cubic through 4 nodes x[0..3] spaced h apart, at point s.
// The denominators are multiplied left to right as in rxnparam.cpp:174-177.
inline void cubic_weights(double s, const double x[4], double h, double z[4]) {
  z[0] = (s - x[1]) * (s - x[2]) * (s - x[3]) / (-6.0 * h * h * h);
  z[1] = (s - x[0]) * (s - x[2]) * (s - x[3]) / (2.0 * h * h * h);
  z[2] = (s - x[0]) * (s - x[1]) * (s - x[3]) / (-2.0 * h * h * h);
  z[3] = (s - x[0]) * (s - x[1]) * (s - x[2]) / (6.0 * h * h * h);
}

}  // namespace

double numrxnrate(double step, double a, double b) {
  using namespace bd_tables;
  const double s0 = 3.0, ds = -0.2;   // ln(step/a) of column 0 and spacing
  const double bf0 = 0.0, dbf = 0.2;  // ln(b/a) of row 0 of kRevFar, spacing
  const double bn0 = 0.0, dbn = 0.1;  // b/a of row 0 of kRevNear, spacing
  if (step < 0 || a < 0) return -1;
  if (step == 0 && b >= 0 && b < 1) return -1;
  if (step == 0) return 0;
  const double ls = log(step / a);
  b /= a;

  int col = (int)((ls - s0) / ds);
  double x[4], z[4], y[4];
  for (int i = 0; i < 4; i++) x[i] = s0 + (col - 1 + i) * ds;
  cubic_weights(ls, x, ds, z);

  double ans;
  if (b < 0) {
    // irreversible: beyond the small-step end the Smoluchowski limit
    // 2 pi (s/a)^2, beyond the large-step end the well-mixed 4 pi / 3
    ans = 0;
    for (int i = 0; i < 4; i++) {
      const int c = col - 1 + i;
      if (c >= kSteps) ans += z[i] * 2.0 * kPi * exp(2.0 * x[i]);
      else if (c < 0) ans += z[i] * 4.0 * kPi / 3.0;
      else ans += z[i] * kIrrev[c];
    }
  } else if (b < 1.0) {
    int row = (int)((b - bn0) / dbn);
    if (row < 1) row = 1;
    else if (row + 2 >= kRowsB) row = kRowsB - 3;
    // move the stencil away from diverged (-1) entries
    while (col + 3 >= kSteps || (col > 0 && kRevNear[(row - 1) * kSteps + col + 3] < 0)) col--;
    for (int i = 0; i < 4; i++) x[i] = s0 + (col - 1 + i) * ds;
    cubic_weights(ls, x, ds, z);
    for (int j = 0; j < 4; j++) {
      y[j] = 0;
      for (int i = 0; i < 4; i++) {
        const int c = col - 1 + i;
        if (c >= kSteps) y[j] += z[i] * kRevNear[(row - 1 + j) * kSteps];
        else if (c < 0) y[j] += z[i] * 4.0 * kPi / 3.0;
        else y[j] += z[i] * kRevNear[(row - 1 + j) * kSteps + c];
      }
    }
    for (int j = 0; j < 4; j++) x[j] = bn0 + (row - 1 + j) * dbn;
    cubic_weights(b, x, dbn, z);
    ans = z[0] * y[0] + z[1] * y[1] + z[2] * y[2] + z[3] * y[3];
  } else {
    b = log(b);
    int row = (int)((b - bf0) / dbf);
    if (row < 1) row = 1;
    else if (row + 2 >= kRowsR) row = kRowsR - 3;
    for (int j = 0; j < 4; j++) {
      y[j] = 0;
      for (int i = 0; i < 4; i++) {
        const int c = col - 1 + i;
        if (c >= kSteps && b == 0) y[j] += z[i] * 2.0 * kPi * exp(x[i]) * (1.0 + exp(x[i]));
        else if (c >= kSteps) y[j] += z[i] * 2.0 * kPi * exp(2.0 * x[i]) * exp(b) / (exp(b) - 1.0);
        else if (c < 0) y[j] += z[i] * 4.0 * kPi / 3.0;
        else y[j] += z[i] * kRevFar[(row - 1 + j) * kSteps + c];
      }
    }
    for (int j = 0; j < 4; j++) x[j] = bf0 + (row - 1 + j) * dbf;
    cubic_weights(b, x, dbf, z);
    ans = z[0] * y[0] + z[1] * y[1] + z[2] * y[2] + z[3] * y[3];
  }
  return ans * a * a * a;
}

// Activation-limited rate (rxnparam.cpp:226-239): the rate if the pair
// distribution stayed uniform outside a.  std::erfc replaces the reference's
// rational approximation (relative error < 1.2e-7).
double actrxnrate(double step, double a) {
  if (step < 0 || a <= 0) return -1;
  if (step == 0) return 0;
  step /= a;
  double ka = 4.0 * kPi / 3.0 * (std::erfc(sqrt(2.0) / step) + step * sqrt(2.0 / kPi));
  ka += 2.0 * sqrt(2.0 * kPi) / 3.0 * step * (step * step - 1.0) * (exp(-2.0 / step / step) - 1.0);
  return ka * a * a * a;
}

// Binding radius for a rate constant (rxnparam.cpp:242-277): doubling
// search then 15 bisections on the monotone numrxnrate(step, a, b).
double bindingradius(double rate, double dt, double difc, double b, int rel) {
  if (rate < 0 || dt < 0 || difc <= 0) return -1;
  if (rate == 0) return 0;
  if (dt == 0) {
    if (b < 0) return rate / (4 * kPi * difc);
    if (rel && b > 1) return rate * (1 - 1 / b) / (4 * kPi * difc);
    if (rel && b <= 1) return -1;
    if (b > 0) return rate / (4 * kPi * difc + rate / b);
    return -1;
  }
  const double step = sqrt(2.0 * difc * dt);
  double lo = 0, a = step;
  while (numrxnrate(step, a, rel ? b * a : b) < rate * dt) {
    lo = a;
    a *= 2.0;
  }
  double dif = a - lo;
  for (int n = 0; n < 15; n++) {
    dif *= 0.5;
    a = lo + dif;
    if (numrxnrate(step, a, rel ? b * a : b) < rate * dt) lo = a;
  }
  return lo + 0.5 * dif;
}

// Unbinding radius for a geminate-recombination probability
// (rxnparam.cpp:280-308); returns -2 for illegal input and -pgem_max when
// the request exceeds the attainable maximum (reached at b = 0).
double unbindingradius(double pgem, double dt, double difc, double a) {
  if (pgem <= 0 || pgem >= 1 || difc <= 0 || a <= 0 || dt < 0) return -2;
  if (dt == 0) return a / pgem;
  const double step = sqrt(2.0 * difc * dt);
  const double ki = numrxnrate(step, a, -1);
  const double kmax = numrxnrate(step, a, 0);
  if (1.0 - ki / kmax < pgem) return ki / kmax - 1.0;
  double lo = 0, b = a;
  while (1.0 - ki / numrxnrate(step, a, b) > pgem) {
    lo = b;
    b *= 2.0;
  }
  double dif = b - lo;
  for (int n = 0; n < 15; n++) {
    dif *= 0.5;
    b = lo + dif;
    if (1.0 - ki / numrxnrate(step, a, b) > pgem) lo = b;
  }
  return lo + 0.5 * dif;
}

void gauss_quantiles(float* out, int n) {
  // Phi^-1((i + 1/2) / n) by bisection on the normal CDF in double precision;
  // the table is antisymmetric like the reference's (stats.cpp:202-211).
  for (int i = 0; i < n / 2; i++) {
    const double p = (i + 0.5) / n;
    double lo = -40.0, hi = 0.0;
    for (int it = 0; it < 200 && hi - lo > 0; it++) {
      const double mid = 0.5 * (lo + hi);
      if (mid == lo || mid == hi) break;
      if (0.5 * std::erfc(-mid / sqrt(2.0)) < p) lo = mid;
      else hi = mid;
    }
    out[i] = (float)(0.5 * (lo + hi));
    out[n - 1 - i] = -out[i];
  }
}

void poisson_cdf(double mean, std::vector<double>* cdf, int* kmin) {
  cdf->clear();
  if (!(mean > 0)) {
    *kmin = 0;
    cdf->push_back(1.0);
    return;
  }
  const double sd = sqrt(mean);
  const int lo = std::max(0, (int)floor(mean - 12.0 * sd - 10.0));
  const int hi = (int)ceil(mean + 12.0 * sd + 10.0);
  const double lm = log(mean);
  double acc = 0;
  for (int k = lo; k <= hi; k++) {
    acc += exp(-mean + k * lm - std::lgamma(k + 1.0));
    cdf->push_back(std::min(acc, 1.0));
  }
  cdf->back() = 1.0;
  *kmin = lo;
}

namespace {

bool same_pair(const int a[2], const int b[2]) {
  return (a[0] == b[0] && a[1] == b[1]) || (a[0] == b[1] && a[1] == b[0]);
}

// The reaction that undoes r (findreverserxn, smolreact.cpp:73-146): its
// order equals r's product count, its reactants are r's products and its
// products are r's reactants.
int find_reverse(const std::vector<ReactionDef>& rx, int r) {
  const ReactionDef& f = rx[r];
  if (f.order == 0 || f.nprod < 1) return -1;
  for (int q = 0; q < (int)rx.size(); q++) {
    if (q == r) continue;
    const ReactionDef& g = rx[q];
    if (g.order != f.nprod || g.nprod != f.order) continue;
    bool rct, prd;
    if (g.order == 1) rct = g.reactants[0] == f.products[0];
    else rct = same_pair(g.reactants, f.products);
    if (f.order == 1) prd = g.products[0] == f.reactants[0];
    else prd = same_pair(g.products, f.reactants);
    if (rct && prd) return q;
  }
  return -1;
}

void set_status(DerivedParams* P, int code, const std::string& msg) {
  if (P->status == 0) {
    P->status = code;
    P->message = msg;
  }
}

}  // namespace

DerivedParams derive_params(const std::vector<float>& D0, const std::vector<ReactionDef>& rx, float dt,
                            float volume, float d_scale, float k2_scale, bool channels) {
  DerivedParams P;
  const int S = (int)D0.size(), R = (int)rx.size();
  P.D.resize(S);
  P.sigma.resize(S);
  for (int s = 0; s < S; s++) {
    P.D[s] = D0[s] * d_scale;
    // molSetTimestep (particleSystem.cpp:137-142)
    P.sigma[s] = sqrtf(2.0f * P.D[s] * dt);
  }
  P.rx.assign(R, DerivedReaction());
  P.cdf.assign(R, std::vector<double>());
  P.cdf_kmin.assign(R, 0);
  for (int r = 0; r < R; r++) P.rx[r].reverse = find_reverse(rx, r);
  // channel mode: reactant pairs with several second-order reactions
  std::vector<std::vector<int>> groups;
  std::vector<int> group_of(R, -1);
  if (channels) {
    for (int r = 0; r < R; r++) {
      if (rx[r].order != 2 || !(rx[r].rate > 0)) continue;
      const int a = std::min(rx[r].reactants[0], rx[r].reactants[1]);
      const int b = std::max(rx[r].reactants[0], rx[r].reactants[1]);
      int g = -1;
      for (size_t k = 0; k < groups.size() && g < 0; k++) {
        const ReactionDef& f = rx[groups[k][0]];
        if (std::min(f.reactants[0], f.reactants[1]) == a && std::max(f.reactants[0], f.reactants[1]) == b)
          g = (int)k;
      }
      if (g < 0) {
        g = (int)groups.size();
        groups.emplace_back();
      }
      groups[g].push_back(r);
      group_of[r] = g;
    }
    for (const std::vector<int>& m : groups) {
      if (m.size() < 2) continue;
      // competing reactions are calibrated as irreversible (b = 0): the
      // reversible coupling of one reaction to its reverse is per pair
      for (int r : m) {
        const int u = P.rx[r].reverse;
        if (u >= 0) P.rx[u].reverse = -1;
        P.rx[r].reverse = -1;
      }
    }
  }

  // order 0: Poisson mean k dt V (smolreact.cpp:295-303)
  for (int r = 0; r < R; r++) {
    if (rx[r].order != 0) continue;
    if (rx[r].rate < 0) {
      set_status(&P, BD_ERR_NEGATIVE_RATE, "negative zeroth-order rate");
      continue;
    }
    P.rx[r].prob = rx[r].rate * dt * volume;
    poisson_cdf(P.rx[r].prob, &P.cdf[r], &P.cdf_kmin[r]);
  }

  // order 1: probabilities conditioned on the earlier reactions of the same
  // reactant, in reaction-index order (smolreact.cpp:304-353)
  for (int r = 0; r < R; r++) {
    if (rx[r].order != 1) continue;
    if (rx[r].rate < 0) {
      set_status(&P, BD_ERR_NEGATIVE_RATE, "negative first-order rate");
      continue;
    }
    const int sp = rx[r].reactants[0];
    float sum = 0;
    for (int q = 0; q < R; q++)
      if (rx[q].order == 1 && rx[q].reactants[0] == sp && rx[q].rate > 0) sum += rx[q].rate;
    if (rx[r].rate == 0) {
      P.rx[r].prob = 0;
      continue;
    }
    float prob = 0;
    if (sum > 0) {
      const float e = std::exp(-dt * sum);
      prob = rx[r].rate / sum * (1.0f - e);
    }
    float prior = 0;
    for (int q = 0; q < r; q++)
      if (rx[q].order == 1 && rx[q].reactants[0] == sp) prior += P.rx[q].prob;
    P.rx[r].prob = prob / (1.0f - prior);
  }

  // order 2: binding radius (smolreact.cpp:354-395), with the reversible
  // coupling to the unbinding radius of the reverse reaction
  for (int r = 0; r < R; r++) {
    if (rx[r].order != 2) continue;
    DerivedReaction& d = P.rx[r];
    d.prob = rx[r].user_prob >= 0.0f ? rx[r].user_prob : 1.0f;
    const int i1 = rx[r].reactants[0], i2 = rx[r].reactants[1];
    if (rx[r].rate < 0) {
      set_status(&P, BD_ERR_NEGATIVE_RATE, "negative second-order rate");
      continue;
    }
    float rate3 = rx[r].rate * k2_scale;
    const int g = group_of[r];
    if (g >= 0 && groups[g].size() > 1) {
      // one radius for the pair from the summed rate; each reaction's share
      // of it picks the reaction of an accepted pair
      float total = 0.0f, upto = 0.0f;
      for (int m : groups[g]) total += rx[m].rate;
      for (size_t k = 0; k < groups[g].size(); k++) {
        const int m = groups[g][k];
        upto += rx[m].rate;
        if (m == r) {
          d.thresh = k + 1 == groups[g].size() ? 1.0f : upto / total;
          d.next = k + 1 < groups[g].size() ? groups[g][k + 1] : -1;
        }
      }
      if (rx[r].user_prob >= 0.0f) {
        set_status(&P, BD_ERR_UNSUPPORTED, "a reaction probability on competing reactions of one pair");
        continue;
      }
      rate3 = total * k2_scale;
    }
    if (i1 == i2) rate3 *= 2;
    const float dsum = P.D[i1] + P.D[i2];
    const float D1 = P.D[i1], D2 = P.D[i2];
    d.x = (D1 == 0 && D2 == 0) ? 0.5f : D2 / (D1 + D2);
    d.omx = 1.0f - d.x;
    if (rate3 <= 0) {
      d.bind_r2 = 0;
      continue;
    }
    if (dsum <= 0) {
      set_status(&P, BD_ERR_ZERO_DIFFUSION, "both reactant diffusion coefficients are 0");
      continue;
    }
    double a;
    const int u = d.reverse;
    if (u >= 0 && rx[u].order == 1 && rx[u].nprod == 2) {
      int kind = rx[u].pp_kind;
      double p = rx[u].pp_param;
      if (kind == BD_PP_DEFAULT) {
        kind = BD_PP_PGEMMAX;
        p = 0.2;
      }
      double b = 0;
      const double step = sqrt(2.0 * (double)dsum * (double)dt);
      if (kind == BD_PP_UNBINDRAD) {
        b = p;
        a = bindingradius(rate3, dt, dsum, b, 0);
      } else if (kind == BD_PP_OFFSET0) {
        a = bindingradius(rate3, dt, dsum, 0, 0);
      } else {
        const double a0 = bindingradius(rate3, dt, dsum, 0, 0);
        const double pmax = 1.0 - numrxnrate(step, a0, -1) / numrxnrate(step, a0, 0);
        if (!(p > 0 && p < 1)) {
          set_status(&P, BD_ERR_ILLEGAL_UNBIND, "geminate probability outside (0, 1)");
          a = a0;
        } else if (p >= pmax) {
          if (kind == BD_PP_PGEM)
            set_status(&P, BD_ERR_PGEM_UNATTAINABLE, "requested geminate probability exceeds the maximum");
          a = a0;
          P.rx[u].flags |= 1;
          P.rx[u].gem_prob = (float)pmax;
        } else {
          // fixed point: b from pgem at the current a, then a from the rate at b
          a = a0;
          for (int it = 0; it < 200; it++) {
            b = unbindingradius(p, dt, dsum, a);
            if (b < 0) break;
            const double an = bindingradius(rate3, dt, dsum, b, 0);
            const bool done = fabs(an - a) <= 1e-9 * a;
            a = an;
            if (done) break;
          }
          if (b < 0) {
            set_status(&P, BD_ERR_PGEM_UNATTAINABLE, "geminate probability unattainable");
            b = 0;
            a = a0;
            P.rx[u].flags |= 1;
          }
          P.rx[u].gem_prob = (float)p;
        }
      }
      P.rx[u].unbind_radius = (float)b;
    } else {
      a = bindingradius(rate3, dt, dsum, -1, 0);
    }
    d.bind_radius = (float)a;
    d.bind_r2 = d.bind_radius * d.bind_radius;
  }

  // product placement (rxnsetproduct, smolreact.cpp:410-483): two products
  // sit at +b D1/(D1+D2) and -b D2/(D1+D2) along one random direction
  for (int r = 0; r < R; r++) {
    if (rx[r].nprod != 2) continue;
    DerivedReaction& d = P.rx[r];
    float dc1 = P.D[rx[r].products[0]], dc2 = P.D[rx[r].products[1]];
    float dsum = dc1 + dc2;
    float b = d.unbind_radius;
    const bool coupled = d.reverse >= 0 && rx[d.reverse].order == 2 && rx[r].order == 1;
    if (!coupled) {
      b = rx[r].pp_kind == BD_PP_UNBINDRAD ? rx[r].pp_param : 0.0f;
      d.unbind_radius = b;
      if (dsum == 0) {
        dc1 = 1.0f;
        dc2 = 1.0f;
        dsum = 0.5f;
      }
    } else if (dsum <= 0) {
      set_status(&P, BD_ERR_ZERO_DIFFUSION, "sum of product diffusion coefficients is 0");
      continue;
    }
    d.off[0] = b * dc1 / dsum;
    d.off[1] = -b * dc2 / dsum;
  }
  return P;
}

}  // namespace bd

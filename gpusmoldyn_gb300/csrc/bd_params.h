// bd_params.h -- host-side reaction-parameter derivation.
#pragma once
#include <stdint.h>

#include <string>
#include <vector>

namespace bd {

// rxnparam restatements (Andrews-Bray tables, rxnparam.cpp:42-308).
double numrxnrate(double step, double a, double b);
double actrxnrate(double step, double a);
double bindingradius(double rate, double dt, double difc, double b, int rel);
double unbindingradius(double pgem, double dt, double difc, double a);

// 4096 standard-normal quantiles at (i + 1/2) / n, ascending.
void gauss_quantiles(float* out, int n);

struct ReactionDef {
  int order = 0;
  int reactants[2] = {-1, -1};
  int products[2] = {-1, -1};
  int nprod = 0;
  float rate = 0.0f;
  int pp_kind = 0;       // BD_PP_*
  float pp_param = 0.0f;
  float user_prob = -1.0f;  // order 2: per-encounter probability, < 0 = 1
};

struct DerivedReaction {
  float prob = 0.0f;          // per-step probability (order 0: Poisson mean)
  float bind_radius = 0.0f;   // order 2
  float bind_r2 = 0.0f;       // order 2, bind_radius^2 in float
  float unbind_radius = 0.0f; // for the products of this reaction
  float gem_prob = 0.0f;
  float off[2] = {0.0f, 0.0f};
  float x = 0.5f, omx = 0.5f; // order 2 reaction point weights
  int reverse = -1;
  int flags = 0;              // bit 0: pgem fell back to b = 0
  // competing second-order reactions of one reactant pair (channel mode):
  // cumulative share of the pair's total rate up to this reaction, and the
  // next reaction of the pair (-1: last)
  float thresh = 1.0f;
  int next = -1;
};

struct DerivedParams {
  std::vector<float> D;       // per species, scaled
  std::vector<float> sigma;   // sqrt(2 D dt) per species
  std::vector<DerivedReaction> rx;
  std::vector<std::vector<double>> cdf;   // per reaction (order 0 only)
  std::vector<int> cdf_kmin;
  int status = 0;             // first setup error (BD_ERR_* / reference codes)
  std::string message;
};

// Derive every reaction's parameters for one parameter block.  d_scale and
// k2_scale multiply the diffusion coefficients and the second-order rates
// (ensemble instances); volume is the box volume (zeroth order).
// channels: second-order reactions that share a reactant pair compete (one
// binding radius from their summed rate, the reaction picked by its share of
// it); otherwise the last listed reaction of a pair is the pair's reaction.
DerivedParams derive_params(const std::vector<float>& D, const std::vector<ReactionDef>& rx, float dt,
                            float volume, float d_scale, float k2_scale, bool channels = false);

// Poisson CDF over [kmin, kmin + len) covering all but ~1e-30 of the mass.
void poisson_cdf(double mean, std::vector<double>* cdf, int* kmin);

}  // namespace bd

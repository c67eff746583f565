// ref_kat.cpp -- TEST INFRASTRUCTURE: known-answer driver linked against the
// reference's own host sources (rxnparam.cpp, smolreact.cpp, stats.cpp,
// SFMT/SFMT.cpp, rnd/genmtrand.cpp, reaction_cpu.cpp), compiled where they
// lie by oracle/build.py into oracle/_ref/.  It prints, as JSON, the values
// the reference computes for the parameter derivation of the step:
// numrxnrate / actrxnrate / bindingradius / unbindingradius on a grid,
// rxnsetrate + rxnsetproduct results for small networks, the normal-quantile
// table, and Poisson sample moments.  tests/golden/reference_kat.json is its
// output; the library's restatements are checked against that file.
#include <math.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "particleSystem.h"
#include "rxnparam.h"
#include "smolreact.h"
#include "stats.h"

// The reference's destructor lives in particleSystem.cpp (GL and CUDA code);
// the setup functions only need the object's fields.
ParticleSystem::~ParticleSystem() {}

void randtableF(float* a, int n, int eq);  // stats.cpp:202

// JSON goes to the file named on the command line; the reference writes its
// own diagnostics to stdout.
static FILE* g_out = stdout;

// Sets the protected fields the setup code reads (getDeltaTime,
// getSystemVolume, getDiffusionCoefficients, reactionOrderInfo).
class KatSystem : public ParticleSystem {
 public:
  KatSystem(float dt, float vol, const std::vector<float>& D) {
    deltaTime = dt;
    systemVolume = vol;
    m_numTypes = (uint)D.size();
    m_hDiffusionCoefficients = new float[D.size()];
    for (size_t i = 0; i < D.size(); i++) m_hDiffusionCoefficients[i] = D[i];
  }
};

struct Rx {
  int order;
  int r0, r1, p0, p1, nprod;
  float rate;
};

static void run_network(const char* name, float dt, float vol, const std::vector<float>& D, const std::vector<Rx>& rx,
                        bool last) {
  KatSystem sim(dt, vol, D);
  const int R = (int)rx.size();
  Reaction* L = new Reaction;
  L->order = new int[R];
  L->bindRadiusSquared = new float[R];
  L->unbindRadius = new float[R];
  L->geminateProbability = new float[R];
  L->prob = new float[R];
  L->rate = new float[R];
  L->nprod = new int[R];
  L->products = new int2[R];
  L->reactants = new int2[R];
  L->productPositions = new float[R * 6];
  int per[3] = {0, 0, 0};
  for (int i = 0; i < R; i++) {
    L->order[i] = rx[i].order;
    L->rate[i] = rx[i].rate;
    L->prob[i] = 1.0f;
    L->nprod[i] = rx[i].nprod;
    L->reactants[i].x = rx[i].r0;
    L->reactants[i].y = rx[i].r1;
    L->products[i].x = rx[i].p0;
    L->products[i].y = rx[i].p1;
    L->unbindRadius[i] = 0.0f;
    L->geminateProbability[i] = 0.0f;
    L->bindRadiusSquared[i] = 0.0f;
    for (int k = 0; k < 6; k++) L->productPositions[6 * i + k] = 0.0f;
    per[rx[i].order]++;
  }
  fillReactionOrderInfo(per, R, L, sim.reactionOrderInfo, (int)D.size());
  fprintf(g_out, "  \"%s\": {\"dt\": %.9g, \"volume\": %.9g, \"reactions\": [\n", name, dt, vol);
  for (int i = 0; i < R; i++) {
    const int e1 = rxnsetrate(i, L, &sim);
    const int e2 = rxnsetproduct(&sim, L, L->order[i], i);
    fprintf(g_out, "    {\"order\": %d, \"rate\": %.9g, \"prob\": %.9g, \"bind_r2\": %.9g, \"unbind\": %.9g, "
           "\"offsets\": [%.9g, %.9g], \"rxnsetrate\": %d, \"rxnsetproduct\": %d}%s\n",
           L->order[i], L->rate[i], L->prob[i], L->bindRadiusSquared[i], L->unbindRadius[i],
           L->productPositions[6 * i], L->productPositions[6 * i + 3], e1, e2, i + 1 < R ? "," : "");
  }
  fprintf(g_out, "  ]}%s\n", last ? "" : ",");
}

int main(int argc, char** argv) {
  if (argc > 1) g_out = fopen(argv[1], "w");
  if (!g_out) return 1;
  fprintf(g_out, "{\n");
  // numrxnrate on a grid of reduced step lengths and unbinding radii
  fprintf(g_out, "  \"numrxnrate\": [\n");
  const double bs[] = {-1.0, 0.0, 0.05, 0.2, 0.45, 0.5, 0.77, 0.95, 1.0, 1.3, 2.0, 5.0, 12.0, 25.0};
  bool first = true;
  for (double ls = -4.0; ls <= 4.0001; ls += 0.137) {
    for (double b : bs) {
      const double step = exp(ls), a = 0.37;
      const double v = numrxnrate(step * a, a, b < 0 ? -1.0 : b * a);
      fprintf(g_out, "%s    [%.17g, %.17g, %.17g, %.17g]", first ? "" : ",\n", step * a, a, b < 0 ? -1.0 : b * a, v);
      first = false;
    }
  }
  fprintf(g_out, "\n  ],\n");
  fprintf(g_out, "  \"actrxnrate\": [\n");
  first = true;
  for (double ls = -3.0; ls <= 3.0001; ls += 0.5) {
    fprintf(g_out, "%s    [%.17g, %.17g, %.17g]", first ? "" : ",\n", exp(ls), 1.0, actrxnrate(exp(ls), 1.0));
    first = false;
  }
  fprintf(g_out, "\n  ],\n");
  // bindingradius(rate, dt, difc, b, rel)
  fprintf(g_out, "  \"bindingradius\": [\n");
  struct B {
    double rate, dt, difc, b;
    int rel;
  };
  const B bcases[] = {{0.01, 1e-3, 2.0, -1, 0},  {0.05, 5e-4, 2.0, -1, 0}, {0.05, 5e-4, 2.0, 0, 0},
                      {0.05, 5e-4, 2.0, 0.03, 0}, {0.02, 1e-3, 1.0, -1, 0}, {0.1, 1e-3, 20.0, -1, 0},
                      {0.01, 1e-3, 0.2, -1, 0},  {0.2, 1e-3, 0.5, -1, 0},  {1.0, 1e-2, 0.1, -1, 0},
                      {0.05, 5e-4, 2.0, 2.0, 1},  {0.05, 0.0, 2.0, -1, 0},  {0.05, 5e-4, 2.0, 0.5, 1},
                      {2000, 0.1, 0.002, -1, 0},  {0.01, 1e-3, 0.1, -1, 0}, {0.3, 1e-4, 3.0, -1, 0}};
  first = true;
  for (const B& c : bcases) {
    fprintf(g_out, "%s    [%.17g, %.17g, %.17g, %.17g, %d, %.17g]", first ? "" : ",\n", c.rate, c.dt, c.difc, c.b, c.rel,
           bindingradius(c.rate, c.dt, c.difc, c.b, c.rel));
    first = false;
  }
  fprintf(g_out, "\n  ],\n");
  // unbindingradius(pgem, dt, difc, a)
  fprintf(g_out, "  \"unbindingradius\": [\n");
  const double a2 = bindingradius(0.05, 5e-4, 2.0, 0, 0);
  const double ucases[][4] = {{0.2, 5e-4, 2.0, a2},   {0.02, 5e-4, 2.0, a2},  {0.04, 5e-4, 2.0, a2},
                              {0.2, 1e-3, 1.0, 0.05}, {0.5, 1e-2, 0.1, 0.05}, {0.3, 0.0, 1.0, 0.1},
                              {0.1, 1e-3, 0.5, 0.2},  {1.5, 1e-3, 1.0, 0.1}};
  first = true;
  for (const auto& c : ucases) {
    fprintf(g_out, "%s    [%.17g, %.17g, %.17g, %.17g, %.17g]", first ? "" : ",\n", c[0], c[1], c[2], c[3],
           unbindingradius(c[0], c[1], c[2], c[3]));
    first = false;
  }
  fprintf(g_out, "\n  ],\n");
  // normal quantile table (unshuffled: the shuffle's MT state is uninitialised)
  {
    std::vector<float> t(4096);
    randtableF(t.data(), 4096, 1);
    fprintf(g_out, "  \"gauss_table\": [");
    for (int i = 0; i < 4096; i++) fprintf(g_out, "%s%.9g", i ? ", " : "", t[i]);
    fprintf(g_out, "],\n");
  }
  // Poisson sample moments (poisrandF, Numerical Recipes method)
  {
    init_gen_rand(12345);
    fprintf(g_out, "  \"poisson\": [");
    const float means[] = {0.3f, 4.0f, 11.5f, 12.5f, 80.0f, 2500.0f};
    for (int m = 0; m < 6; m++) {
      double s = 0, s2 = 0;
      const int N = 200000;
      for (int k = 0; k < N; k++) {
        const double v = poisrandF(means[m]);
        s += v;
        s2 += v * v;
      }
      const double mu = s / N, var = s2 / N - mu * mu;
      fprintf(g_out, "%s[%.9g, %d, %.9g, %.9g]", m ? ", " : "", means[m], N, mu, var);
    }
    fprintf(g_out, "],\n");
  }
  fprintf(g_out, "  \"networks\": {\n");
  // irreversible A + B -> C (1,2 -> 3), D = 1, 1, 0.5, dt = 1 ms
  run_network("irreversible", 1e-3f, 1000.0f, {0.0f, 1.0f, 1.0f, 0.5f}, {{2, 1, 2, 3, -1, 1, 0.01f}}, false);
  // reversible A + B <-> C, k_off = 10 /s, dt = 0.5 ms
  run_network("reversible", 5e-4f, 216000.0f, {0.0f, 1.0f, 1.0f, 0.5f},
              {{2, 1, 2, 3, -1, 1, 0.05f}, {1, 3, -1, 1, 2, 2, 10.0f}}, false);
  // competing first-order channels of one species, a homodimer and a production
  run_network("mixed", 1e-3f, 90.0f, {0.0f, 0.7f, 0.3f, 2.0f, 0.1f},
              {{1, 1, -1, 2, -1, 1, 5.0f},
               {1, 1, -1, -1, -1, 0, 3.0f},
               {1, 1, -1, 2, 3, 2, 7.5f},
               {2, 3, 3, 4, -1, 1, 0.08f},
               {0, -1, -1, 1, -1, 1, 2.5f},
               {1, 4, -1, -1, -1, 0, 1.0f},
               {2, 2, 4, 1, -1, 1, 0.02f}},
              true);
  fprintf(g_out, "  }\n}\n");
  fclose(g_out);
  return 0;
}

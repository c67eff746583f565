// particle_system.cpp -- the reference's ParticleSystem surface over the C ABI.
#include "../../include/gpusmoldyn_particle_system.hpp"

#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <random>

namespace gpusmoldyn {

namespace {
const float kWorldLo = -1.0f, kWorldHi = 1.0f;  // particleSystem.cpp:73, particleSystem.h:114-120
}

ParticleSystem::ParticleSystem(uint numParticles, uint3v gridSize, bool bUseOpenGL, Preset preset, uint64_t seed)
    : reactionList(&m_reaction), m_preset(preset), m_numParticles(numParticles), m_seed(seed) {
  (void)bUseOpenGL;  // headless only
  memset(reactionOrderInfo, 0, sizeof(reactionOrderInfo));
  bd_config cfg;
  bd_config_default(&cfg);
  for (int a = 0; a < 3; a++) {
    cfg.box_lo[a] = kWorldLo;
    cfg.box_hi[a] = kWorldHi;
  }
  cfg.seed = seed;
  // the reference sizes cells to the grid it is given (particleSystem.cpp:59-76)
  const uint g = std::max(gridSize.x, std::max(gridSize.y, gridSize.z));
  if (g > 0) cfg.cell_size = (kWorldHi - kWorldLo) / (float)g;
  // time step, volume and diffusion coefficients of the presets
  // (test1Types/test2Types/test3Types, particleSystem.cpp:381-571); species 0
  // is the reference's dummy type with D = 0
  switch (preset) {
    case PRESET_TEST1:
      deltaTime = 0.1f;
      systemVolume = 10.0f;
      m_hDiffusionCoefficients = {0.0f, 0.001f, 0.001f};
      break;
    case PRESET_TEST2:
      deltaTime = 0.001f;
      systemVolume = 90.0f;
      m_hDiffusionCoefficients = {0.0f, 0.05f, 0.05f, 0.05f, 0.05f};
      break;
    default:
      deltaTime = 0.01f;
      systemVolume = 90.0f;
      m_hDiffusionCoefficients = {0.0f, 0.3f, 0.1f};
      break;
  }
  cfg.dt = deltaTime;
  m_numTypes = (uint)m_hDiffusionCoefficients.size();
  m_status = bd_create(&cfg, &m_handle);
  if (m_status) return;
  for (float D : m_hDiffusionCoefficients) bd_add_species(m_handle, D, nullptr);
  auto add = [&](int order, int r0, int r1, int p0, int p1, float rate) {
    const int rc[2] = {r0, r1}, pr[2] = {p0, p1};
    int id = -1;
    bd_add_reaction(m_handle, order, rc, pr, rate, &id);
    return id;
  };
  if (preset == PRESET_TEST1) {
    add(1, 1, -1, 1, 1, 10.0f);    // A -> 2A
    add(2, 1, 2, 2, 2, 2000.0f);   // A + B -> 2B
    add(1, 2, -1, -1, -1, 10.0f);  // B -> 0
  } else if (preset == PRESET_TEST2) {
    add(2, 1, 2, 3, -1, 0.01f);                        // E + S -> ES
    const int back = add(1, 3, -1, 1, 2, 1.0f);        // ES -> E + S
    bd_set_product_placement(m_handle, back, BD_PP_PGEMMAX, 0.2f);
    add(1, 3, -1, 1, 4, 1.0f);                         // ES -> E + P
  }
  m_status = bd_finalize(m_handle);
  buildTables();
  reset(CONFIG_GRID);
}

ParticleSystem::~ParticleSystem() {
  if (m_handle) bd_destroy(m_handle);
}

std::vector<int> ParticleSystem::presetTypes() const {
  std::vector<int> t(m_numParticles);
  uint bound;
  if (m_preset == PRESET_TEST1) bound = m_numParticles / 2;
  else if (m_preset == PRESET_TEST2) bound = m_numParticles / 11;
  else bound = 3 * (m_numParticles / 4);
  for (uint i = 0; i < m_numParticles; i++) t[i] = i < bound ? 1 : 2;
  return t;
}

void ParticleSystem::reset(ParticleConfig config) {
  m_hPos.assign((size_t)m_numParticles * 4, 0.0f);
  std::mt19937 gen(1973);
  std::uniform_real_distribution<float> uni(0.0f, 1.0f);
  if (config == CONFIG_GRID) {
    // jittered lattice (initGrid, particleSystem.cpp:1087-1116)
    const uint s = (uint)std::ceil(std::pow((double)m_numParticles, 1.0 / 3.0));
    const float spacing = (kWorldHi - kWorldLo) / (float)std::max<uint>(s, 1);
    const float jitter = spacing * 0.01f;
    for (uint i = 0; i < m_numParticles; i++) {
      const uint x = i % s, y = (i / s) % s, z = i / (s * s);
      const uint c[3] = {x, y, z};
      for (int a = 0; a < 3; a++) {
        float v = kWorldLo + spacing * (c[a] + 0.5f) + (uni(gen) * 2.0f - 1.0f) * jitter;
        m_hPos[4 * i + a] = std::min(std::max(v, kWorldLo), kWorldHi);
      }
      m_hPos[4 * i + 3] = 1.0f;
    }
  } else {
    for (uint i = 0; i < m_numParticles; i++) {
      for (int a = 0; a < 3; a++) m_hPos[4 * i + a] = kWorldLo + (kWorldHi - kWorldLo) * uni(gen);
      m_hPos[4 * i + 3] = 1.0f;
    }
  }
  m_hTypes = presetTypes();
  if (m_handle) m_status = bd_set_particles(m_handle, m_hPos.data(), m_hTypes.data(), m_numParticles);
}

bool ParticleSystem::update() { return update(1); }

bool ParticleSystem::update(int nsteps) {
  if (!m_handle) return false;
  m_status = bd_step(m_handle, nsteps);
  if (m_status) return false;
  m_status = bd_synchronize(m_handle);
  if (m_status) return false;
  uint64_t n = 0;
  bd_get_count(m_handle, &n);
  m_numParticles = (uint)n;
  return n > 0;
}

int ParticleSystem::getNumParticles() const { return (int)m_numParticles; }

float* ParticleSystem::getArray(ParticleArray array) {
  if (array != POSITION || !m_handle) return nullptr;
  uint64_t n = 0;
  bd_get_count(m_handle, &n);
  m_hPos.assign((size_t)n * 4, 0.0f);
  m_hTypes.assign((size_t)n, 0);
  size_t got = 0;
  m_status = bd_get_particles(m_handle, m_hPos.data(), m_hTypes.data(), (size_t)n, &got);
  return m_hPos.data();
}

void ParticleSystem::setArray(ParticleArray array, const float* data, int start, int count) {
  if (array != POSITION || !m_handle || start < 0 || count < 0) return;
  getArray(POSITION);
  if ((size_t)(start + count) * 4 > m_hPos.size()) return;
  memcpy(&m_hPos[(size_t)start * 4], data, (size_t)count * 4 * sizeof(float));
  m_status = bd_set_particles(m_handle, m_hPos.data(), m_hTypes.data(), m_hTypes.size());
}

void* ParticleSystem::getCudaPosVBO() const {
  void* p = nullptr;
  uint64_t n = 0;
  if (m_handle) bd_get_state_pointer(m_handle, &p, &n);
  return p;
}

uint3v ParticleSystem::getGridSize() {
  uint32_t d[3] = {0, 0, 0};
  if (m_handle) bd_get_grid(m_handle, 0, d, nullptr, nullptr);
  return uint3v{d[0], d[1], d[2]};
}

float3v ParticleSystem::getCellSize() {
  float c[3] = {0, 0, 0};
  if (m_handle) bd_get_grid(m_handle, 0, nullptr, c, nullptr);
  return float3v{c[0], c[1], c[2]};
}

void ParticleSystem::dumpGrid() {
  size_t nc = 0;
  if (!m_handle || bd_debug_get_cells(m_handle, nullptr, 0, &nc)) return;
  std::vector<uint32_t> st(nc + 1);
  bd_debug_get_cells(m_handle, st.data(), st.size(), &nc);
  uint32_t mx = 0;
  for (size_t c = 0; c < nc; c++) mx = std::max(mx, st[c + 1] - st[c]);
  printf("maximum particles per cell = %u\n", mx);
}

void ParticleSystem::dumpParticles(uint start, uint count) {
  getArray(POSITION);
  for (uint i = start; i < start + count && (size_t)i * 4 + 3 < m_hPos.size(); i++)
    printf("pos: (%.4f, %.4f, %.4f, %.4f)\n", m_hPos[4 * i], m_hPos[4 * i + 1], m_hPos[4 * i + 2], m_hPos[4 * i + 3]);
}

// Host mirror of the reaction tables: the struct-of-arrays reaction list and
// the per-order CSR built by fillReactionOrderInfo (smolreact.cpp:173-271).
void ParticleSystem::buildTables() {
  int S = 0, R = 0;
  if (!m_handle) return;
  bd_get_counts(m_handle, &S, &R);
  m_order.assign(R, 0);
  m_nprod.assign(R, 0);
  m_r2.assign(R, 0.0f);
  m_unbind.assign(R, 0.0f);
  m_gem.assign(R, 0.0f);
  m_prob.assign(R, 0.0f);
  m_rate.assign(R, 0.0f);
  m_prodPos.assign((size_t)R * 6, 0.0f);
  m_products.assign(R, int2v{-1, -1});
  m_reactants.assign(R, int2v{-1, -1});
  for (int r = 0; r < R; r++) {
    bd_reaction_info ri;
    if (bd_get_reaction_info(m_handle, r, &ri)) continue;
    m_order[r] = ri.order;
    m_nprod[r] = ri.nprod;
    m_r2[r] = ri.bind_radius * ri.bind_radius;
    m_unbind[r] = ri.unbind_radius;
    m_gem[r] = ri.geminate_prob;
    m_prob[r] = ri.prob;
    m_rate[r] = ri.rate;
    m_prodPos[6 * r] = ri.product_offsets[0];
    m_prodPos[6 * r + 3] = ri.product_offsets[1];
    m_products[r] = int2v{ri.products[0], ri.products[1]};
    m_reactants[r] = int2v{ri.reactants[0], ri.reactants[1]};
  }
  m_reaction = Reaction{m_order.data(), m_r2.data(), m_unbind.data(), m_gem.data(), m_prob.data(), m_rate.data(),
                        m_nprod.data(), m_products.data(), m_reactants.data(), m_prodPos.data()};
  for (int o = 0; o < 3; o++) {
    std::vector<int>& count = m_csr[o][0];
    std::vector<int>& idx = m_csr[o][1];
    std::vector<int>& l2g = m_csr[o][2];
    std::vector<int>& list = m_csr[o][3];
    count.assign(S, 0);
    idx.assign(S, 0);
    list.clear();
    for (int r = 0; r < R; r++) {
      if (m_order[r] != o) continue;
      list.push_back(r);
      if (o >= 1) count[m_reactants[r].x]++;
      if (o == 2) count[m_reactants[r].y]++;
    }
    for (int s = 1; s < S; s++) idx[s] = idx[s - 1] + count[s - 1];
    l2g.assign(S ? idx[S - 1] + count[S - 1] : 0, 0);
    std::vector<int> fill(idx);
    for (int r = 0; r < R; r++) {
      if (m_order[r] != o || o == 0) continue;
      l2g[fill[m_reactants[r].x]++] = r;
      if (o == 2) l2g[fill[m_reactants[r].y]++] = r;
    }
    reactionOrderInfo[o] = ReactionOrderInfo{o, (int)list.size(), idx.data(), l2g.data(), (int)l2g.size(),
                                             count.data(), list.data()};
  }
}

}  // namespace gpusmoldyn

// gpusmoldyn_particle_system.hpp -- C++ drop-in for the reference's
// ParticleSystem class (particleSystem.h:50-218), implemented over the C ABI
// of gpusmoldyn.h.  Method names, argument meaning and return conventions
// follow the reference: update() advances one step and returns false when no
// particle is left or the capacity is exhausted; reactionOrderInfo[3] and
// reactionList expose the host reaction tables (reaction.h:36-66).
// OpenGL members are absent (headless); the device record array replaces the
// position/type VBOs.
#ifndef GPUSMOLDYN_PARTICLE_SYSTEM_HPP
#define GPUSMOLDYN_PARTICLE_SYSTEM_HPP

#include <stdint.h>

#include <vector>

#include "gpusmoldyn.h"

namespace gpusmoldyn {

typedef unsigned int uint;

struct uint3v {
  uint x, y, z;
};
struct float3v {
  float x, y, z;
};
struct int2v {
  int x, y;
};

// Struct-of-arrays reaction list (reaction.h:36-48).
struct Reaction {
  int* order;
  float* bindRadiusSquared;
  float* unbindRadius;
  float* geminateProbability;
  float* prob;
  float* rate;
  int* nprod;
  int2v* products;
  int2v* reactants;
  float* productPositions;  // [6] per reaction: product offsets (x, y, z) x 2
};

// Per-order CSR tables (reaction.h:52-66).
struct ReactionOrderInfo {
  int order;
  int reactionsPerOrder;
  int* reactionsPerTypeIdx;
  int* localToGlobal;
  int localToGlobalSize;
  int* numberOfReactionsPerType;
  int* reactionIndexes;
};

class __attribute__((visibility("default"))) ParticleSystem {
 public:
  enum ParticleConfig { CONFIG_RANDOM, CONFIG_GRID, _NUM_CONFIGS };
  enum ParticleArray { POSITION, VELOCITY };
  // The reference's built-in scenarios (particleSystem.cpp:319-571).
  enum Preset { PRESET_TEST1, PRESET_TEST2, PRESET_TEST3 };

  ParticleSystem(uint numParticles, uint3v gridSize, bool bUseOpenGL = false, Preset preset = PRESET_TEST3,
                 uint64_t seed = 1);
  ~ParticleSystem();

  bool update();
  bool update(int nsteps);
  void reset(ParticleConfig config);

  float* getArray(ParticleArray array);
  void setArray(ParticleArray array, const float* data, int start, int count);

  int getNumParticles() const;
  int getNumTypes() const { return m_numTypes; }
  float getDeltaTime() const { return deltaTime; }
  float getSystemVolume() const { return systemVolume; }
  void* getCudaPosVBO() const;      // device float4 records (x, y, z, species bits)
  void* getCudaTypesVBO() const { return nullptr; }
  float* getDiffusionCoefficients() { return m_hDiffusionCoefficients.data(); }
  uint3v getGridSize();
  float3v getWorldOrigin() { return float3v{-1.0f, -1.0f, -1.0f}; }
  float3v getCellSize();
  void dumpGrid();
  void dumpParticles(uint start, uint count);
  bd_handle handle() const { return m_handle; }
  bd_status lastStatus() const { return m_status; }

 public:
  ReactionOrderInfo reactionOrderInfo[3];
  Reaction* reactionList;

 private:
  ParticleSystem(const ParticleSystem&) = delete;
  ParticleSystem& operator=(const ParticleSystem&) = delete;
  void buildTables();
  std::vector<int> presetTypes() const;

  bd_handle m_handle = nullptr;
  bd_status m_status = BD_OK;
  Preset m_preset;
  uint m_numParticles;
  uint m_numTypes = 0;
  float deltaTime = 0.0f;
  float systemVolume = 0.0f;
  uint64_t m_seed;
  std::vector<float> m_hDiffusionCoefficients;
  std::vector<float> m_hPos;
  std::vector<int> m_hTypes;
  // storage behind reactionList / reactionOrderInfo
  Reaction m_reaction{};
  std::vector<int> m_order, m_nprod;
  std::vector<float> m_r2, m_unbind, m_gem, m_prob, m_rate, m_prodPos;
  std::vector<int2v> m_products, m_reactants;
  std::vector<int> m_csr[3][4];
};

}  // namespace gpusmoldyn

#endif

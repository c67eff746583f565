// Drives the C++ ParticleSystem drop-in the way the reference's benchmark
// loop drives its class (particles.cpp:163-175, 213-242): construct, reset,
// update() in a loop, read positions back.
#include <stdio.h>

#include "gpusmoldyn_particle_system.hpp"

int main() {
  using gpusmoldyn::ParticleSystem;
  int rc = 0;
  const ParticleSystem::Preset presets[3] = {ParticleSystem::PRESET_TEST1, ParticleSystem::PRESET_TEST2,
                                             ParticleSystem::PRESET_TEST3};
  for (int p = 0; p < 3; p++) {
    // test1's rates make every A-B pair in the [-1,1]^3 world a candidate:
    // keep it small
    const unsigned n0 = p == 0 ? 1000 : 20000;
    ParticleSystem ps(n0, {64, 64, 64}, false, presets[p]);
    if (ps.lastStatus() != BD_OK && ps.lastStatus() != BD_ERR_PGEM_UNATTAINABLE) {
      printf("preset %d: status %d\n", p, ps.lastStatus());
      return 2;
    }
    int steps = 0;
    for (; steps < (p == 0 ? 5 : 50) && ps.update(); ++steps) {
    }
    float* pos = ps.getArray(ParticleSystem::POSITION);
    const int n = ps.getNumParticles();
    int outside = 0;
    for (int i = 0; i < n; i++)
      for (int a = 0; a < 3; a++)
        if (pos[4 * i + a] < -1.0f || pos[4 * i + a] > 1.0f) outside++;
    printf("preset %d: steps %d particles %d types %d dt %g outside %d reactions %d grid %u\n", p + 1, steps, n,
           ps.getNumTypes(), ps.getDeltaTime(), outside, ps.reactionOrderInfo[1].reactionsPerOrder +
           ps.reactionOrderInfo[2].reactionsPerOrder, ps.getGridSize().x);
    if (outside || (p == 2 && (steps != 50 || n != 20000))) rc = 1;
  }
  return rc;
}

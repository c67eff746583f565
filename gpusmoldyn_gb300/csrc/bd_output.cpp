// bd_output.cpp -- headless observables: a snapshot of the molecules written
// to a file, in place of the reference's OpenGL viewer (render_particles.cpp,
// particles.cpp), which has no counterpart on a machine without a display.
#include <stdint.h>
#include <stdio.h>

#include <vector>

#include "../../include/gpusmoldyn.h"

// Text: a header line "# step <s> molecules <n> species <S>", a line
// "# counts c0 c1 ..." and one line "x y z species" per molecule (9
// significant digits, enough to restore a float exactly).  Binary: uint64
// step, uint64 n, then n records of float x, y, z and int32 species.
BD_API bd_status bd_write_snapshot(bd_handle h, const char* path, int format) {
  if (!h || !path || (format != BD_SNAPSHOT_TEXT && format != BD_SNAPSHOT_BINARY)) return BD_ERR_INVALID_ARGUMENT;
  uint64_t step = 0;
  bd_status st = bd_get_step(h, &step);
  if (st && st != BD_ERR_EMPTY) return st;
  size_t n = 0;
  st = bd_get_particles(h, nullptr, nullptr, 0, &n);
  if (st) return st;
  std::vector<float> xyz4(4 * n + 4);
  std::vector<int> sp(n + 1);
  size_t got = 0;
  if ((st = bd_get_particles(h, xyz4.data(), sp.data(), n, &got))) return st;
  int n_species = 0, n_reactions = 0;
  if ((st = bd_get_counts(h, &n_species, &n_reactions))) return st;
  FILE* f = fopen(path, format == BD_SNAPSHOT_TEXT ? "w" : "wb");
  if (!f) return BD_ERR_INVALID_ARGUMENT;
  bool ok = true;
  if (format == BD_SNAPSHOT_TEXT) {
    std::vector<uint64_t> counts(n_species > 0 ? n_species : 1, 0);
    for (size_t i = 0; i < got; i++)
      if (sp[i] >= 0 && sp[i] < n_species) counts[sp[i]]++;
    ok = fprintf(f, "# step %llu molecules %llu species %d\n# counts", (unsigned long long)step,
                 (unsigned long long)got, n_species) > 0;
    for (int s = 0; s < n_species && ok; s++) ok = fprintf(f, " %llu", (unsigned long long)counts[s]) > 0;
    ok = ok && fprintf(f, "\n") > 0;
    for (size_t i = 0; i < got && ok; i++)
      ok = fprintf(f, "%.9g %.9g %.9g %d\n", xyz4[4 * i], xyz4[4 * i + 1], xyz4[4 * i + 2], sp[i]) > 0;
  } else {
    const uint64_t hdr[2] = {step, (uint64_t)got};
    ok = fwrite(hdr, sizeof(hdr), 1, f) == 1;
    for (size_t i = 0; i < got && ok; i++) {
      const float p[3] = {xyz4[4 * i], xyz4[4 * i + 1], xyz4[4 * i + 2]};
      const int32_t s = sp[i];
      ok = fwrite(p, sizeof(p), 1, f) == 1 && fwrite(&s, sizeof(s), 1, f) == 1;
    }
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? BD_OK : BD_ERR_INVALID_ARGUMENT;
}

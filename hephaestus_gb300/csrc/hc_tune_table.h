// hc_tune_table.h -- the launch-configuration table of the hex autotuner
// (hc_tune.cu), host only: the text format of HC_TUNE_FILE, one line per
// tuned problem:
//     p full nx ny nz shape per_sm us kind
// (order, 1 = general parallelepipeds, grid, brick shape, CTAs per SM, the
// chosen configuration's mean launch time, 0 = real / 1 = complex apply).
#pragma once
#include <array>
#include <cstdio>
#include <map>

namespace hc {

struct TuneEntry {
  int shape = 0, per_sm = 0;
};
using TuneKey = std::array<int, 5>;  // p, full, nx, ny, nz

// Entries of f into t: later lines win; lines with an unknown shape or an
// out-of-range CTA count are skipped; reading stops at the first line that
// does not hold nine fields.
inline void tune_read(FILE* f, std::map<TuneKey, TuneEntry>& t) {
  int p, full, nx, ny, nz, shape, per, kind;
  double us;
  while (std::fscanf(f, "%d %d %d %d %d %d %d %lf %d", &p, &full, &nx, &ny, &nz, &shape, &per, &us, &kind) == 9) {
    if (shape < 0 || shape > 1 || per < 0 || per > 64) continue;
    t[TuneKey{p, full, nx, ny, nz}] = TuneEntry{shape, per};
  }
}

// Appends one line; false when the file cannot be opened.
inline bool tune_append(const char* path, const TuneKey& k, const TuneEntry& e, double us, int kind) {
  FILE* f = std::fopen(path, "a");
  if (!f) return false;
  std::fprintf(f, "%d %d %d %d %d %d %d %.3f %d\n", k[0], k[1], k[2], k[3], k[4], e.shape, e.per_sm, us, kind);
  std::fclose(f);
  return true;
}

}  // namespace hc

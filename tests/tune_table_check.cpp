// CPU check of the autotuner's table format (hc_tune_table.h): writes a table
// with tune_append, adds hand-written lines (a later entry for the same
// problem, a bad shape, a bad CTA count), reads it back with tune_read and
// prints the resulting table: "p full nx ny nz shape per_sm" per entry.
#include <cstdio>
#include <map>

#include "hc_tune_table.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const char* path = argv[1];
  std::remove(path);
  using hc::TuneEntry;
  using hc::TuneKey;
  if (!hc::tune_append(path, TuneKey{2, 0, 20, 12, 6}, TuneEntry{1, 3}, 41.5, 0)) return 3;
  if (!hc::tune_append(path, TuneKey{1, 1, 8, 8, 8}, TuneEntry{0, 0}, 7.25, 1)) return 3;
  FILE* f = std::fopen(path, "a");
  if (!f) return 3;
  std::fprintf(f, "2 0 20 12 6 0 2 39.000 1\n");  // later line for the same problem wins
  std::fprintf(f, "3 0 9 9 9 2 0 10.000 0\n");    // shape 2 does not exist: skipped
  std::fprintf(f, "2 1 5 5 5 1 99 10.000 0\n");   // CTA count out of range: skipped
  std::fprintf(f, "garbage\n");                     // stops the reader
  std::fprintf(f, "1 0 4 4 4 1 1 1.000 0\n");     // not reached
  std::fclose(f);
  std::map<TuneKey, TuneEntry> t;
  f = std::fopen(path, "r");
  if (!f) return 4;
  hc::tune_read(f, t);
  std::fclose(f);
  for (const auto& kv : t)
    std::printf("%d %d %d %d %d %d %d\n", kv.first[0], kv.first[1], kv.first[2], kv.first[3], kv.first[4],
                kv.second.shape, kv.second.per_sm);
  return 0;
}

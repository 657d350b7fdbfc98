// hc_host_par.h -- small host-parallel helpers (std::thread): a chunked
// parallel for and a deterministic parallel sort (sorted chunks merged
// pairwise; the result is exactly std::sort's).
#pragma once
#include <algorithm>
#include <cstdint>
#include <thread>
#include <vector>

namespace hc {

inline int host_threads() { return (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency())); }

// Run f(lo, hi) over [0, n) in contiguous chunks of at least `grain` items.
template <typename F>
inline void parallel_for(int64_t n, F f, int64_t grain = 64) {
  const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(host_threads(), n / std::max<int64_t>(1, grain)));
  if (nt <= 1) {
    f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt);
  for (int k = 0; k < nt; ++k) {
    const int64_t lo = n * k / nt, hi = n * (k + 1) / nt;
    th.emplace_back([&f, lo, hi] { f(lo, hi); });
  }
  for (auto& t : th) t.join();
}

template <typename T>
inline void parallel_sort(std::vector<T>& v) {
  const size_t n = v.size();
  int nt = 1;
  while (nt * 2 <= host_threads() && n / (size_t)(nt * 2) >= 65536) nt *= 2;
  if (nt == 1) {
    std::sort(v.begin(), v.end());
    return;
  }
  std::vector<size_t> b(nt + 1);
  for (int k = 0; k <= nt; ++k) b[k] = n * (size_t)k / (size_t)nt;
  {
    std::vector<std::thread> th;
    for (int k = 0; k < nt; ++k) th.emplace_back([&v, &b, k] { std::sort(v.begin() + b[k], v.begin() + b[k + 1]); });
    for (auto& t : th) t.join();
  }
  for (int w = 1; w < nt; w *= 2) {
    std::vector<std::thread> th;
    for (int k = 0; k + w < nt; k += 2 * w) {
      const size_t lo = b[k], mid = b[k + w], hi = b[std::min(k + 2 * w, nt)];
      th.emplace_back([&v, lo, mid, hi] { std::inplace_merge(v.begin() + lo, v.begin() + mid, v.begin() + hi); });
    }
    for (auto& t : th) t.join();
  }
}

}  // namespace hc

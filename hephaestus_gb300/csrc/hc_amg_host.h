// hc_amg_host.h -- host (FP64, C++17) set-up of the smoothed-aggregation AMG
// used by the tet auxiliary-space preconditioner (hc_tetaux.cu): CSR
// products, strength-based aggregation, the smoothed prolongator and the
// dense inverse of the diagonally scaled coarsest operator.  Plain C++ with
// std::thread, so it is unit-tested on the CPU (tests/amg_host_check.cpp).
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <thread>
#include <utility>
#include <vector>

#include "hc_host_par.h"

namespace hc {
namespace amg {

struct HCsr {
  int n = 0, m = 0;  // rows, columns
  std::vector<int> rp, ci;
  std::vector<double> va;
};

// Build an n-row CSR whose rows are produced independently: row_fn(i, marker,
// scratch, ci, va) appends row i's sorted (column, value) entries.  Rows are
// computed in contiguous chunks on host threads (each with its own marker
// array of width m) and concatenated in order, so the result does not depend
// on the thread count.
template <typename RowFn>
inline HCsr build_rows(int n, int m, RowFn row_fn) {
  const int nt = std::max(1, std::min(host_threads(), n / 256));
  std::vector<std::vector<int>> cis(nt), lens(nt);
  std::vector<std::vector<double>> vas(nt);
  auto work = [&](int c) {
    const int lo = (int)((int64_t)n * c / nt), hi = (int)((int64_t)n * (c + 1) / nt);
    std::vector<int> marker(m, -1);
    std::vector<std::pair<int, double>> scratch;
    lens[c].reserve(hi - lo);
    for (int i = lo; i < hi; ++i) {
      const size_t before = cis[c].size();
      row_fn(i, marker, scratch, cis[c], vas[c]);
      lens[c].push_back((int)(cis[c].size() - before));
    }
  };
  if (nt == 1) {
    work(0);
  } else {
    std::vector<std::thread> th;
    for (int c = 0; c < nt; ++c) th.emplace_back(work, c);
    for (auto& t : th) t.join();
  }
  HCsr C;
  C.n = n;
  C.m = m;
  C.rp.assign(1, 0);
  C.rp.reserve(n + 1);
  size_t tot = 0;
  for (int c = 0; c < nt; ++c) tot += cis[c].size();
  C.ci.reserve(tot);
  C.va.reserve(tot);
  for (int c = 0; c < nt; ++c) {
    for (int l : lens[c]) C.rp.push_back(C.rp.back() + l);
    C.ci.insert(C.ci.end(), cis[c].begin(), cis[c].end());
    C.va.insert(C.va.end(), vas[c].begin(), vas[c].end());
  }
  return C;
}

// appends the marker-accumulated scratch row, sorted by column, and clears the marker
inline void flush_row(std::vector<int>& marker, std::vector<std::pair<int, double>>& row, std::vector<int>& ci,
                      std::vector<double>& va) {
  for (auto& q : row) marker[q.first] = -1;
  std::sort(row.begin(), row.end());
  for (auto& q : row) {
    ci.push_back(q.first);
    va.push_back(q.second);
  }
  row.clear();
}

inline void marker_add(std::vector<int>& marker, std::vector<std::pair<int, double>>& row, int col, double v) {
  if (marker[col] < 0) {
    marker[col] = (int)row.size();
    row.push_back({col, v});
  } else {
    row[marker[col]].second += v;
  }
}

inline std::vector<double> diagonal(const HCsr& A) {
  std::vector<double> d(A.n, 0.0);
  for (int i = 0; i < A.n; ++i)
    for (int k = A.rp[i]; k < A.rp[i + 1]; ++k)
      if (A.ci[k] == i) d[i] = A.va[k];
  return d;
}

// Three-pass greedy aggregation on the strength graph
// |a_ij| > theta sqrt(|a_ii a_jj|): (1) a node whose strong neighbours are all
// free starts an aggregate with them; (2) a remaining node joins the aggregate
// of its strongest already-aggregated strong neighbour; (3) leftovers start
// aggregates with their free strong neighbours.  Returns the aggregate count.
inline int aggregate(const HCsr& A, const std::vector<double>& dg, double theta, std::vector<int>& agg) {
  const int n = A.n;
  auto strong = [&](int i, int k) {
    const int j = A.ci[k];
    return j != i && std::fabs(A.va[k]) > theta * std::sqrt(std::fabs(dg[i] * dg[j]));
  };
  agg.assign(n, -1);
  int na = 0;
  for (int i = 0; i < n; ++i) {
    if (agg[i] != -1) continue;
    bool ok = true;
    for (int k = A.rp[i]; k < A.rp[i + 1] && ok; ++k)
      if (strong(i, k) && agg[A.ci[k]] != -1) ok = false;
    if (!ok) continue;
    agg[i] = na;
    for (int k = A.rp[i]; k < A.rp[i + 1]; ++k)
      if (strong(i, k)) agg[A.ci[k]] = na;
    ++na;
  }
  const std::vector<int> a1 = agg;
  for (int i = 0; i < n; ++i) {
    if (a1[i] != -1) continue;
    int best = -1;
    double bs = 0.0;
    for (int k = A.rp[i]; k < A.rp[i + 1]; ++k)
      if (strong(i, k) && a1[A.ci[k]] >= 0 && std::fabs(A.va[k]) > bs) {
        bs = std::fabs(A.va[k]);
        best = a1[A.ci[k]];
      }
    if (best >= 0) agg[i] = best;
  }
  for (int i = 0; i < n; ++i) {
    if (agg[i] != -1) continue;
    agg[i] = na;
    for (int k = A.rp[i]; k < A.rp[i + 1]; ++k)
      if (strong(i, k) && agg[A.ci[k]] == -1) agg[A.ci[k]] = na;
    ++na;
  }
  return na;
}

// Largest eigenvalue of D^-1 A (power iteration on D^-1/2 A D^-1/2 from a fixed start).
inline double lmax_scaled(const HCsr& A, const std::vector<double>& dg, int iters = 40) {
  const int n = A.n;
  std::vector<double> s(n), x(n), y(n);
  for (int i = 0; i < n; ++i) {
    s[i] = 1.0 / std::sqrt(std::fabs(dg[i]));
    x[i] = 1.0 + 0.37 * std::sin(1.0 + 7.3 * i);
  }
  double lam = 1.0;
  for (int it = 0; it < iters; ++it) {
    double nx = 0.0;
    for (double v : x) nx += v * v;
    nx = std::sqrt(nx);
    for (double& v : x) v /= nx;
    double xy = 0.0;
    for (int i = 0; i < n; ++i) {
      double t = 0.0;
      for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) t += A.va[k] * s[A.ci[k]] * x[A.ci[k]];
      y[i] = s[i] * t;
      xy += x[i] * y[i];
    }
    lam = xy;
    x.swap(y);
  }
  return lam;
}

// P = (I - omega D^-1 A) P_tent, P_tent[i][agg[i]] = 1 / sqrt(|aggregate|).
// Rows are accumulated through a marker array over the aggregates (linear in
// the row's nonzeros, also on the dense rows of coarse Galerkin operators) and
// computed on host threads.
inline HCsr smooth_prolongator(const HCsr& A, const std::vector<double>& dg, const std::vector<int>& agg, int na,
                               double omega) {
  std::vector<int> cnt(na, 0);
  for (int a : agg) ++cnt[a];
  std::vector<double> pt(A.n);
  for (int i = 0; i < A.n; ++i) pt[i] = 1.0 / std::sqrt((double)cnt[agg[i]]);
  return build_rows(A.n, na, [&](int i, std::vector<int>& marker, std::vector<std::pair<int, double>>& row,
                                 std::vector<int>& ci, std::vector<double>& va) {
    marker_add(marker, row, agg[i], pt[i]);
    for (int k = A.rp[i]; k < A.rp[i + 1]; ++k)
      marker_add(marker, row, agg[A.ci[k]], -omega / dg[i] * A.va[k] * pt[A.ci[k]]);
    flush_row(marker, row, ci, va);
  });
}

inline HCsr transpose(const HCsr& P) {
  HCsr T;
  T.n = P.m;
  T.m = P.n;
  T.rp.assign(P.m + 1, 0);
  for (int c : P.ci) ++T.rp[c + 1];
  for (int i = 0; i < P.m; ++i) T.rp[i + 1] += T.rp[i];
  T.ci.resize(P.ci.size());
  T.va.resize(P.va.size());
  std::vector<int> pos(T.rp.begin(), T.rp.end() - 1);
  for (int i = 0; i < P.n; ++i)
    for (int k = P.rp[i]; k < P.rp[i + 1]; ++k) {
      const int q = pos[P.ci[k]]++;
      T.ci[q] = i;
      T.va[q] = P.va[k];
    }
  return T;
}

// C = A B (Gustavson with a marker array per thread; rows sorted by column).
inline HCsr spgemm(const HCsr& A, const HCsr& B) {
  return build_rows(A.n, B.m, [&](int i, std::vector<int>& marker, std::vector<std::pair<int, double>>& row,
                                  std::vector<int>& ci, std::vector<double>& va) {
    for (int ka = A.rp[i]; ka < A.rp[i + 1]; ++ka) {
      const int j = A.ci[ka];
      const double av = A.va[ka];
      for (int kb = B.rp[j]; kb < B.rp[j + 1]; ++kb) marker_add(marker, row, B.ci[kb], av * B.va[kb]);
    }
    flush_row(marker, row, ci, va);
  });
}

// inv = (S A S)^-1 with S = diag^-1/2, sc = S (both FP32, for the device), by a
// Cholesky factor L of S A S (row-major, contiguous inner products, rows below
// each column block on host threads), the rows
// of L^-1's transpose (row j = column j of L^-1, computed independently on
// host threads) and inv[i][j] = sum_k L^-1[k][i] L^-1[k][j] (threads over i).
// Returns false if S A S is not positive definite.
inline bool dense_scaled_inverse(const HCsr& A, const std::vector<double>& dg, std::vector<float>& inv,
                                 std::vector<float>& sc) {
  const int n = A.n;
  std::vector<double> M((size_t)n * n, 0.0), s(n);
  for (int i = 0; i < n; ++i) s[i] = 1.0 / std::sqrt(std::fabs(dg[i]));
  for (int i = 0; i < n; ++i)
    for (int k = A.rp[i]; k < A.rp[i + 1]; ++k) M[(size_t)i * n + A.ci[k]] = s[i] * A.va[k] * s[A.ci[k]];
  // Cholesky, lower triangle in place, by column blocks of 64: the block's own
  // rows in order, then every row below it on host threads.  Each entry is
  // L[i][j] = (M[i][j] - sum_{k<j} L[i][k] L[j][k]) / L[j][j] with the sum in
  // ascending k, as in the column-by-column algorithm.
  constexpr int kBlock = 64;
  for (int j0 = 0; j0 < n; j0 += kBlock) {
    const int j1 = std::min(n, j0 + kBlock);
    for (int j = j0; j < j1; ++j) {
      const double* rj = &M[(size_t)j * n];
      double d = rj[j];
      for (int k = 0; k < j; ++k) d -= rj[k] * rj[k];
      if (!(d > 1e-12)) return false;
      d = std::sqrt(d);
      M[(size_t)j * n + j] = d;
      for (int i = j + 1; i < j1; ++i) {
        double* ri = &M[(size_t)i * n];
        double v = ri[j];
        for (int k = 0; k < j; ++k) v -= ri[k] * rj[k];
        ri[j] = v / d;
      }
    }
    parallel_for(n - j1, [&](int64_t lo, int64_t hi) {
      for (int64_t ii = lo; ii < hi; ++ii) {
        double* ri = &M[(size_t)(j1 + ii) * n];
        for (int j = j0; j < j1; ++j) {
          const double* rj = &M[(size_t)j * n];
          double v = ri[j];
          for (int k = 0; k < j; ++k) v -= ri[k] * rj[k];
          ri[j] = v / rj[j];
        }
      }
    }, 16);
  }
  // LiT[j][k] = (L^-1)[k][j], k >= j: forward substitution L y = e_j
  std::vector<double> LiT((size_t)n * n, 0.0);
  parallel_for(n, [&](int lo, int hi) {
    for (int j = lo; j < hi; ++j) {
      double* y = &LiT[(size_t)j * n];
      y[j] = 1.0 / M[(size_t)j * n + j];
      for (int i = j + 1; i < n; ++i) {
        const double* ri = &M[(size_t)i * n];
        double v = 0.0;
        for (int k = j; k < i; ++k) v -= ri[k] * y[k];
        y[i] = v / ri[i];
      }
    }
  });
  inv.assign((size_t)n * n, 0.f);
  parallel_for(n, [&](int lo, int hi) {
    for (int i = lo; i < hi; ++i) {
      const double* yi = &LiT[(size_t)i * n];
      for (int j = 0; j <= i; ++j) {
        const double* yj = &LiT[(size_t)j * n];
        double v = 0.0;
        for (int k = i; k < n; ++k) v += yi[k] * yj[k];
        inv[(size_t)i * n + j] = (float)v;
      }
    }
  });
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) inv[(size_t)i * n + j] = inv[(size_t)j * n + i];
  sc.resize(n);
  for (int i = 0; i < n; ++i) sc[i] = (float)s[i];
  return true;
}

}  // namespace amg
}  // namespace hc

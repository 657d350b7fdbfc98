// hc_tetaux_host.h -- host (C++17) structure of the tet auxiliary-space
// preconditioner, from the element dofs, sorted element vertices, essential
// flags and the element nodal matrices (vertex block upper triangle, then the
// 6 edge-bubble diagonals for order 2, as k_ta_elem writes them):
//   * free vertices: used by an element and carrying no essential dof (one
//     vertex is pinned when there is no essential boundary: G's kernel holds
//     the constants); free edge bubbles (order 2): edges without essential dofs;
//   * gnode / gedge: per dof the free vertex / edge-bubble indices of its (at
//     most 3) gradient slots, -1 for none; essential dofs have none;
//   * Gt: (PG)^T over the nodal rows [free vertices | free edge bubbles];
//   * A: the P1 nodal operator (PG)^T J (PG) on the free vertices (CSR, rows sorted);
//   * dl (order 2): 1 / diagonal of the P2 nodal operator on the nodal rows.
// Shared by hc_tetaux.cu and a CPU test against numpy (tests/tetaux_host_check.cpp).
#pragma once
#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "hc_amg_host.h"
#include "hc_host_par.h"
#include "hc_tet_grad.h"

namespace hc {

struct AuxStructure {
  int nfree = 0, nfe = 0, nn = 0;
  int64_t nface0 = 0;
  std::vector<int> gnode, gedge;
  amg::HCsr Gt, A;
  std::vector<float> dl;
};

inline bool build_aux_structure(int p, int64_t ne, int64_t N, int64_t n_edges, const int32_t* sv, const int32_t* ed,
                                const uint8_t* ess, const double* Ae, AuxStructure& S, std::string& msg) {
  using amg::HCsr;
  const int L = p == 1 ? 6 : 20;
  const int nout = p == 1 ? 10 : 16;

  // nodes: fixed where a vertex carries an essential dof of an element
  int nv = 0;
  for (int64_t i = 0; i < ne * 4; ++i) nv = std::max(nv, sv[i] + 1);
  std::vector<uint8_t> used(nv, 0), fixed(nv, 0);
  for (int64_t e = 0; e < ne; ++e) {
    for (int k = 0; k < 4; ++k) used[sv[4 * e + k]] = 1;
    for (int I = 0; I < L; ++I) {
      if (!ess[ed[e * L + I]]) continue;
      int v[3];
      float c[3];
      const int nn = ta_local(p, I, kHEdges, kHFaces, v, c);
      for (int k = 0; k < nn; ++k) fixed[sv[4 * e + v[k]]] = 1;
    }
  }
  bool any_fixed = false;
  for (int v = 0; v < nv; ++v) any_fixed |= used[v] && fixed[v];
  if (!any_fixed)  // no essential boundary: pin one vertex (G has the constants in its kernel)
    for (int v = 0; v < nv; ++v)
      if (used[v]) {
        fixed[v] = 1;
        break;
      }
  std::vector<int> fmap(nv, -1);
  int nfree = 0;
  for (int v = 0; v < nv; ++v)
    if (used[v] && !fixed[v]) fmap[v] = nfree++;
  if (nfree == 0) {
    msg = "auxiliary-space preconditioner: no free vertex";
    return false;
  }

  // G structure: free nodes of every non-essential dof
  std::vector<int> gnode(3 * N, -1);
  for (int64_t e = 0; e < ne; ++e)
    for (int I = 0; I < L; ++I) {
      const int64_t d = ed[e * L + I];
      if (ess[d]) continue;
      int v[3];
      float c[3];
      const int nn = ta_local(p, I, kHEdges, kHFaces, v, c);
      for (int k = 0; k < nn; ++k) gnode[3 * d + k] = fmap[sv[4 * e + v[k]]];
    }
  const int64_t nface0 = p == 1 ? N : 2 * n_edges;
  // order 2: free edge bubbles (an edge with essential dofs is fixed) and their dofs
  std::vector<int> gedge;
  std::vector<int> emap;
  int nfe = 0;
  if (p == 2) {
    const int64_t nE = n_edges;
    emap.assign(nE, -1);
    for (int64_t g = 0; g < nE; ++g)
      if (!ess[2 * g] && !ess[2 * g + 1]) emap[g] = nfe++;
    gedge.assign(3 * N, -1);
    const int le[4][3] = {{0, 1, 3}, {0, 2, 4}, {1, 2, 5}, {3, 4, 5}};  // local edges ij, ik, jk of each face
    for (int64_t e = 0; e < ne; ++e)
      for (int I = 0; I < L; ++I) {
        const int64_t d = ed[e * L + I];
        if (ess[d]) continue;
        if (I < 12) {
          gedge[3 * d] = emap[d / 2];
        } else {
          const int f = (I - 12) / 2;
          for (int k = 0; k < 3; ++k) gedge[3 * d + k] = emap[ed[e * L + 2 * le[f][k]] / 2];
        }
      }
  }
  const int nn = nfree + nfe;
  auto slot_coef = [&](int64_t d, int k, bool bubble) -> float {
    const bool face = d >= nface0, s1 = face && ((d - nface0) & 1);
    if (!bubble) {
      const float c[3] = {-1.f, face ? (s1 ? -1.f : 2.f) : 1.f, face ? (s1 ? 2.f : -1.f) : 0.f};
      return c[k];
    }
    if (!face) return k == 0 ? ((d & 1) == 0 ? 1.f : -1.f) : 0.f;
    const float c[3] = {s1 ? -2.f : 1.f, s1 ? 1.f : -2.f, 1.f};
    return c[k];
  };
  HCsr Gt;
  Gt.n = nn;
  Gt.m = (int)N;
  Gt.rp.assign(nn + 1, 0);
  for (int64_t d = 0; d < N; ++d)
    for (int k = 0; k < 3; ++k) {
      if (gnode[3 * d + k] >= 0) ++Gt.rp[gnode[3 * d + k] + 1];
      if (nfe && gedge[3 * d + k] >= 0) ++Gt.rp[nfree + gedge[3 * d + k] + 1];
    }
  for (int i = 0; i < nn; ++i) Gt.rp[i + 1] += Gt.rp[i];
  Gt.ci.resize(Gt.rp[nn]);
  Gt.va.resize(Gt.rp[nn]);
  {
    std::vector<int> pos(Gt.rp.begin(), Gt.rp.end() - 1);
    for (int64_t d = 0; d < N; ++d)
      for (int k = 0; k < 3; ++k) {
        const int nd = gnode[3 * d + k];
        if (nd >= 0) {
          const int q = pos[nd]++;
          Gt.ci[q] = (int)d;
          Gt.va[q] = slot_coef(d, k, false);
        }
        if (nfe && gedge[3 * d + k] >= 0) {
          const int q = pos[nfree + gedge[3 * d + k]]++;
          Gt.ci[q] = (int)d;
          Gt.va[q] = slot_coef(d, k, true);
        }
      }
  }

  // nodal operator on free nodes: pattern = vertex graph of the elements
  HCsr A;
  A.n = A.m = nfree;
  {
    std::vector<uint64_t> keys;
    keys.assign(ne * 6, ~(uint64_t)0);  // ~0: an edge with a fixed vertex (sorted last, dropped)
    parallel_for(ne, [&](int64_t lo_e, int64_t hi_e) {
      for (int64_t e = lo_e; e < hi_e; ++e)
        for (int k = 0; k < 6; ++k) {
          const int a = fmap[sv[4 * e + kHEdges[k][0]]], b = fmap[sv[4 * e + kHEdges[k][1]]];
          if (a >= 0 && b >= 0)
            keys[6 * e + k] = (uint64_t)std::min(a, b) * (uint64_t)nfree + (uint64_t)std::max(a, b);
        }
    });
    parallel_sort(keys);
    while (!keys.empty() && keys.back() == ~(uint64_t)0) keys.pop_back();
    keys.erase(std::unique(keys.begin(), keys.end()), keys.end());
    A.rp.assign(nfree + 1, 0);
    for (int i = 0; i < nfree; ++i) A.rp[i + 1] = 1;
    for (uint64_t k : keys) {
      ++A.rp[k / nfree + 1];
      ++A.rp[k % nfree + 1];
    }
    for (int i = 0; i < nfree; ++i) A.rp[i + 1] += A.rp[i];
    A.ci.resize(A.rp[nfree]);
    A.va.assign(A.rp[nfree], 0.0);
    std::vector<int> pos(A.rp.begin(), A.rp.end() - 1);
    for (int i = 0; i < nfree; ++i) A.ci[pos[i]++] = i;
    for (uint64_t k : keys) {
      const int a = (int)(k / nfree), b = (int)(k % nfree);
      A.ci[pos[a]++] = b;
      A.ci[pos[b]++] = a;
    }
    for (int i = 0; i < nfree; ++i) std::sort(A.ci.begin() + A.rp[i], A.ci.begin() + A.rp[i + 1]);
    const int tri[4][4] = {{0, 1, 2, 3}, {1, 4, 5, 6}, {2, 5, 7, 8}, {3, 6, 8, 9}};
    // CSR positions of every element's 16 entries on host threads (-1: fixed
    // vertex), then the sums in element order
    std::vector<int> pos16(ne * 16, -1);
    parallel_for(ne, [&](int64_t lo_e, int64_t hi_e) {
      for (int64_t e = lo_e; e < hi_e; ++e)
        for (int a = 0; a < 4; ++a) {
          const int i = fmap[sv[4 * e + a]];
          if (i < 0) continue;
          for (int b = 0; b < 4; ++b) {
            const int j = fmap[sv[4 * e + b]];
            if (j < 0) continue;
            const int* lo = &A.ci[A.rp[i]];
            const int* hi = &A.ci[A.rp[i + 1]];
            pos16[e * 16 + 4 * a + b] = (int)(std::lower_bound(lo, hi, j) - &A.ci[0]);
          }
        }
    });
    for (int64_t e = 0; e < ne; ++e)
      for (int ab = 0; ab < 16; ++ab)
        if (pos16[e * 16 + ab] >= 0) A.va[pos16[e * 16 + ab]] += Ae[e * nout + tri[ab / 4][ab % 4]];
  }

  // order 2: D_L^-1 on the nodal rows (vertex block diagonal, edge-bubble diagonal)
  std::vector<float> dl;
  if (p == 2) {
    dl.assign(nn, 0.f);
    std::vector<double> bd(nfe, 0.0);
    for (int64_t e = 0; e < ne; ++e)
      for (int ke = 0; ke < 6; ++ke) {
        const int fe = emap[ed[e * L + 2 * ke] / 2];
        if (fe >= 0) bd[fe] += Ae[e * nout + 10 + ke];
      }
    for (int i = 0; i < nfree; ++i)
      for (int k = A.rp[i]; k < A.rp[i + 1]; ++k)
        if (A.ci[k] == i) dl[i] = A.va[k] > 0 ? (float)(1.0 / A.va[k]) : 0.f;
    for (int i = 0; i < nfe; ++i) dl[nfree + i] = bd[i] > 0 ? (float)(1.0 / bd[i]) : 0.f;
  }

  S.nfree = nfree;
  S.nfe = nfe;
  S.nn = nn;
  S.nface0 = nface0;
  S.gnode.swap(gnode);
  S.gedge.swap(gedge);
  S.Gt = std::move(Gt);
  S.A = std::move(A);
  S.dl.swap(dl);
  return true;
}

}  // namespace hc

// hc_tet_topo.h -- host topology of a Nedelec tet mesh (orders 1 and 2): element
// vertices sorted by global index, global edge and face numbering, element dof
// lists and essential flags.  Plain C++ on host threads (per-element work in
// parallel, deterministic parallel sorts), shared by hc_create (hc_tet.cu) and
// a CPU test against the oracle's numbering (tests/tet_topo_check.cpp).
//
// Numbering: edges and faces in lexicographic order of their sorted vertex
// tuples; dofs p * edge + s, then (order 2) 2 n_edges + 2 face + s.  A dof is
// essential when its edge (or face) lies on a boundary triangle whose attribute
// a has bit a - 1 set in ess_attr_bits, or when an explicit mask marks it.
#pragma once
#include <algorithm>
#include <array>
#include <cstdint>
#include <string>
#include <vector>

#include "hc_host_par.h"

namespace hc {
namespace topo {

const int kEdges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
const int kFaces[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

struct TetTopology {
  std::vector<int32_t> edofs;         // ne * L element dofs
  std::vector<int32_t> sorted_verts;  // ne * 4
  std::vector<uint8_t> ess;           // ndof flags
  int64_t ndof = 0, n_edges = 0, n_faces = 0;
  bool explicit_mask = false;
};

enum { kOk = 0, kInvalid = 1, kTooLarge = 2 };

// Returns kOk, or kInvalid / kTooLarge with msg set (the first failing element
// in element order, the first failing boundary triangle in order).
inline int build_tet_topology(int64_t ne, int64_t nv, const int64_t* elem_verts, int p, const uint8_t* ess_mask,
                              int64_t n_bdr, const int64_t* bdr_tris, const int32_t* bdr_attr, int ess_attr_bits,
                              TetTopology& T, std::string& msg) {
  const int L = p == 1 ? 6 : 20;
  T.sorted_verts.assign(ne * 4, 0);
  // 1. sorted element vertices, with a status per element (0 ok, 1 vertex out of
  //    range, 2 repeated vertex); the first failing element in order is reported
  {
    std::vector<uint8_t> bad(ne, 0);
    parallel_for(ne, [&](int64_t lo, int64_t hi) {
      for (int64_t e = lo; e < hi; ++e) {
        int64_t s[4];
        bool in_range = true;
        for (int k = 0; k < 4; ++k) {
          s[k] = elem_verts[4 * e + k];
          if (s[k] < 0 || s[k] >= nv) in_range = false;
        }
        if (!in_range) {
          bad[e] = 1;
          continue;
        }
        std::sort(s, s + 4);
        if (s[0] == s[1] || s[1] == s[2] || s[2] == s[3]) {
          bad[e] = 2;
          continue;
        }
        for (int k = 0; k < 4; ++k) T.sorted_verts[4 * e + k] = (int32_t)s[k];
      }
    });
    for (int64_t e = 0; e < ne; ++e)
      if (bad[e]) {
        msg = bad[e] == 1 ? "hc_create: tet vertex index out of range" : "hc_create: degenerate tet (repeated vertex)";
        return kInvalid;
      }
  }
  const std::vector<int32_t>& sv = T.sorted_verts;
  // 2. edges
  std::vector<uint64_t> ekeys(ne * 6);
  parallel_for(ne, [&](int64_t lo, int64_t hi) {
    for (int64_t e = lo; e < hi; ++e)
      for (int k = 0; k < 6; ++k)
        ekeys[6 * e + k] =
            (uint64_t)sv[4 * e + kEdges[k][0]] * (uint64_t)nv + (uint64_t)sv[4 * e + kEdges[k][1]];
  });
  parallel_sort(ekeys);
  ekeys.erase(std::unique(ekeys.begin(), ekeys.end()), ekeys.end());
  // 3. faces (order 2)
  std::vector<std::array<int32_t, 3>> fkeys;
  if (p == 2) {
    fkeys.resize(ne * 4);
    parallel_for(ne, [&](int64_t lo, int64_t hi) {
      for (int64_t e = lo; e < hi; ++e)
        for (int f = 0; f < 4; ++f)
          fkeys[4 * e + f] = {sv[4 * e + kFaces[f][0]], sv[4 * e + kFaces[f][1]], sv[4 * e + kFaces[f][2]]};
    });
    parallel_sort(fkeys);
    fkeys.erase(std::unique(fkeys.begin(), fkeys.end()), fkeys.end());
  }
  const int64_t nE = (int64_t)ekeys.size(), nF = (int64_t)fkeys.size();
  T.n_edges = nE;
  T.n_faces = nF;
  T.ndof = p == 1 ? nE : 2 * nE + 2 * nF;
  if (T.ndof >= ((int64_t)1 << 31)) {
    msg = "hc_create: more than 2^31 - 1 dofs per problem is not supported";
    return kTooLarge;
  }
  // 4. element dofs
  T.edofs.assign(ne * L, 0);
  parallel_for(ne, [&](int64_t lo, int64_t hi) {
    for (int64_t e = lo; e < hi; ++e) {
      int32_t* dd = &T.edofs[e * L];
      for (int k = 0; k < 6; ++k) {
        const uint64_t key =
            (uint64_t)sv[4 * e + kEdges[k][0]] * (uint64_t)nv + (uint64_t)sv[4 * e + kEdges[k][1]];
        const int64_t g = std::lower_bound(ekeys.begin(), ekeys.end(), key) - ekeys.begin();
        if (p == 1) {
          dd[k] = (int32_t)g;
        } else {
          dd[2 * k] = (int32_t)(2 * g);
          dd[2 * k + 1] = (int32_t)(2 * g + 1);
        }
      }
      if (p == 2)
        for (int f = 0; f < 4; ++f) {
          const std::array<int32_t, 3> key{sv[4 * e + kFaces[f][0]], sv[4 * e + kFaces[f][1]],
                                           sv[4 * e + kFaces[f][2]]};
          const int64_t g = std::lower_bound(fkeys.begin(), fkeys.end(), key) - fkeys.begin();
          dd[12 + 2 * f] = (int32_t)(2 * nE + 2 * g);
          dd[12 + 2 * f + 1] = (int32_t)(2 * nE + 2 * g + 1);
        }
    }
  });
  // 5. essential flags
  T.ess.assign(T.ndof, 0);
  T.explicit_mask = false;
  if (ess_mask) {
    for (int64_t i = 0; i < T.ndof; ++i) T.ess[i] = ess_mask[i] ? 1 : 0;
    T.explicit_mask = true;
  } else if (n_bdr > 0 && bdr_tris && bdr_attr) {
    for (int64_t b = 0; b < n_bdr; ++b) {
      const int a = bdr_attr[b];
      if (a < 1 || a > 31 || !((ess_attr_bits >> (a - 1)) & 1)) continue;
      int64_t s[3] = {bdr_tris[3 * b], bdr_tris[3 * b + 1], bdr_tris[3 * b + 2]};
      std::sort(s, s + 3);
      const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};
      for (auto& q : pr) {
        const uint64_t key = (uint64_t)s[q[0]] * (uint64_t)nv + (uint64_t)s[q[1]];
        auto it = std::lower_bound(ekeys.begin(), ekeys.end(), key);
        if (it == ekeys.end() || *it != key) {
          msg = "hc_create: boundary triangle edge is not an edge of the mesh";
          return kInvalid;
        }
        const int64_t g = it - ekeys.begin();
        if (p == 1) {
          T.ess[g] = 1;
        } else {
          T.ess[2 * g] = T.ess[2 * g + 1] = 1;
        }
      }
      if (p == 2) {
        const std::array<int32_t, 3> key{(int32_t)s[0], (int32_t)s[1], (int32_t)s[2]};
        auto it = std::lower_bound(fkeys.begin(), fkeys.end(), key);
        if (it == fkeys.end() || *it != key) {
          msg = "hc_create: boundary triangle is not a face of the mesh";
          return kInvalid;
        }
        const int64_t g = it - fkeys.begin();
        T.ess[2 * nE + 2 * g] = T.ess[2 * nE + 2 * g + 1] = 1;
      }
    }
  }
  return kOk;
}

}  // namespace topo
}  // namespace hc

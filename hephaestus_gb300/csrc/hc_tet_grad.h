// hc_tet_grad.h -- local coefficients of the exact discrete gradient on a
// Nedelec tet (basis of hc_tet.cu: vertices sorted by global index,
// W_ab = l_a grad l_b - l_b grad l_a; order 2: l_a W_ab, l_b W_ab per edge ab
// and F0 = l_k W_ij, F1 = l_j W_ik per face i<j<k).  Shared by the CUDA kernels
// of hc_tetaux.cu and a CPU test (tests/tet_grad_check.cpp), which checks the
// tables against the oracle's basis.
//
//   grad l_v:        edge ab: u_b - u_a (both order-2 dofs of the edge);
//                    face ijk: F0 = -u_i + 2u_j - u_k, F1 = -u_i - u_j + 2u_k.
//   grad(l_a l_b):   l_a W_ab - l_b W_ab, and on each face containing ab
//                    (F0, F1) x (1, -2) if ab = ij, (-2, 1) if ab = ik, (1, 1) if ab = jk.
#pragma once

#ifdef __CUDACC__
#define HC_HD __host__ __device__
#else
#define HC_HD
#endif

namespace hc {

const int kHEdges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
const int kHFaces[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

// local vertices (up to 3) and coefficients of local dof I in the gradient of
// the vertex hat functions; returns the number of vertices
HC_HD inline int ta_local(int p, int I, const int (*E)[2], const int (*F)[3], int v[3], float c[3]) {
  if (p == 1 || I < 12) {
    const int k = p == 1 ? I : I / 2;
    v[0] = E[k][0];
    v[1] = E[k][1];
    c[0] = -1.f;
    c[1] = 1.f;
    return 2;
  }
  const int f = (I - 12) / 2, s = (I - 12) % 2;
  v[0] = F[f][0];
  v[1] = F[f][1];
  v[2] = F[f][2];
  c[0] = -1.f;
  c[1] = s == 0 ? 2.f : -1.f;
  c[2] = s == 0 ? -1.f : 2.f;
  return 3;
}

// coefficient of local order-2 dof I in the gradient of the bubble of local edge ke
HC_HD inline float ta_bubble(int I, int ke, const int (*E)[2], const int (*F)[3]) {
  if (I < 12) return (I / 2 == ke) ? ((I % 2 == 0) ? 1.f : -1.f) : 0.f;
  const int f = (I - 12) / 2, s = (I - 12) % 2;
  const int i = F[f][0], j = F[f][1], k = F[f][2], a = E[ke][0], b = E[ke][1];
  if (a == i && b == j) return s == 0 ? 1.f : -2.f;
  if (a == i && b == k) return s == 0 ? -2.f : 1.f;
  if (a == j && b == k) return 1.f;
  return 0.f;
}

}  // namespace hc

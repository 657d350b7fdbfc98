// hc_tetaux.cu -- auxiliary-space gradient correction for Nedelec tets:
//
//   B = D^-1 + (PG) V (PG)^T,   V ~ ((PG)^T J (PG))^-1,
//
// the gradient part of the AMS preconditioner HypreAMS builds for the H(curl)
// solve (the Hiptmair-Xu splitting; hcurl_formulation.cpp:81-85 installs
// HypreAMS).  G is the exact discrete gradient from nodal functions (P1
// vertex hats; for order 2 also the quadratic edge bubbles) into this Nedelec
// space (P masks essential dofs), and V applies one V-cycle of a
// smoothed-aggregation algebraic multigrid to the P1 nodal operator
// A_n = (PG)^T K (PG), assembled from the element matrices.
//
// Discrete gradient, in the basis of hc_tet.cu (vertices sorted by global
// index, W_ab = l_a grad l_b - l_b grad l_a):
//   grad l_v = sum_{j != v} W_jv, so G u has W_ab-coefficient u_b - u_a;
//   W_ab = l_a W_ab + l_b W_ab + sum_{c != a,b} l_c W_ab, and on a face i<j<k
//   (functions F0 = l_k W_ij, F1 = l_j W_ik) l_i W_jk = F1 - F0, so
//   order 1: edge ab: u_b - u_a;
//   order 2: both dofs of edge ab: u_b - u_a; face ijk: F0 = -u_i + 2u_j - u_k,
//            F1 = -u_i - u_j + 2u_k.
// Order 2 adds the gradients of the quadratic edge bubbles l_a l_b (a < b), the
// slow modes of Jacobi on order-2 meshes with coefficient jumps:
//   grad(l_a l_b) = l_a W_ab - l_b W_ab + sum over faces containing ab of
//   (F0, F1) x (1, -2) for the face's edge ij, (-2, 1) for ik, (1, 1) for jk,
// so on the P2 nodal space (vertices + edge bubbles) V = D_L^-1 + P0 V1 P0^T
// with V1 the AMG V-cycle on the vertex block and D_L the diagonal of the P2
// nodal operator (P0 injects P1 into the vertex functions of the hierarchical
// P2 basis).
//
// AMG (setup on the host in FP64, V-cycle on the device in FP32, all right-hand
// sides at once in the [node][rhs] layout): strength |a_ij| > 0.08 sqrt(a_ii a_jj),
// three-pass greedy aggregation, tentative prolongator normalised per
// aggregate, one damped-Jacobi smoothing step (omega = 4/3 / lambda_max(D^-1 A)),
// Galerkin coarse operators R A P with R = P^T, Chebyshev-Jacobi degree 2
// smoothing on the interval [lambda_max / 30, lambda_max], and a dense inverse
// of the diagonally scaled coarsest operator (<= 1500 nodes).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "hc_amg_host.h"
#include "hc_tet_grad.h"
#include "hc_tetaux_host.h"
#include "hc_internal.h"

namespace hc {

namespace {
constexpr int kTaMaxLevels = 10;
constexpr int kTaCoarse = 1500;
constexpr int kTaDenseMax = 1500;
constexpr double kTaTheta = 0.08;
constexpr double kTaRatio = 30.0;
constexpr int kTaThreads = 256;
constexpr int kTaMaxBlocks = 152 * 8;

__constant__ int c_ta_edges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
__constant__ int c_ta_faces[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
struct DCsr {
  const int* rp = nullptr;
  const int* ci = nullptr;
  const float* va = nullptr;
};
struct TaLevel {
  int n = 0;
  DCsr A, P, R;
  float* dinv = nullptr;
  float c0 = 0, c1 = 0, c2 = 0;  // Chebyshev: step 0 d = c0 D^-1 r, step 1 d = c1 d + c2 D^-1 r
  float *xa = nullptr, *xb = nullptr, *b = nullptr, *r = nullptr, *d = nullptr;
};

// one warp per row, at most 16 blocks of 8 warps per SM
static unsigned ta_rows_grid(int64_t rows) {
  const int64_t b = (rows + kTaThreads / 32 - 1) / (kTaThreads / 32);
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}
static unsigned ta_grid(int64_t work) {
  const int64_t b = (work + kTaThreads - 1) / kTaThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, kTaMaxBlocks));
}
}  // namespace

struct TetAux {
  int nlev = 0;  // levels with sparse operators; the last of them is solved densely
  TaLevel lev[kTaMaxLevels];
  float* cinv = nullptr;  // nc x nc inverse of S A S (coarsest)
  float* cs = nullptr;    // S = diag^-1/2 (coarsest)
  int nfree = 0;          // free vertices (rows of the AMG)
  int nn = 0;             // nodal rows: free vertices, then free edge bubbles (order 2)
  int* gnode = nullptr;   // 3 per dof: free vertex indices, -1 = none
  int* gedge = nullptr;   // 3 per dof: free edge-bubble indices (order 2), -1 = none
  float* dl = nullptr;    // 1 / diag of the nodal operator, nn (order 2)
  float* rn = nullptr;    // nodal residual G^T r, nn x rcap
  DCsr Gt;                // G^T, nn x ndof
  int64_t nface0 = 0;     // first face dof (order 2); ndof for order 1
  int rcap = 0;
  std::vector<void*> owned;  // device blocks
};

// ---- device kernels ---------------------------------------------------------------
// element nodal matrices A_e = G_e^T K_e G_e (G_e rows of essential dofs zeroed), upper triangle
template <int L>
__global__ void k_ta_elem(int64_t ne, int p, const double* __restrict__ K, const int32_t* __restrict__ edofs,
                          const uint8_t* __restrict__ ess, double* __restrict__ out) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  float g[L][4];
  for (int I = 0; I < L; ++I) {
    int v[3];
    float c[3];
    const int nn = ta_local(p, I, c_ta_edges, c_ta_faces, v, c);
    for (int k = 0; k < 4; ++k) g[I][k] = 0.f;
    if (ess[edofs[e * L + I]]) continue;
    for (int k = 0; k < nn; ++k) g[I][v[k]] = c[k];
  }
  const double* Ke = K + e * L * L;
  double A[4][4];
  for (int b = 0; b < 4; ++b) {
    double t[L];
    for (int I = 0; I < L; ++I) {
      double s = 0.0;
      for (int J = 0; J < L; ++J) s += Ke[I * L + J] * (double)g[J][b];
      t[I] = s;
    }
    for (int a = 0; a < 4; ++a) {
      double s = 0.0;
      for (int I = 0; I < L; ++I) s += (double)g[I][a] * t[I];
      A[a][b] = s;
    }
  }
  const int nout = p == 1 ? 10 : 16;
  int k = 0;
  for (int a = 0; a < 4; ++a)
    for (int b = a; b < 4; ++b) out[e * nout + k++] = 0.5 * (A[a][b] + A[b][a]);
  if (p == 1) return;
  // diagonal of the edge-bubble block: g_k^T K g_k for the 6 local edges
  for (int ke = 0; ke < 6; ++ke) {
    float gb[L];
    for (int I = 0; I < L; ++I) gb[I] = ess[edofs[e * L + I]] ? 0.f : ta_bubble(I, ke, c_ta_edges, c_ta_faces);
    double sacc = 0.0;
    for (int I = 0; I < L; ++I) {
      if (gb[I] == 0.f) continue;
      double t = 0.0;
      for (int J = 0; J < L; ++J) t += Ke[I * L + J] * (double)gb[J];
      sacc += (double)gb[I] * t;
    }
    out[e * nout + 10 + ke] = sacc;
  }
}

// y = G u on all dofs (u on mesh vertices): every element writes its dofs (equal values)
template <int L>
__global__ void k_ta_grad(int64_t ne, int p, const int32_t* __restrict__ sv, const int32_t* __restrict__ edofs,
                          const double* __restrict__ u, double* __restrict__ y) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double uv[4];
  for (int k = 0; k < 4; ++k) uv[k] = u[sv[4 * e + k]];
  for (int I = 0; I < L; ++I) {
    int v[3];
    float c[3];
    const int nn = ta_local(p, I, c_ta_edges, c_ta_faces, v, c);
    double s = 0.0;
    for (int k = 0; k < nn; ++k) s += (double)c[k] * uv[v[k]];
    y[edofs[e * L + I]] = s;
  }
}

// Node-major kernels over [row][R] blocks: a thread owns W consecutive columns of
// one row (W = 4 for R >= 4: 128-bit accesses for FP32, two 128-bit for FP64).
template <int R>
struct TaW {
  static constexpr int W = R >= 4 ? 4 : 1;
  static constexpr int G = R / W;  // threads per row
};
#define TA_VLOOP(t, n, R)                                                                          \
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < (int64_t)(n) * TaW<R>::G; \
       t += (int64_t)gridDim.x * blockDim.x)

template <int W>
__device__ __forceinline__ void ldv(const float* __restrict__ p, float (&o)[W]) {
  if constexpr (W == 4) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    o[0] = q.x;
    o[1] = q.y;
    o[2] = q.z;
    o[3] = q.w;
  } else {
    o[0] = *p;
  }
}
template <int W>
__device__ __forceinline__ void ldv(const double* __restrict__ p, double (&o)[W]) {
  if constexpr (W == 4) {
    const double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
    o[0] = a.x;
    o[1] = a.y;
    o[2] = b.x;
    o[3] = b.y;
  } else {
    o[0] = *p;
  }
}
template <int W>
__device__ __forceinline__ void stv(float* __restrict__ p, const float (&o)[W]) {
  if constexpr (W == 4)
    *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
  else
    *p = o[0];
}
template <int W>
__device__ __forceinline__ void stv(double* __restrict__ p, const double (&o)[W]) {
  if constexpr (W == 4) {
    *reinterpret_cast<double2*>(p) = make_double2(o[0], o[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(o[2], o[3]);
  } else {
    *p = o[0];
  }
}

// Row-block kernels of the V-cycle: one warp per row, lane = column c (R
// lanes) x nonzero slice (32 / R slices), slices combined by shuffles; the
// row's elementwise work is done by the first slice.
template <int R>
struct TaRow {
  static constexpr int S = 32 / R;
};
#define TA_WARP_ROWS(i, n)                                                              \
  const int lane = threadIdx.x & 31, c = lane % R, slice = lane / R;                    \
  (void)c;                                                                              \
  (void)slice;                                                                          \
  for (int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < (n);   \
       i += (int)(((int64_t)gridDim.x * blockDim.x) >> 5))

template <int R>
__device__ __forceinline__ float ta_row(const DCsr& M, int i, int c, int slice, const float* __restrict__ x) {
  float s = 0.f;
  const int e = M.rp[i + 1];
  for (int k = M.rp[i] + slice; k < e; k += TaRow<R>::S) s += M.va[k] * x[(int64_t)M.ci[k] * R + c];
#pragma unroll
  for (int o = R; o < 32; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  return s;
}

// b = G^T r (nn nodal rows); fuse: x = d = c0 D^-1 b on the nv vertex rows
// (first Chebyshev step of the AMG's finest level).  One warp per row: lane =
// column group (W columns, 128-bit accesses) x nonzero slice.
template <typename T, int R>
__global__ void __launch_bounds__(kTaThreads)
    k_ta_gt(int n, int nv, DCsr Gt, const T* __restrict__ r, float* __restrict__ b, float* __restrict__ x,
            float* __restrict__ d, const float* __restrict__ dinv, float c0, int fuse, const int* done) {
  if (done && *done) return;
  constexpr int W = TaW<R>::W, G = TaW<R>::G, S = 32 / G;
  const int lane = threadIdx.x & 31, c = (lane % G) * W, slice = lane / G;
  for (int i = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < n;
       i += (int)(((int64_t)gridDim.x * blockDim.x) >> 5)) {
    T sacc[W];
#pragma unroll
    for (int w = 0; w < W; ++w) sacc[w] = T(0);
    const int e = Gt.rp[i + 1];
    for (int k = Gt.rp[i] + slice; k < e; k += S) {
      const T a = (T)Gt.va[k];
      T rv[W];
      ldv<W>(r + (int64_t)Gt.ci[k] * R + c, rv);
#pragma unroll
      for (int w = 0; w < W; ++w) sacc[w] += a * rv[w];
    }
#pragma unroll
    for (int o = G; o < 32; o <<= 1)
#pragma unroll
      for (int w = 0; w < W; ++w) sacc[w] += __shfl_xor_sync(0xffffffffu, sacc[w], o);
    if (slice == 0) {
      const int64_t q = (int64_t)i * R + c;
      float bs[W];
#pragma unroll
      for (int w = 0; w < W; ++w) bs[w] = (float)sacc[w];
      stv<W>(b + q, bs);
      if (fuse && i < nv) {
        const float f = c0 * dinv[i];
#pragma unroll
        for (int w = 0; w < W; ++w) bs[w] *= f;
        stv<W>(d + q, bs);
        stv<W>(x + q, bs);
      }
    }
  }
}

// Chebyshev step: r = b - A xin; d = (first ? 0 : c1 d) + c2 D^-1 r; xout = xin + d
template <int R>
__global__ void __launch_bounds__(kTaThreads)
    k_ta_step(int n, DCsr A, const float* __restrict__ dinv, const float* __restrict__ b,
              const float* __restrict__ xin, float* __restrict__ xout, float* __restrict__ d, float c1, float c2,
              int first, const int* done) {
  if (done && *done) return;
  TA_WARP_ROWS(i, n) {
    const float ax = ta_row<R>(A, i, c, slice, xin);
    if (slice == 0) {
      const int64_t q = (int64_t)i * R + c;
      const float dn = (first ? 0.f : c1 * d[q]) + c2 * dinv[i] * (b[q] - ax);
      d[q] = dn;
      xout[q] = xin[q] + dn;
    }
  }
}

template <int R>
__global__ void __launch_bounds__(kTaThreads)
    k_ta_resid(int n, DCsr A, const float* __restrict__ b, const float* __restrict__ x, float* __restrict__ r,
               const int* done) {
  if (done && *done) return;
  TA_WARP_ROWS(i, n) {
    const float ax = ta_row<R>(A, i, c, slice, x);
    if (slice == 0) {
      const int64_t q = (int64_t)i * R + c;
      r[q] = b[q] - ax;
    }
  }
}

// bc = R r; fuse: xc = dc = c0 D^-1 bc
template <int R>
__global__ void __launch_bounds__(kTaThreads)
    k_ta_restrict(int nc, DCsr Rm, const float* __restrict__ r, float* __restrict__ bc, float* __restrict__ xc,
                  float* __restrict__ dc, const float* __restrict__ dinv, float c0, int fuse, const int* done) {
  if (done && *done) return;
  TA_WARP_ROWS(i, nc) {
    const float sv = ta_row<R>(Rm, i, c, slice, r);
    if (slice == 0) {
      const int64_t q = (int64_t)i * R + c;
      bc[q] = sv;
      if (fuse) {
        const float dv = c0 * dinv[i] * sv;
        dc[q] = dv;
        xc[q] = dv;
      }
    }
  }
}

template <int R>
__global__ void __launch_bounds__(kTaThreads)
    k_ta_prolong(int n, DCsr P, const float* __restrict__ xc, float* __restrict__ x, const int* done) {
  if (done && *done) return;
  TA_WARP_ROWS(i, n) {
    const float pv = ta_row<R>(P, i, c, slice, xc);
    if (slice == 0) x[(int64_t)i * R + c] += pv;
  }
}

// x = S Cinv S b (coarsest level)
template <int R>
__global__ void __launch_bounds__(kTaThreads)
    k_ta_dense(int nc, const float* __restrict__ cinv, const float* __restrict__ cs, const float* __restrict__ b,
               float* __restrict__ x, const int* done) {
  if (done && *done) return;
  TA_WARP_ROWS(i, nc) {
    const float* row = cinv + (int64_t)i * nc;
    float acc = 0.f;
    for (int j = slice; j < nc; j += TaRow<R>::S) acc += row[j] * cs[j] * b[(int64_t)j * R + c];
#pragma unroll
    for (int o = R; o < 32; o <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (slice == 0) x[(int64_t)i * R + c] = cs[i] * acc;
  }
}

// z = D^-1 r + (PG) x with the nodal correction x = V rn: vertex rows
// x = x0 + D_L^-1 rn (x0 the V-cycle result), edge-bubble rows x = D_L^-1 rn
// (order 2; gedge == nullptr for order 1: x = x0)
template <typename T, int R>
__global__ void __launch_bounds__(kTaThreads)
    k_ta_g(int64_t ndof, const int* __restrict__ gnode, const int* __restrict__ gedge, int64_t nface0, int nv,
           const float* __restrict__ x0, const float* __restrict__ rn, const float* __restrict__ dl,
           const T* __restrict__ r, const T* __restrict__ dinv, T* __restrict__ z, const int* done) {
  if (done && *done) return;
  constexpr int W = TaW<R>::W, G = TaW<R>::G;
  TA_VLOOP(t, ndof, R) {
    const int64_t dof = t / G;
    const int c = (int)(t % G) * W;
    const bool face = dof >= nface0;
    const bool s1 = face && ((dof - nface0) & 1);
    float v[W];
#pragma unroll
    for (int w = 0; w < W; ++w) v[w] = 0.f;
    auto addv = [&](int nd, float coef) {  // vertex row: coef (x0 + D_L^-1 rn)
      const int64_t q = (int64_t)nd * R + c;
      float xv[W];
      ldv<W>(x0 + q, xv);
      if (dl) {
        float rv[W];
        ldv<W>(rn + q, rv);
        const float f = dl[nd];
#pragma unroll
        for (int w = 0; w < W; ++w) xv[w] += f * rv[w];
      }
#pragma unroll
      for (int w = 0; w < W; ++w) v[w] += coef * xv[w];
    };
    auto adde = [&](int ge, float coef) {  // edge-bubble row: coef D_L^-1 rn
      const int nd = nv + ge;
      float rv[W];
      ldv<W>(rn + (int64_t)nd * R + c, rv);
      const float f = coef * dl[nd];
#pragma unroll
      for (int w = 0; w < W; ++w) v[w] += f * rv[w];
    };
    {
      const int n0 = gnode[3 * dof], n1 = gnode[3 * dof + 1], n2 = gnode[3 * dof + 2];
      if (n0 >= 0) addv(n0, -1.f);
      if (n1 >= 0) addv(n1, face ? (s1 ? -1.f : 2.f) : 1.f);
      if (n2 >= 0) addv(n2, s1 ? 2.f : -1.f);
    }
    if (gedge) {
      const int e0 = gedge[3 * dof], e1 = gedge[3 * dof + 1], e2 = gedge[3 * dof + 2];
      // edge dofs: (+1 | -1) on their own bubble; face dofs F0: (1, -2, 1), F1: (-2, 1, 1) on edges ij, ik, jk
      if (e0 >= 0) adde(e0, face ? (s1 ? -2.f : 1.f) : (((dof & 1) == 0) ? 1.f : -1.f));
      if (e1 >= 0) adde(e1, s1 ? 1.f : -2.f);
      if (e2 >= 0) adde(e2, 1.f);
    }
    const int64_t o = dof * R + c;
    T rv[W], zv[W];
    ldv<W>(r + o, rv);
    const T di = dinv[dof];
#pragma unroll
    for (int w = 0; w < W; ++w) zv[w] = di * rv[w] + (T)v[w];
    stv<W>(z + o, zv);
  }
}

// ---- host AMG setup: hc_amg_host.h ------------------------------------------------------
using amg::HCsr;

template <typename V>
static cudaError_t upload(hcop* h, TetAux* X, const std::vector<V>& v, const V** out) {
  void* p = nullptr;
  const size_t bytes = std::max<size_t>(1, v.size()) * sizeof(V);
  cudaError_t e = dmalloc(h, &p, bytes);
  if (e != cudaSuccess) return e;
  X->owned.push_back(p);
  if (!v.empty()) e = cudaMemcpyAsync(p, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice, h->stream);
  *out = static_cast<const V*>(p);
  return e;
}

static cudaError_t upload_csr(hcop* h, TetAux* X, const HCsr& M, DCsr& D) {
  std::vector<float> vf(M.va.begin(), M.va.end());
  cudaError_t e = upload(h, X, M.rp, &D.rp);
  if (e == cudaSuccess) e = upload(h, X, M.ci, &D.ci);
  if (e == cudaSuccess) e = upload(h, X, vf, &D.va);
  return e;
}

void tetaux_free(hcop* h) {
  TetAux* X = static_cast<TetAux*>(h->taux);
  if (!X) return;
  for (void* p : X->owned) dfree(h, p);
  delete X;
  h->taux = nullptr;
}

hc_status tetaux_setup(hcop* h) {
  if (h->taux) return HC_OK;
  if (h->type != HC_TET) {
    h->err = "tetaux_setup: tet meshes only";
    return HC_ENOTSUP;
  }
  const int p = h->p, L = p == 1 ? 6 : 20;
  const int64_t ne = h->ne, N = h->ndof;
  cudaStream_t s = h->stream;
  std::vector<int32_t> sv(ne * 4), ed(ne * L);
  const int nout = p == 1 ? 10 : 16;  // vertex block (upper triangle) + edge-bubble diagonal
  std::vector<double> Ae(ne * nout);
  double* dAe = nullptr;
  HC_CUDA_TRY(h, dmalloc(h, (void**)&dAe, Ae.size() * sizeof(double)));
  if (L == 6)
    k_ta_elem<6><<<(unsigned)((ne + 127) / 128), 128, 0, s>>>(ne, p, h->tetK64, h->tet_edofs, h->ess, dAe);
  else
    k_ta_elem<20><<<(unsigned)((ne + 127) / 128), 128, 0, s>>>(ne, p, h->tetK64, h->tet_edofs, h->ess, dAe);
  HC_CUDA_TRY(h, cudaGetLastError());
  HC_CUDA_TRY(h, cudaMemcpyAsync(Ae.data(), dAe, Ae.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
  HC_CUDA_TRY(h, cudaMemcpyAsync(sv.data(), h->tet_sv, sv.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  HC_CUDA_TRY(h, cudaMemcpyAsync(ed.data(), h->tet_edofs, ed.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  HC_CUDA_TRY(h, cudaStreamSynchronize(s));
  dfree(h, dAe);
  AuxStructure S;
  std::string smsg;
  if (!build_aux_structure(p, ne, N, h->n_edges, sv.data(), ed.data(), h->ess_host.data(), Ae.data(), S, smsg)) {
    h->err = smsg;
    return HC_ENOTSUP;
  }
  const int nfree = S.nfree, nn = S.nn;
  const int64_t nface0 = S.nface0;
  std::vector<int>& gnode = S.gnode;
  std::vector<int>& gedge = S.gedge;
  std::vector<float>& dl = S.dl;
  HCsr& Gt = S.Gt;
  HCsr& A = S.A;

  TetAux* X = new TetAux();
  h->taux = X;
  X->nfree = nfree;
  X->nn = nn;
  X->nface0 = nface0;
  cudaError_t e = cudaSuccess;
  {
    const int* gp = nullptr;
    e = upload(h, X, gnode, &gp);
    X->gnode = const_cast<int*>(gp);
    if (e == cudaSuccess && p == 2) {
      e = upload(h, X, gedge, &gp);
      X->gedge = const_cast<int*>(gp);
      const float* dp = nullptr;
      if (e == cudaSuccess) e = upload(h, X, dl, &dp);
      X->dl = const_cast<float*>(dp);
    }
  }
  if (e == cudaSuccess) e = upload_csr(h, X, Gt, X->Gt);
  // hierarchy
  HCsr cur = std::move(A);
  int nl = 0;
  std::vector<float> cinv, csc;
  for (;;) {
    TaLevel& Lv = X->lev[nl];
    Lv.n = cur.n;
    const std::vector<double> dg = amg::diagonal(cur);
    for (int i = 0; i < cur.n; ++i)
      if (!(dg[i] > 0.0)) {
        h->err = "auxiliary-space preconditioner: nodal operator has a non-positive diagonal";
        tetaux_free(h);
        return HC_ENOTSUP;
      }
    const double lmax = 1.1 * amg::lmax_scaled(cur, dg);
    const double lmin = lmax / kTaRatio;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    const double s1 = theta / delta, rho0 = 1.0 / s1, rho1 = 1.0 / (2.0 * s1 - rho0);
    Lv.c0 = (float)(1.0 / theta);
    Lv.c1 = (float)(rho1 * rho0);
    Lv.c2 = (float)(2.0 * rho1 / delta);
    std::vector<float> di(cur.n);
    for (int i = 0; i < cur.n; ++i) di[i] = (float)(1.0 / dg[i]);
    const float* dd = nullptr;
    if (e == cudaSuccess) e = upload(h, X, di, &dd);
    Lv.dinv = const_cast<float*>(dd);
    if (e == cudaSuccess) e = upload_csr(h, X, cur, Lv.A);
    ++nl;
    const bool last_allowed = cur.n <= kTaDenseMax;
    if (cur.n <= kTaCoarse || nl == kTaMaxLevels) {
      if (!last_allowed || !amg::dense_scaled_inverse(cur, dg, cinv, csc)) cinv.clear();
      break;
    }
    std::vector<int> agg;
    const int na = amg::aggregate(cur, dg, kTaTheta, agg);
    if (na >= (int)(0.85 * cur.n) && last_allowed) {  // coarsening stalled
      if (!amg::dense_scaled_inverse(cur, dg, cinv, csc)) cinv.clear();
      break;
    }
    const double lraw = lmax / 1.1;
    HCsr P = amg::smooth_prolongator(cur, dg, agg, na, 4.0 / (3.0 * lraw));
    HCsr R = amg::transpose(P);
    HCsr Ac = amg::spgemm(R, amg::spgemm(cur, P));
    if (e == cudaSuccess) e = upload_csr(h, X, P, Lv.P);
    if (e == cudaSuccess) e = upload_csr(h, X, R, Lv.R);
    cur = std::move(Ac);
  }
  X->nlev = nl;
  if (!cinv.empty()) {
    const float* ci = nullptr;
    const float* cs = nullptr;
    if (e == cudaSuccess) e = upload(h, X, cinv, &ci);
    if (e == cudaSuccess) e = upload(h, X, csc, &cs);
    X->cinv = const_cast<float*>(ci);
    X->cs = const_cast<float*>(cs);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    h->err = std::string("auxiliary-space preconditioner setup: ") + cudaGetErrorString(e);
    tetaux_free(h);
    return HC_ECUDA;
  }
  return HC_OK;
}

hc_status tetaux_reserve(hcop* h, int R) {
  TetAux* X = static_cast<TetAux*>(h->taux);
  if (!X) return HC_EINVAL;
  if (X->rcap >= R) return HC_OK;
  // older (smaller) blocks stay owned until the handle goes
  auto grab = [&](float** q, size_t rows) -> bool {
    void* pnew = nullptr;
    if (dmalloc(h, &pnew, rows * R * sizeof(float)) != cudaSuccess) return false;
    X->owned.push_back(pnew);
    *q = static_cast<float*>(pnew);
    return true;
  };
  bool ok = grab(&X->rn, X->nn);
  for (int l = 0; l < X->nlev && ok; ++l) {
    TaLevel& Lv = X->lev[l];
    ok = grab(&Lv.xa, Lv.n) && grab(&Lv.xb, Lv.n) && grab(&Lv.r, Lv.n) && grab(&Lv.d, Lv.n);
    if (ok && l > 0) ok = grab(&Lv.b, Lv.n);
  }
  if (!ok) {
    h->err = "auxiliary-space work vectors allocation failed";
    return HC_ENOMEM;
  }
  X->lev[0].b = X->rn;
  X->rcap = R;
  return HC_OK;
}

template <int R>
static float* ta_vcycle(const TetAux* X, int l, const int* done, cudaStream_t s) {
  const TaLevel& Lv = X->lev[l];
  const unsigned g = ta_rows_grid(Lv.n);
  if (l == X->nlev - 1) {
    if (X->cinv) {
      k_ta_dense<R><<<g, kTaThreads, 0, s>>>(Lv.n, X->cinv, X->cs, Lv.b, Lv.xb, done);
      return Lv.xb;
    }
    // no dense inverse: Chebyshev steps only (x = d = c0 D^-1 b was set by the producer)
    k_ta_step<R><<<g, kTaThreads, 0, s>>>(Lv.n, Lv.A, Lv.dinv, Lv.b, Lv.xa, Lv.xb, Lv.d, Lv.c1, Lv.c2, 0, done);
    return Lv.xb;
  }
  const TaLevel& Nx = X->lev[l + 1];
  const bool next_dense = (l + 1 == X->nlev - 1) && X->cinv;
  k_ta_step<R><<<g, kTaThreads, 0, s>>>(Lv.n, Lv.A, Lv.dinv, Lv.b, Lv.xa, Lv.xb, Lv.d, Lv.c1, Lv.c2, 0, done);
  k_ta_resid<R><<<g, kTaThreads, 0, s>>>(Lv.n, Lv.A, Lv.b, Lv.xb, Lv.r, done);
  k_ta_restrict<R><<<ta_rows_grid(Nx.n), kTaThreads, 0, s>>>(Nx.n, Lv.R, Lv.r, Nx.b, Nx.xa, Nx.d, Nx.dinv,
                                                                      Nx.c0, next_dense ? 0 : 1, done);
  const float* xc = ta_vcycle<R>(X, l + 1, done, s);
  k_ta_prolong<R><<<g, kTaThreads, 0, s>>>(Lv.n, Lv.P, xc, Lv.xb, done);
  k_ta_step<R><<<g, kTaThreads, 0, s>>>(Lv.n, Lv.A, Lv.dinv, Lv.b, Lv.xb, Lv.xa, Lv.d, 0.f, Lv.c0, 1, done);
  k_ta_step<R><<<g, kTaThreads, 0, s>>>(Lv.n, Lv.A, Lv.dinv, Lv.b, Lv.xa, Lv.xb, Lv.d, Lv.c1, Lv.c2, 0, done);
  return Lv.xb;
}

template <typename T, int R>
static cudaError_t ta_apply_r(const hcop* h, const T* r, T* z, const T* dinv, const int* done, cudaStream_t s) {
  const TetAux* X = static_cast<const TetAux*>(h->taux);
  const TaLevel& L0 = X->lev[0];
  const bool dense0 = X->nlev == 1 && X->cinv;
  // level 0's right-hand side is the vertex block of rn (L0.b == X->rn)
  k_ta_gt<T, R><<<ta_rows_grid(X->nn), kTaThreads, 0, s>>>(X->nn, X->nfree, X->Gt, r, X->rn, L0.xa, L0.d,
                                                                    L0.dinv, L0.c0, dense0 ? 0 : 1, done);
  const float* x0 = ta_vcycle<R>(X, 0, done, s);
  k_ta_g<T, R><<<ta_grid(h->ndof * TaW<R>::G), kTaThreads, 0, s>>>(h->ndof, X->gnode, X->gedge, X->nface0, X->nfree, x0,
                                                            X->rn, X->dl, r, dinv, z, done);
  return cudaGetLastError();
}

template <typename T>
cudaError_t tetaux_apply(const hcop* h, int R, const T* r, T* z, const T* dinv, const int* done, cudaStream_t s) {
  const TetAux* X = static_cast<const TetAux*>(h->taux);
  if (!X || X->rcap < R) return cudaErrorInvalidValue;
  switch (R) {
    case 1: return ta_apply_r<T, 1>(h, r, z, dinv, done, s);
    case 2: return ta_apply_r<T, 2>(h, r, z, dinv, done, s);
    case 4: return ta_apply_r<T, 4>(h, r, z, dinv, done, s);
    case 8: return ta_apply_r<T, 8>(h, r, z, dinv, done, s);
    case 16: return ta_apply_r<T, 16>(h, r, z, dinv, done, s);
    case 32: return ta_apply_r<T, 32>(h, r, z, dinv, done, s);
    default: return cudaErrorInvalidValue;
  }
}
template cudaError_t tetaux_apply<double>(const hcop*, int, const double*, double*, const double*, const int*,
                                          cudaStream_t);
template cudaError_t tetaux_apply<float>(const hcop*, int, const float*, float*, const float*, const int*,
                                         cudaStream_t);

cudaError_t tet_gradient(const hcop* h, const double* u, double* y, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(y, 0, h->ndof * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const unsigned b = (unsigned)((h->ne + 127) / 128);
  if (h->p == 1)
    k_ta_grad<6><<<b, 128, 0, s>>>(h->ne, 1, h->tet_sv, h->tet_edofs, u, y);
  else
    k_ta_grad<20><<<b, 128, 0, s>>>(h->ne, 2, h->tet_sv, h->tet_edofs, u, y);
  return cudaGetLastError();
}

}  // namespace hc

extern "C" int32_t hc_aux_levels(const hcop_t* h, int64_t* sizes, int32_t max_levels) {
  if (!h || !h->taux) return 0;
  const hc::TetAux* X = static_cast<const hc::TetAux*>(h->taux);
  for (int l = 0; l < X->nlev && l < max_levels; ++l) sizes[l] = X->lev[l].n;
  if (max_levels > X->nlev) sizes[X->nlev] = X->nn - X->nfree;  // edge-bubble rows after the levels
  return X->nlev;
}

// hc_tet.cu -- Nedelec (first kind) element-matrix path on tetrahedra, orders 1 and 2.
//
// Basis on the element's vertices sorted by global index (conforming without
// sign flips):  W_bc = l_b grad l_c - l_c grad l_b,
//   p = 1: W_ij on the 6 edges;
//   p = 2: l_i W_ij, l_j W_ij on each edge ij, and l_k W_ij, l_j W_ik on each face ijk.
// Edges / faces are numbered in lexicographic order of their sorted vertex
// tuples; dofs: p*edge + s, then 2*n_edges + 2*face + s.
//
// Element matrices K_e = dt nu_e C_e + sigma_e M_e are built in FP64 in closed
// form: every basis function is a sum of (coefficient x barycentric monomial x
// constant vector) terms, its curl likewise, and integrals of barycentric
// monomials over a tet are exact (6|T| prod k_i! / (sum k + 3)!).  They are the
// element matrices MFEM's CurlCurlIntegrator + VectorFEMassIntegrator form
// for element-constant coefficients (src/kernels/curl_curl_kernel.cpp:21-24,
// src/kernels/vector_fe_mass_kernel.cpp:21-24), in this basis.
//
// Apply: one warp per element; lane = (right-hand side, half of the rows); the
// element's dof vectors are gathered (coalesced over right-hand sides), the
// 20 x 20 product accumulated in FP32/FP64, rows scattered with atomic adds.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "hc_internal.h"
#include "hc_reduce.cuh"
#include "hc_tet_topo.h"

namespace hc {

// ---- host topology (hc_tet_topo.h) ------------------------------------------------
hc_status tet_topology(hcop* h, const hc_problem_desc* d, std::vector<int32_t>& edofs,
                       std::vector<int32_t>& sorted_verts) {
  topo::TetTopology T;
  std::string msg;
  const int st = topo::build_tet_topology(d->n_elem, d->n_vert, d->elem_verts, d->order, d->ess_mask, d->n_bdr,
                                          d->bdr_tris, d->bdr_attr, d->ess_attr_bits, T, msg);
  if (st != topo::kOk) {
    h->err = msg;
    return st == topo::kTooLarge ? HC_ENOTSUP : HC_EINVAL;
  }
  edofs.swap(T.edofs);
  sorted_verts.swap(T.sorted_verts);
  h->ess_host.swap(T.ess);
  h->ndof = T.ndof;
  h->n_edges = T.n_edges;
  h->n_faces = T.n_faces;
  h->explicit_mask = T.explicit_mask;
  return HC_OK;
}

// ---- closed-form element matrices ------------------------------------------------
__constant__ int c_tet_edges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
__constant__ int c_tet_faces[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
__device__ __forceinline__ int kEdgesD(int k, int s) { return c_tet_edges[k][s]; }
__device__ __forceinline__ int kFacesD(int f, int s) { return c_tet_faces[f][s]; }

// basis function as value terms (coef, lambda multiset, grad index) and curl
// terms (coef, lambda index or -1, cross(grad u, grad v))
struct VTerm {
  double c;
  int l0, l1;  // lambda indices (-1 = none)
  int g;       // gradient index
};
struct CTerm {
  double c;
  int l;       // lambda index (-1 = none)
  int u, v;    // cross(grad l_u, grad l_v)
};

__device__ __forceinline__ void basis_terms(int p, int I, VTerm* vt, int* nv, CTerm* ct, int* nc) {
  // p = 1: W_bc ; p = 2: l_a W_bc
  int a = -1, b, c;
  if (p == 1) {
    b = kEdgesD(I, 0);
    c = kEdgesD(I, 1);
  } else if (I < 12) {
    const int k = I / 2;
    b = kEdgesD(k, 0);
    c = kEdgesD(k, 1);
    a = (I % 2 == 0) ? b : c;
  } else {
    const int f = (I - 12) / 2, s = (I - 12) % 2;
    const int i = kFacesD(f, 0), j = kFacesD(f, 1), k = kFacesD(f, 2);
    if (s == 0) {
      a = k;
      b = i;
      c = j;
    } else {
      a = j;
      b = i;
      c = k;
    }
  }
  // value: l_a l_b grad l_c - l_a l_c grad l_b
  vt[0] = {1.0, a, b, c};
  vt[1] = {-1.0, a, c, b};
  *nv = 2;
  if (a < 0) {
    // curl W_bc = 2 grad l_b x grad l_c
    ct[0] = {2.0, -1, b, c};
    *nc = 1;
  } else {
    // curl(l_a W_bc) = l_b (grad a x grad c) - l_c (grad a x grad b) + 2 l_a (grad b x grad c)
    ct[0] = {1.0, b, a, c};
    ct[1] = {-1.0, c, a, b};
    ct[2] = {2.0, a, b, c};
    *nc = 3;
  }
}

// integral over the unit-volume-normalised tet of prod lambda_i^{k_i}:
// 6 prod k_i! / (K + 3)!  (multiply by |T|)
__device__ __forceinline__ double mono_int(const int k[4]) {
  const double fact[7] = {1, 1, 2, 6, 24, 120, 720};
  const double inv_fact3[8] = {1.0 / 6, 1.0 / 24, 1.0 / 120, 1.0 / 720, 1.0 / 5040, 1.0 / 40320, 1.0 / 362880,
                               1.0 / 3628800};
  const int K = k[0] + k[1] + k[2] + k[3];
  return 6.0 * fact[k[0]] * fact[k[1]] * fact[k[2]] * fact[k[3]] * inv_fact3[K];
}

__global__ void tet_elem_matrix_kernel(int64_t ne, int p, const double* __restrict__ V,
                                       const int32_t* __restrict__ sv, const double* __restrict__ nu,
                                       const double* __restrict__ sigma, double dt, double* __restrict__ K64,
                                       float* __restrict__ K32, int* __restrict__ bad) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const int L = p == 1 ? 6 : 20;
  const double* v0 = V + 3 * (int64_t)sv[4 * e];
  double J[9];
  for (int cidx = 0; cidx < 3; ++cidx) {
    const double* vc = V + 3 * (int64_t)sv[4 * e + cidx + 1];
    for (int r = 0; r < 3; ++r) J[3 * r + cidx] = vc[r] - v0[r];
  }
  const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
  if (!(fabs(det) > 0.0) || !isfinite(det)) {
    atomicExch(bad, 1);
    return;
  }
  // rows of J^-1 are grad lambda_1..3 (J columns are v_k - v_0)
  double gl[4][3];
  gl[1][0] = (J[4] * J[8] - J[5] * J[7]) / det;
  gl[1][1] = (J[2] * J[7] - J[1] * J[8]) / det;
  gl[1][2] = (J[1] * J[5] - J[2] * J[4]) / det;
  gl[2][0] = (J[5] * J[6] - J[3] * J[8]) / det;
  gl[2][1] = (J[0] * J[8] - J[2] * J[6]) / det;
  gl[2][2] = (J[2] * J[3] - J[0] * J[5]) / det;
  gl[3][0] = (J[3] * J[7] - J[4] * J[6]) / det;
  gl[3][1] = (J[1] * J[6] - J[0] * J[7]) / det;
  gl[3][2] = (J[0] * J[4] - J[1] * J[3]) / det;
  for (int r = 0; r < 3; ++r) gl[0][r] = -(gl[1][r] + gl[2][r] + gl[3][r]);
  double G[4][4];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) G[i][j] = gl[i][0] * gl[j][0] + gl[i][1] * gl[j][1] + gl[i][2] * gl[j][2];
  // cross products grad u x grad v, indexed [u][v]
  double X[4][4][3];
  for (int u = 0; u < 4; ++u)
    for (int v = 0; v < 4; ++v) {
      X[u][v][0] = gl[u][1] * gl[v][2] - gl[u][2] * gl[v][1];
      X[u][v][1] = gl[u][2] * gl[v][0] - gl[u][0] * gl[v][2];
      X[u][v][2] = gl[u][0] * gl[v][1] - gl[u][1] * gl[v][0];
    }
  const double vol = fabs(det) / 6.0;
  const double a = dt * nu[e], s = sigma ? sigma[e] : 0.0;
  for (int I = 0; I < L; ++I) {
    VTerm vi[2], vj[2];
    CTerm ci[3], cj[3];
    int nvi, nci, nvj, ncj;
    basis_terms(p, I, vi, &nvi, ci, &nci);
    for (int Jj = I; Jj < L; ++Jj) {
      basis_terms(p, Jj, vj, &nvj, cj, &ncj);
      double m = 0.0, c = 0.0;
      for (int x = 0; x < nvi; ++x)
        for (int y = 0; y < nvj; ++y) {
          int k[4] = {0, 0, 0, 0};
          if (vi[x].l0 >= 0) k[vi[x].l0]++;
          k[vi[x].l1]++;
          if (vj[y].l0 >= 0) k[vj[y].l0]++;
          k[vj[y].l1]++;
          m += vi[x].c * vj[y].c * G[vi[x].g][vj[y].g] * mono_int(k);
        }
      for (int x = 0; x < nci; ++x)
        for (int y = 0; y < ncj; ++y) {
          int k[4] = {0, 0, 0, 0};
          if (ci[x].l >= 0) k[ci[x].l]++;
          if (cj[y].l >= 0) k[cj[y].l]++;
          const double* A = X[ci[x].u][ci[x].v];
          const double* B = X[cj[y].u][cj[y].v];
          c += ci[x].c * cj[y].c * (A[0] * B[0] + A[1] * B[1] + A[2] * B[2]) * mono_int(k);
        }
      const double val = vol * (a * c + s * m);
      K64[(e * L + I) * L + Jj] = val;
      K64[(e * L + Jj) * L + I] = val;
      K32[(e * L + I) * L + Jj] = (float)val;
      K32[(e * L + Jj) * L + I] = (float)val;
    }
  }
}

// ---- apply -----------------------------------------------------------------------
// y (+)= P K P x for nrhs right-hand sides stored row-major ([dof][rhs]).
// One warp per element: lane = rhs + nrhs * part, rows split between parts.
__device__ __forceinline__ float kval(float v) { return v; }
__device__ __forceinline__ double kval(double v) { return v; }
__device__ __forceinline__ float kval(__nv_bfloat16 v) { return __bfloat162float(v); }

// Y (+)= scale * P K P X for R right-hand sides ([dof][rhs] row-major).  One
// warp per element: the element's X block (L x R) is staged once in shared
// memory, lane i < L owns row i of the element matrix (read once, in TK =
// double, float or bf16), accumulates its R outputs in registers and adds them
// with R/4 128-bit atomics (FP32) or R scalar atomics (FP64).
template <typename T, int L, int R, typename TK>
__global__ void __launch_bounds__(256) tet_apply_rows(int64_t ne, const int32_t* __restrict__ edofs,
                                                      const TK* __restrict__ K, const uint8_t* __restrict__ ess,
                                                      int masked, T scale, const T* __restrict__ x,
                                                      T* __restrict__ y, int vec_ok, const int* done) {
  if (done && *done) return;
  constexpr int W = 8;  // warps per block
  __shared__ __align__(16) T xs_all[W][L * R];
  __shared__ int sdof_all[W][L];
  __shared__ unsigned char sess_all[W][L];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T* xs = xs_all[wid];
  int* sdof = sdof_all[wid];
  unsigned char* sess = sess_all[wid];
  for (int64_t e = (int64_t)blockIdx.x * W + wid; e < ne; e += (int64_t)gridDim.x * W) {
    if (lane < L) {
      const int d = __ldg(edofs + e * L + lane);
      sdof[lane] = d;
      sess[lane] = (masked && ess[d]) ? 1 : 0;
    }
    __syncwarp();
    for (int idx = lane; idx < L * R; idx += 32) {
      const int j = idx / R, r = idx - j * R;
      T v = __ldg(x + (int64_t)sdof[j] * R + r);
      if (sess[j]) v = T(0);
      xs[idx] = v;
    }
    __syncwarp();
    if (lane < L && !sess[lane]) {
      T kr[L];
      const TK* Krow = K + (e * L + lane) * L;
      if constexpr (sizeof(TK) == 2 && L % 4 == 0) {
        // 8-byte loads of 4 bf16
#pragma unroll
        for (int j = 0; j < L; j += 4) {
          const uint2 v = __ldg(reinterpret_cast<const uint2*>(Krow) + j / 4);
          const __nv_bfloat162 a = *reinterpret_cast<const __nv_bfloat162*>(&v.x);
          const __nv_bfloat162 b = *reinterpret_cast<const __nv_bfloat162*>(&v.y);
          const float2 fa = __bfloat1622float2(a), fb = __bfloat1622float2(b);
          kr[j] = fa.x;
          kr[j + 1] = fa.y;
          kr[j + 2] = fb.x;
          kr[j + 3] = fb.y;
        }
      } else {
#pragma unroll
        for (int j = 0; j < L; ++j) kr[j] = (T)kval(Krow[j]);
      }
      T acc[R];
#pragma unroll
      for (int r = 0; r < R; ++r) acc[r] = T(0);
      if constexpr (sizeof(T) == 4 && R % 4 == 0) {
        // 128-bit shared-memory reads of the staged block (broadcast to all rows)
#pragma unroll
        for (int j = 0; j < L; ++j)
#pragma unroll
          for (int r = 0; r < R; r += 4) {
            const float4 xv = *reinterpret_cast<const float4*>(xs + j * R + r);
            acc[r] += kr[j] * xv.x;
            acc[r + 1] += kr[j] * xv.y;
            acc[r + 2] += kr[j] * xv.z;
            acc[r + 3] += kr[j] * xv.w;
          }
      } else {
#pragma unroll
        for (int j = 0; j < L; ++j)
#pragma unroll
          for (int r = 0; r < R; ++r) acc[r] += kr[j] * xs[j * R + r];
      }
      T* yr = y + (int64_t)sdof[lane] * R;
      if constexpr (sizeof(T) == 4 && R % 4 == 0) {
        if (vec_ok) {
#pragma unroll
          for (int q = 0; q < R / 4; ++q)
            atomicAdd(reinterpret_cast<float4*>(yr) + q,
                      make_float4(scale * acc[4 * q], scale * acc[4 * q + 1], scale * acc[4 * q + 2],
                                  scale * acc[4 * q + 3]));
        } else {
#pragma unroll
          for (int r = 0; r < R; ++r) atomicAdd(yr + r, scale * acc[r]);
        }
      } else {
#pragma unroll
        for (int r = 0; r < R; ++r) atomicAdd(yr + r, scale * acc[r]);
      }
    }
    __syncwarp();  // xs is rewritten for the next element
  }
}

// FP64: all 32 lanes stay busy (the FP64 apply is bound by FP64 throughput):
// lanes split into (right-hand side, row subset), element matrix rows read
// by every lane of a subset.
template <int L>
__global__ void __launch_bounds__(256) tet_apply_lanes64(int64_t ne, const int32_t* __restrict__ edofs,
                                                         const double* __restrict__ K,
                                                         const uint8_t* __restrict__ ess, int masked, int nrhs,
                                                         double scale, const double* __restrict__ x,
                                                         double* __restrict__ y, const int* done) {
  if (done && *done) return;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nparts = 32 / nrhs;  // nrhs in {1, 2, 4, 8, 16, 32}
  const int r = lane % nrhs, part = lane / nrhs;
  for (int64_t e = warp; e < ne; e += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    int dof[L];
    double xe[L];
#pragma unroll
    for (int j = 0; j < L; ++j) {
      dof[j] = __ldg(edofs + e * L + j);
      double v = __ldg(x + (int64_t)dof[j] * nrhs + r);
      if (masked && ess[dof[j]]) v = 0.0;
      xe[j] = v;
    }
    const double* Ke = K + e * L * L;
    for (int i = part; i < L; i += nparts) {
      if (masked && ess[dof[i]]) continue;
      double acc = 0.0;
#pragma unroll
      for (int j = 0; j < L; ++j) acc += __ldg(Ke + i * L + j) * xe[j];
      atomicAdd(y + (int64_t)dof[i] * nrhs + r, scale * acc);
    }
  }
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit_wait() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

// Order 2, FP32 vectors, R in {4, 8, 16, 32}: register-tiled, software-pipelined
// form.  32 / R elements per warp; lane (row group g < 4, column group c < R/4)
// of an element computes the 5 x 4 output tile Y[5g .. 5g+4][4c .. 4c+3]: per
// 4-column chunk of the element matrix it reads 5 K quads (128-bit, shared by
// the lanes of its row group) and 4 X quads of the staged block (128-bit
// shared-memory reads), 80 FMAs; outputs leave as 5 128-bit atomic adds.
// Pipeline (per warp, element groups i = 0, 1, ...): before group i computes,
// cp.async copies the X rows of group i + 1 (dofs already in shared memory)
// into the other X buffer and the dof indices of group i + 2 into the third
// dof slot; they land while group i computes and adds.  Rows of essential dofs
// are zeroed after the copies complete.
template <int R, typename TK>
__global__ void __launch_bounds__(256, 3) tet_apply_tiles20(int64_t ne, const int32_t* __restrict__ edofs,
                                                            const TK* __restrict__ K, const uint8_t* __restrict__ ess,
                                                            int masked, float scale, const float* __restrict__ x,
                                                            float* __restrict__ y, const int* done) {
  if (done && *done) return;
  constexpr int L = 20, W = 8, EPW = 32 / R, CG = R / 4;
  constexpr int ND = (L + R - 1) / R;  // dof indices a lane copies per element
  constexpr int NX = L * CG / R;       // X quads a lane copies per element (= 5)
  static_assert(NX * R == L * CG, "X quads split evenly over the element's lanes");
  __shared__ __align__(16) float xs_all[W][2][EPW][L * R];
  __shared__ __align__(16) int sdof_all[W][3][EPW][L];
  __shared__ unsigned char sess_all[W][3][EPW][L];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane / R, t = lane % R, g = t / CG, c = t % CG;
  const int64_t wstride = (int64_t)gridDim.x * W * EPW;
  const int64_t first = ((int64_t)blockIdx.x * W + wid) * EPW;
  if (first >= ne) return;  // uniform over the warp: no shared state with other warps

  auto copy_dofs = [&](int64_t e, int ds) {  // async: dof indices of element e -> slot ds
    if (e >= ne) return;
#pragma unroll
    for (int k = 0; k < ND; ++k) {
      const int j = t + k * R;
      if (j < L) cp_async4(&sdof_all[wid][ds][sub][j], edofs + e * L + j);
    }
  };
  auto copy_x = [&](int64_t e, int ds, int xb) {  // async: X rows of element e (dofs in slot ds) -> buffer xb
    if (e >= ne) return;
#pragma unroll
    for (int k = 0; k < NX; ++k) {
      const int q = t + k * R, j = q / CG, c4 = q - j * CG;
      cp_async16(&xs_all[wid][xb][sub][j * R + 4 * c4],
                 x + (int64_t)sdof_all[wid][ds][sub][j] * R + 4 * c4);
    }
  };
  auto ess_flags = [&](int64_t e, int ds, unsigned char (&er)[NX]) {
#pragma unroll
    for (int k = 0; k < NX; ++k) {
      const int j = (t + k * R) / CG;
      er[k] = (e < ne && masked) ? ess[sdof_all[wid][ds][sub][j]] : 0;
    }
  };
  auto mask_rows = [&](int64_t e, int ds, int xb, const unsigned char (&er)[NX]) {  // after the copies landed
    if (e >= ne) return;
#pragma unroll
    for (int k = 0; k < NX; ++k) {
      const int q = t + k * R, j = q / CG, c4 = q - j * CG;
      if (er[k]) *reinterpret_cast<float4*>(&xs_all[wid][xb][sub][j * R + 4 * c4]) = make_float4(0.f, 0.f, 0.f, 0.f);
      if (c4 == 0) sess_all[wid][ds][sub][j] = er[k];
    }
  };

  // prologue: dofs of groups 0 and 1, X of group 0
  copy_dofs(first + sub, 0);
  copy_dofs(first + wstride + sub, 1);
  cp_async_commit_wait();
  __syncwarp();
  {
    unsigned char er[NX];
    ess_flags(first + sub, 0, er);
    copy_x(first + sub, 0, 0);
    cp_async_commit_wait();
    mask_rows(first + sub, 0, 0, er);
    __syncwarp();
  }
  int it = 0;
  for (int64_t e0 = first; e0 < ne; e0 += wstride, ++it) {
    const int d0 = it % 3, d1 = (it + 1) % 3, d2 = (it + 2) % 3, xb = it & 1;
    const int64_t e = e0 + sub;
    // in flight during the compute: X of group it + 1, dofs of group it + 2
    copy_x(e + wstride, d1, xb ^ 1);
    copy_dofs(e + 2 * wstride, d2);
    if (e < ne) {
      const float* xs = xs_all[wid][xb][sub];
      float acc[5][4];
#pragma unroll
      for (int i = 0; i < 5; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) acc[i][k] = 0.f;
      const TK* Kg = K + (e * L + 5 * g) * L;
#pragma unroll
      for (int j0 = 0; j0 < L; j0 += 4) {
        float kq[5][4];
#pragma unroll
        for (int i = 0; i < 5; ++i) {
          if constexpr (sizeof(TK) == 2) {
            const uint2 v = __ldg(reinterpret_cast<const uint2*>(Kg + i * L + j0));
            const float2 fa = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&v.x));
            const float2 fb = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&v.y));
            kq[i][0] = fa.x;
            kq[i][1] = fa.y;
            kq[i][2] = fb.x;
            kq[i][3] = fb.y;
          } else {
            const float4 v = __ldg(reinterpret_cast<const float4*>(Kg + i * L + j0));
            kq[i][0] = v.x;
            kq[i][1] = v.y;
            kq[i][2] = v.z;
            kq[i][3] = v.w;
          }
        }
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
          const float4 xv = *reinterpret_cast<const float4*>(xs + (j0 + jj) * R + 4 * c);
#pragma unroll
          for (int i = 0; i < 5; ++i) {
            acc[i][0] += kq[i][jj] * xv.x;
            acc[i][1] += kq[i][jj] * xv.y;
            acc[i][2] += kq[i][jj] * xv.z;
            acc[i][3] += kq[i][jj] * xv.w;
          }
        }
      }
#pragma unroll
      for (int i = 0; i < 5; ++i) {
        const int row = 5 * g + i;
        if (sess_all[wid][d0][sub][row]) continue;
        atomicAdd(reinterpret_cast<float4*>(y + (int64_t)sdof_all[wid][d0][sub][row] * R) + c,
                  make_float4(scale * acc[i][0], scale * acc[i][1], scale * acc[i][2], scale * acc[i][3]));
      }
    }
    unsigned char en[NX];
    ess_flags(e + wstride, d1, en);  // reads only the next group's dof slot
    cp_async_commit_wait();
    mask_rows(e + wstride, d1, xb ^ 1, en);
    __syncwarp();  // next group's X, flags and dofs visible to the warp; buffers of this group free
  }
}

// ---- tensor-core form: order 2, 16 right-hand sides, BF16 element matrices ----------------
// One warp per element and step: Y_e^T (16 x 20) = X_e^T (16 x 20) K_e^T with
// mma.sync m16n8k16 + m16n8k8 (BF16 operands, FP32 accumulation): M = the 16
// right-hand sides, K = the element's 20 dofs (16 + 8, the last 4 zero), N =
// its 20 output rows (three tiles of 8).  The B fragments are read straight
// from the BF16 element matrix in HBM (32-bit loads, every entry once); the A
// fragments come from the element's X rows staged in shared memory, split
// into BF16 hi + lo parts (two MMAs) so that the result carries the rounding
// of the BF16 matrix alone.  Y_e goes through shared memory to 128-bit atomic
// adds, one per 4 columns of a row.  Staging is the cp.async pipeline of
// tet_apply_tiles20: X rows of the next element and dof indices of the one
// after land while the current element computes.
constexpr int kTcW = 8;    // warps per block
constexpr int kTcXS = 20;  // row stride (floats) of the staged blocks: conflict-free fragment reads

__device__ __forceinline__ void split_bf16(float v0, float v1, uint32_t& hi, uint32_t& lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(v0, v1);  // .x (low half) = v0
  const __nv_bfloat162 l = __floats2bfloat162_rn(v0 - __low2float(h), v1 - __high2float(h));
  hi = *reinterpret_cast<const uint32_t*>(&h);
  lo = *reinterpret_cast<const uint32_t*>(&l);
}
__device__ __forceinline__ void mma_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
__device__ __forceinline__ void mma_1688(float (&d)[4], const uint32_t (&a)[2], uint32_t b0) {
  asm volatile("mma.sync.aligned.m16n8k8.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5}, {%6}, {%0,%1,%2,%3};\n"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(b0));
}

__global__ void __launch_bounds__(32 * kTcW, 5) tet_apply_mma16(int64_t ne, const int32_t* __restrict__ edofs,
                                                             const __nv_bfloat16* __restrict__ K,
                                                             const uint8_t* __restrict__ ess, int masked, float scale,
                                                             const float* __restrict__ x, float* __restrict__ y,
                                                             const int* done) {
  if (done && *done) return;
  constexpr int L = 20, R = 16;
  __shared__ __align__(16) float xs_all[kTcW][2][L][kTcXS];  // X rows: [dof j][rhs r]
  __shared__ __align__(16) float ds_all[kTcW][L][kTcXS];     // Y_e rows for the scatter
  __shared__ __align__(16) int sdof_all[kTcW][3][L];
  __shared__ unsigned char sess_all[kTcW][3][L];
  const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, tig = lane & 3;
  const int64_t wstride = (int64_t)gridDim.x * kTcW;
  const int64_t first = (int64_t)blockIdx.x * kTcW + wid;
  if (first >= ne) return;  // uniform over the warp: warps share no state

  auto copy_dofs = [&](int64_t e, int ds) {
    if (e < ne && lane < L) cp_async4(&sdof_all[wid][ds][lane], edofs + e * L + lane);
  };
  auto copy_x = [&](int64_t e, int ds, int xb) {  // 20 rows x 4 chunks of 16 bytes
    if (e >= ne) return;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int q = lane + 32 * k;
      if (q < 4 * L) {
        const int j = q >> 2, c4 = q & 3;
        cp_async16(&xs_all[wid][xb][j][4 * c4], x + (int64_t)sdof_all[wid][ds][j] * R + 4 * c4);
      }
    }
  };
  auto mask_rows = [&](int64_t e, int ds, int xb) {  // after the copies landed
    if (e >= ne) return;
    unsigned char f[3] = {0, 0, 0};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int q = lane + 32 * k;
      if (q < 4 * L && masked) f[k] = ess[sdof_all[wid][ds][q >> 2]];
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int q = lane + 32 * k;
      if (q < 4 * L) {
        const int j = q >> 2, c4 = q & 3;
        if (f[k]) *reinterpret_cast<float4*>(&xs_all[wid][xb][j][4 * c4]) = make_float4(0.f, 0.f, 0.f, 0.f);
        if (c4 == 0) sess_all[wid][ds][j] = f[k];
      }
    }
  };

  copy_dofs(first, 0);
  copy_dofs(first + wstride, 1);
  cp_async_commit_wait();
  __syncwarp();
  copy_x(first, 0, 0);
  cp_async_commit_wait();
  __syncwarp();
  mask_rows(first, 0, 0);
  __syncwarp();
  int it = 0;
  for (int64_t e = first; e < ne; e += wstride, ++it) {
    const int d0 = it % 3, d1 = (it + 1) % 3, d2 = (it + 2) % 3, xb = it & 1;
    copy_x(e + wstride, d1, xb ^ 1);
    copy_dofs(e + 2 * wstride, d2);
    const float* xs = &xs_all[wid][xb][0][0];
    // A fragments: A[r][j] = X[dof j][r]; k16 over j < 16, k8 over 16 <= j < 24 (j >= 20 zero)
    uint32_t ah[4], al[4], bh[2] = {0u, 0u}, bl[2] = {0u, 0u};
    split_bf16(xs[(2 * tig) * kTcXS + g], xs[(2 * tig + 1) * kTcXS + g], ah[0], al[0]);
    split_bf16(xs[(2 * tig) * kTcXS + g + 8], xs[(2 * tig + 1) * kTcXS + g + 8], ah[1], al[1]);
    split_bf16(xs[(2 * tig + 8) * kTcXS + g], xs[(2 * tig + 9) * kTcXS + g], ah[2], al[2]);
    split_bf16(xs[(2 * tig + 8) * kTcXS + g + 8], xs[(2 * tig + 9) * kTcXS + g + 8], ah[3], al[3]);
    if (tig < 2) {
      split_bf16(xs[(16 + 2 * tig) * kTcXS + g], xs[(17 + 2 * tig) * kTcXS + g], bh[0], bl[0]);
      split_bf16(xs[(16 + 2 * tig) * kTcXS + g + 8], xs[(17 + 2 * tig) * kTcXS + g + 8], bh[1], bl[1]);
    }
    const uint32_t* Ke = reinterpret_cast<const uint32_t*>(K + e * (L * L));  // 200 words, 4-byte aligned
    float acc[3][4];
#pragma unroll
    for (int nt = 0; nt < 3; ++nt) {
      acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
      const int row = 8 * nt + g;  // output row i = B column n
      uint32_t b0 = 0u, b1 = 0u, b2 = 0u;
      if (row < L) {
        // B[j][i] = K_e[i][j]: pairs along j.  (Streaming, evict-first loads
        // of K were measured: +63 MB of DRAM reads per apply, no faster --
        // a K row's sectors are shared with the next row's loads.)
        const uint32_t* Kr = Ke + row * (L / 2);
        b0 = __ldg(Kr + tig);                   // j = 2 tig, 2 tig + 1
        b1 = __ldg(Kr + 4 + tig);               // j = 2 tig + 8, + 9
        if (tig < 2) b2 = __ldg(Kr + 8 + tig);  // j = 16 + 2 tig, + 1
      }
      mma_16816(acc[nt], ah, b0, b1);
      mma_16816(acc[nt], al, b0, b1);
      mma_1688(acc[nt], bh, b2);
      mma_1688(acc[nt], bl, b2);
    }
    // D[r][i] = Y_e[i][r]: rows r = g, g + 8; columns i = 8 nt + 2 tig, + 1
    float* ds = &ds_all[wid][0][0];
#pragma unroll
    for (int nt = 0; nt < 3; ++nt) {
      const int i0 = 8 * nt + 2 * tig;
      if (i0 < L) {
        ds[i0 * kTcXS + g] = acc[nt][0];
        ds[(i0 + 1) * kTcXS + g] = acc[nt][1];
        ds[i0 * kTcXS + g + 8] = acc[nt][2];
        ds[(i0 + 1) * kTcXS + g + 8] = acc[nt][3];
      }
    }
    __syncwarp();
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int q = lane + 32 * k;
      if (q < 4 * L) {
        const int j = q >> 2, c4 = q & 3;
        if (!sess_all[wid][d0][j]) {
          const float4 v = *reinterpret_cast<const float4*>(&ds[j * kTcXS + 4 * c4]);
          atomicAdd(reinterpret_cast<float4*>(y + (int64_t)sdof_all[wid][d0][j] * R) + c4,
                    make_float4(scale * v.x, scale * v.y, scale * v.z, scale * v.w));
        }
      }
    }
    cp_async_commit_wait();  // X rows of the next element, dofs of the one after
    __syncwarp();
    mask_rows(e + wstride, d1, xb ^ 1);
    __syncwarp();  // flags and rows visible; this element's buffers free
  }
}

static bool tet_mma16_launch(const hcop* h, const __nv_bfloat16* K, const float* x, float* y, int nrhs, bool masked,
                             float scale, const int* done, cudaStream_t s) {
  if (h->p != 2 || nrhs != 16 || ((uintptr_t)x | (uintptr_t)y) % 16 != 0) return false;
  static int resident = 0;  // blocks resident on the device: warps stride over the elements
  if (!resident) {
    int dev = 0, nsm = 0, occ = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    // all of the SM's shared memory for this kernel: 5 blocks of 40.8 KB
    cudaFuncSetAttribute(tet_apply_mma16, cudaFuncAttributePreferredSharedMemoryCarveout,
                         cudaSharedmemCarveoutMaxShared);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, tet_apply_mma16, 32 * kTcW, 0);
    resident = std::max(1, occ) * std::max(1, nsm);
  }
  const int64_t b = (h->ne + kTcW - 1) / kTcW;
  const unsigned blocks = (unsigned)std::min<int64_t>(b, resident);
  tet_apply_mma16<<<blocks, 32 * kTcW, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, masked ? 1 : 0, scale, x, y, done);
  return true;
}

template <typename TK>
static bool tet_tiles20_launch(const hcop* h, const TK* K, const float* x, float* y, int nrhs, bool masked,
                               float scale, const int* done, cudaStream_t s) {
  // 128-bit accesses: x, y 16-byte aligned (rows of R >= 4 floats keep the alignment)
  if (h->p != 2 || ((uintptr_t)x | (uintptr_t)y) % 16 != 0) return false;
  const int m = masked ? 1 : 0;
  auto blocks = [&](int epw) {
    const int64_t b = (h->ne + 8 * epw - 1) / (8 * epw);
    return (unsigned)std::min<int64_t>(b, 152 * 16);
  };
  switch (nrhs) {
    case 4: tet_apply_tiles20<4, TK><<<blocks(8), 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, done); return true;
    case 8: tet_apply_tiles20<8, TK><<<blocks(4), 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, done); return true;
    case 16: tet_apply_tiles20<16, TK><<<blocks(2), 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, done); return true;
    case 32: tet_apply_tiles20<32, TK><<<blocks(1), 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, done); return true;
    default: return false;
  }
}

template <typename T, int L, typename TK>
static cudaError_t tet_rows_launch(const hcop* h, const TK* K, const T* x, T* y, int nrhs, bool masked, T scale,
                                   const int* done, cudaStream_t s) {
  const int W = 8;
  int64_t blocks = (h->ne + W - 1) / W;
  blocks = std::min<int64_t>(blocks, 152 * 16);
  const int vec_ok = ((uintptr_t)y % 16) == 0 ? 1 : 0;
  const int m = masked ? 1 : 0;
  const unsigned b = (unsigned)blocks;
  switch (nrhs) {
    case 1: tet_apply_rows<T, L, 1, TK><<<b, 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, vec_ok, done); break;
    case 2: tet_apply_rows<T, L, 2, TK><<<b, 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, vec_ok, done); break;
    case 4: tet_apply_rows<T, L, 4, TK><<<b, 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, vec_ok, done); break;
    case 8: tet_apply_rows<T, L, 8, TK><<<b, 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, vec_ok, done); break;
    case 16: tet_apply_rows<T, L, 16, TK><<<b, 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, vec_ok, done); break;
    case 32: tet_apply_rows<T, L, 32, TK><<<b, 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, m, scale, x, y, vec_ok, done); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <typename T>
cudaError_t tet_apply_launch(const hcop* h, const T* K, const T* x, T* y, int nrhs, bool masked, double scale,
                             const int* done, cudaStream_t s) {
  {
    const cudaError_t prior = cudaGetLastError();  // report a failure of an earlier call
    if (prior != cudaSuccess) return prior;
  }
  if constexpr (sizeof(T) == 8) {
    int64_t blocks = (h->ne + 7) / 8;
    blocks = std::min<int64_t>(blocks, 152 * 16);
    if (h->p == 1)
      tet_apply_lanes64<6><<<(unsigned)blocks, 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, masked ? 1 : 0, nrhs,
                                                            scale, x, y, done);
    else
      tet_apply_lanes64<20><<<(unsigned)blocks, 256, 0, s>>>(h->ne, h->tet_edofs, K, h->ess, masked ? 1 : 0, nrhs,
                                                             scale, x, y, done);
    return cudaGetLastError();
  } else {
    if (h->p == 1) return tet_rows_launch<T, 6, T>(h, K, x, y, nrhs, masked, (T)scale, done, s);
    if (tet_tiles20_launch<float>(h, K, x, y, nrhs, masked, (float)scale, done, s)) return cudaGetLastError();
    return tet_rows_launch<T, 20, T>(h, K, x, y, nrhs, masked, (T)scale, done, s);
  }
}
template cudaError_t tet_apply_launch<double>(const hcop*, const double*, const double*, double*, int, bool, double,
                                              const int*, cudaStream_t);
template cudaError_t tet_apply_launch<float>(const hcop*, const float*, const float*, float*, int, bool, double,
                                             const int*, cudaStream_t);

// FP32 vectors with BF16 element matrices (FP32 accumulation)
cudaError_t tet_apply_launch_bf16(const hcop* h, const float* x, float* y, int nrhs, bool masked, cudaStream_t s) {
  const __nv_bfloat16* K = static_cast<const __nv_bfloat16*>(h->tetK16);
  if (h->p == 1) return tet_rows_launch<float, 6, __nv_bfloat16>(h, K, x, y, nrhs, masked, 1.0f, nullptr, s);
  if (tet_mma16_launch(h, K, x, y, nrhs, masked, 1.0f, nullptr, s)) return cudaGetLastError();
  if (tet_tiles20_launch<__nv_bfloat16>(h, K, x, y, nrhs, masked, 1.0f, nullptr, s)) return cudaGetLastError();
  return tet_rows_launch<float, 20, __nv_bfloat16>(h, K, x, y, nrhs, masked, 1.0f, nullptr, s);
}

__global__ void k_to_bf16(int64_t n, const double* __restrict__ a, __nv_bfloat16* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __double2bfloat16(a[i]);
}
// BF16 copy of the element matrices, made on first use (rounded from FP64)
cudaError_t tet_ensure_bf16(hcop* h) {
  if (h->tetK16) return cudaSuccess;
  const int L = h->p == 1 ? 6 : 20;
  const int64_t n = h->ne * L * L;
  cudaError_t e = dmalloc(h, &h->tetK16, (size_t)n * sizeof(__nv_bfloat16));
  if (e != cudaSuccess) return e;
  k_to_bf16<<<2048, 256, 0, h->stream>>>(n, h->tetK64, static_cast<__nv_bfloat16*>(h->tetK16));
  return cudaGetLastError();
}

template <int L>
__global__ void tet_diag_kernel(int64_t ne, const int32_t* __restrict__ edofs, const double* __restrict__ K,
                                double* __restrict__ d) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  for (int i = 0; i < L; ++i) atomicAdd(d + edofs[e * L + i], K[(e * L + i) * L + i]);
}

cudaError_t tet_setup_device(hcop* h, const hc_problem_desc* desc, const std::vector<int32_t>& edofs,
                             const std::vector<int32_t>& sv) {
  const int L = h->p == 1 ? 6 : 20;
  const int64_t ne = h->ne;
  double* V = nullptr;
  int32_t* dsv = nullptr;
  double *dnu = nullptr, *dsig = nullptr;
  int* bad = nullptr;
  cudaStream_t cs = h->stream;
  cudaError_t e = dmalloc(h, (void**)&h->tet_edofs, edofs.size() * sizeof(int32_t));
  if (e == cudaSuccess) e = dmalloc(h, (void**)&h->tetK64, (size_t)ne * L * L * sizeof(double));
  if (e == cudaSuccess) e = dmalloc(h, (void**)&h->tetK32, (size_t)ne * L * L * sizeof(float));
  if (e == cudaSuccess) e = dmalloc(h, (void**)&V, desc->n_vert * 3 * sizeof(double));
  if (e == cudaSuccess) e = dmalloc(h, (void**)&dsv, sv.size() * sizeof(int32_t));
  if (e == cudaSuccess) e = dmalloc(h, (void**)&dnu, ne * sizeof(double));
  if (e == cudaSuccess && desc->sigma) e = dmalloc(h, (void**)&dsig, ne * sizeof(double));
  if (e == cudaSuccess) e = dmalloc(h, (void**)&bad, sizeof(int));
  if (e == cudaSuccess) {
    cudaMemcpyAsync(h->tet_edofs, edofs.data(), edofs.size() * sizeof(int32_t), cudaMemcpyHostToDevice, cs);
    cudaMemcpyAsync(V, desc->vertices, desc->n_vert * 3 * sizeof(double), cudaMemcpyHostToDevice, cs);
    cudaMemcpyAsync(dsv, sv.data(), sv.size() * sizeof(int32_t), cudaMemcpyHostToDevice, cs);
    cudaMemcpyAsync(dnu, desc->nu, ne * sizeof(double), cudaMemcpyHostToDevice, cs);
    if (dsig) cudaMemcpyAsync(dsig, desc->sigma, ne * sizeof(double), cudaMemcpyHostToDevice, cs);
    cudaMemsetAsync(bad, 0, sizeof(int), cs);
    tet_elem_matrix_kernel<<<(unsigned)((ne + 127) / 128), 128, 0, cs>>>(ne, h->p, V, dsv, dnu, dsig, h->dt,
                                                                         h->tetK64, h->tetK32, bad);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
    if (e != cudaSuccess) {
      h->err = std::string("tet element-matrix kernel: ") + cudaGetErrorString(e);
    } else {
      cudaMemsetAsync(h->diag, 0, h->ndof * sizeof(double), cs);
      if (L == 6)
        tet_diag_kernel<6><<<(unsigned)((ne + 127) / 128), 128, 0, cs>>>(ne, h->tet_edofs, h->tetK64, h->diag);
      else
        tet_diag_kernel<20><<<(unsigned)((ne + 127) / 128), 128, 0, cs>>>(ne, h->tet_edofs, h->tetK64, h->diag);
      e = cudaGetLastError();
      if (e == cudaSuccess) e = cudaStreamSynchronize(cs);
      if (e != cudaSuccess) h->err = std::string("tet diagonal kernel: ") + cudaGetErrorString(e);
      int hb = 0;
      cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, cs);
      cudaStreamSynchronize(cs);
      if (e == cudaSuccess && hb) e = cudaErrorInvalidValue;
    }
  }
  cudaStreamSynchronize(cs);
  // vertices and sorted element vertices stay resident (load vectors)
  h->verts = V;
  h->tet_sv = dsv;
  dfree(h, dnu);
  dfree(h, dsig);
  dfree(h, bad);
  return e;
}

// ---- coil load b_i = (J, W_i) -------------------------------------------------------
// Collapsed (Duffy) Gauss-Legendre rule with q^3 points per tet: lambda_1 = u,
// lambda_2 = v (1 - u), lambda_3 = t (1 - u)(1 - v), weight w_u w_v w_t (1 - u)^2 (1 - v)
// (weights sum to 1/6), times |det J|.  One thread per element; the element
// vector is scattered with atomic adds.
struct TetQuad {
  int q;
  double x[8], w[8];
  double coil[7];  // I0, xc, yc, r0, r1, z0, z1
};

template <int L>
__global__ void __launch_bounds__(128) tet_load_coil_kernel(int64_t ne, int p, const double* __restrict__ V,
                                                            const int32_t* __restrict__ sv,
                                                            const int32_t* __restrict__ edofs, TetQuad Q,
                                                            double* __restrict__ b) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double vx[4][3];
  for (int k = 0; k < 4; ++k)
    for (int r = 0; r < 3; ++r) vx[k][r] = V[3 * (int64_t)sv[4 * e + k] + r];
  double J[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) J[3 * r + c] = vx[c + 1][r] - vx[0][r];
  const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
  double gl[4][3];
  gl[1][0] = (J[4] * J[8] - J[5] * J[7]) / det;
  gl[1][1] = (J[2] * J[7] - J[1] * J[8]) / det;
  gl[1][2] = (J[1] * J[5] - J[2] * J[4]) / det;
  gl[2][0] = (J[5] * J[6] - J[3] * J[8]) / det;
  gl[2][1] = (J[0] * J[8] - J[2] * J[6]) / det;
  gl[2][2] = (J[2] * J[3] - J[0] * J[5]) / det;
  gl[3][0] = (J[3] * J[7] - J[4] * J[6]) / det;
  gl[3][1] = (J[1] * J[6] - J[0] * J[7]) / det;
  gl[3][2] = (J[0] * J[4] - J[1] * J[3]) / det;
  for (int r = 0; r < 3; ++r) gl[0][r] = -(gl[1][r] + gl[2][r] + gl[3][r]);
  const double adet = fabs(det);
  const double I0 = Q.coil[0], xc = Q.coil[1], yc = Q.coil[2], r0 = Q.coil[3], r1 = Q.coil[4], z0 = Q.coil[5],
               z1 = Q.coil[6];
  double be[L];
#pragma unroll
  for (int i = 0; i < L; ++i) be[i] = 0.0;
  for (int ia = 0; ia < Q.q; ++ia)
    for (int ib = 0; ib < Q.q; ++ib)
      for (int ic = 0; ic < Q.q; ++ic) {
        const double u = Q.x[ia], v = Q.x[ib], t = Q.x[ic];
        double lam[4];
        lam[1] = u;
        lam[2] = v * (1 - u);
        lam[3] = t * (1 - u) * (1 - v);
        lam[0] = 1.0 - lam[1] - lam[2] - lam[3];
        double x[3];
        for (int r = 0; r < 3; ++r)
          x[r] = vx[0][r] + lam[1] * (vx[1][r] - vx[0][r]) + lam[2] * (vx[2][r] - vx[0][r]) +
                 lam[3] * (vx[3][r] - vx[0][r]);
        const double dx = x[0] - xc, dy = x[1] - yc;
        const double rr = sqrt(dx * dx + dy * dy);
        if (!(rr >= r0 && rr <= r1 && x[2] >= z0 && x[2] <= z1)) continue;
        const double wq = Q.w[ia] * Q.w[ib] * Q.w[ic] * (1 - u) * (1 - u) * (1 - v) * adet;
        const double f0 = -I0 * dy * wq, f1 = I0 * dx * wq;
#pragma unroll
        for (int I = 0; I < L; ++I) {
          VTerm vt[2];
          CTerm ct[3];
          int nv, nc;
          basis_terms(p, I, vt, &nv, ct, &nc);
          double acc = 0.0;
          for (int k = 0; k < nv; ++k) {
            const double m = vt[k].c * (vt[k].l0 >= 0 ? lam[vt[k].l0] : 1.0) * lam[vt[k].l1];
            acc += m * (f0 * gl[vt[k].g][0] + f1 * gl[vt[k].g][1]);
          }
          be[I] += acc;
        }
      }
#pragma unroll
  for (int i = 0; i < L; ++i)
    if (be[i] != 0.0) atomicAdd(b + edofs[e * L + i], be[i]);
}

// ---- fields on tets: quadrature points, (J, w_i), (nu curl A, w_i), curl at points ------
// Geometry of tet e on its sorted vertices: corner, gradients of the
// barycentrics, |det J|.
struct TetGeom {
  double v[4][3];
  double gl[4][3];
  double adet;
};
__device__ __forceinline__ void tet_geom(const double* __restrict__ V, const int32_t* __restrict__ sv, int64_t e,
                                         TetGeom& g) {
  for (int k = 0; k < 4; ++k)
    for (int r = 0; r < 3; ++r) g.v[k][r] = V[3 * (int64_t)sv[4 * e + k] + r];
  double J[9];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) J[3 * r + c] = g.v[c + 1][r] - g.v[0][r];
  const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
  g.gl[1][0] = (J[4] * J[8] - J[5] * J[7]) / det;
  g.gl[1][1] = (J[2] * J[7] - J[1] * J[8]) / det;
  g.gl[1][2] = (J[1] * J[5] - J[2] * J[4]) / det;
  g.gl[2][0] = (J[5] * J[6] - J[3] * J[8]) / det;
  g.gl[2][1] = (J[0] * J[8] - J[2] * J[6]) / det;
  g.gl[2][2] = (J[2] * J[3] - J[0] * J[5]) / det;
  g.gl[3][0] = (J[3] * J[7] - J[4] * J[6]) / det;
  g.gl[3][1] = (J[1] * J[6] - J[0] * J[7]) / det;
  g.gl[3][2] = (J[0] * J[4] - J[1] * J[3]) / det;
  for (int r = 0; r < 3; ++r) g.gl[0][r] = -(g.gl[1][r] + g.gl[2][r] + g.gl[3][r]);
  g.adet = fabs(det);
}
// physical value (val) and curl (cur) of basis function I at barycentrics lam
__device__ __forceinline__ void tet_basis_eval(int p, int I, const TetGeom& g, const double lam[4], double val[3],
                                               double cur[3]) {
  VTerm vt[2];
  CTerm ct[3];
  int nv, nc;
  basis_terms(p, I, vt, &nv, ct, &nc);
  for (int r = 0; r < 3; ++r) val[r] = cur[r] = 0.0;
  for (int k = 0; k < nv; ++k) {
    const double m = vt[k].c * (vt[k].l0 >= 0 ? lam[vt[k].l0] : 1.0) * lam[vt[k].l1];
    for (int r = 0; r < 3; ++r) val[r] += m * g.gl[vt[k].g][r];
  }
  for (int k = 0; k < nc; ++k) {
    const double m = ct[k].c * (ct[k].l >= 0 ? lam[ct[k].l] : 1.0);
    const double* a = g.gl[ct[k].u];
    const double* b = g.gl[ct[k].v];
    cur[0] += m * (a[1] * b[2] - a[2] * b[1]);
    cur[1] += m * (a[2] * b[0] - a[0] * b[2]);
    cur[2] += m * (a[0] * b[1] - a[1] * b[0]);
  }
}
__device__ __forceinline__ void duffy_lam(double u, double v, double t, double lam[4]) {
  lam[1] = u;
  lam[2] = v * (1 - u);
  lam[3] = t * (1 - u) * (1 - v);
  lam[0] = 1.0 - lam[1] - lam[2] - lam[3];
}

__global__ void tet_quad_points_kernel(int64_t ne, const double* __restrict__ V, const int32_t* __restrict__ sv,
                                       TetQuad Q, double* __restrict__ xyz) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  TetGeom g;
  tet_geom(V, sv, e, g);
  const int q = Q.q, q3 = q * q * q;
  for (int ia = 0; ia < q; ++ia)
    for (int ib = 0; ib < q; ++ib)
      for (int ic = 0; ic < q; ++ic) {
        double lam[4];
        duffy_lam(Q.x[ia], Q.x[ib], Q.x[ic], lam);
        double* out = xyz + 3 * (e * q3 + ic + q * (ib + q * ia));
        for (int r = 0; r < 3; ++r)
          out[r] = lam[0] * g.v[0][r] + lam[1] * g.v[1][r] + lam[2] * g.v[2][r] + lam[3] * g.v[3][r];
      }
}

// mode 0: b = (J, w_i), J per element (per_point = 0) or per point; mode 1:
// b = (nu curl A, w_i)
template <int L>
__global__ void __launch_bounds__(128) tet_field_load_kernel(int64_t ne, int p, const double* __restrict__ V,
                                                             const int32_t* __restrict__ sv,
                                                             const int32_t* __restrict__ edofs, TetQuad Q, int mode,
                                                             int per_point, const double* __restrict__ src,
                                                             const double* __restrict__ nu, double* __restrict__ b) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  TetGeom g;
  tet_geom(V, sv, e, g);
  double ae[L];
  if (mode == 1) {
    for (int i = 0; i < L; ++i) ae[i] = src[edofs[e * L + i]];
  }
  double be[L];
#pragma unroll
  for (int i = 0; i < L; ++i) be[i] = 0.0;
  const int q = Q.q, q3 = q * q * q;
  for (int ia = 0; ia < q; ++ia)
    for (int ib = 0; ib < q; ++ib)
      for (int ic = 0; ic < q; ++ic) {
        const double u = Q.x[ia], v = Q.x[ib];
        double lam[4];
        duffy_lam(u, v, Q.x[ic], lam);
        const double wq = Q.w[ia] * Q.w[ib] * Q.w[ic] * (1 - u) * (1 - u) * (1 - v) * g.adet;
        double f[3];
        if (mode == 0) {
          const double* jc = per_point ? src + 3 * (e * q3 + ic + q * (ib + q * ia)) : src + 3 * e;
          for (int r = 0; r < 3; ++r) f[r] = wq * jc[r];
        } else {
          double cu[3] = {0.0, 0.0, 0.0};
          for (int I = 0; I < L; ++I) {
            double vv[3], cc[3];
            tet_basis_eval(p, I, g, lam, vv, cc);
            for (int r = 0; r < 3; ++r) cu[r] += ae[I] * cc[r];
          }
          const double s = wq * nu[e];
          for (int r = 0; r < 3; ++r) f[r] = s * cu[r];
        }
        for (int I = 0; I < L; ++I) {
          double vv[3], cc[3];
          tet_basis_eval(p, I, g, lam, vv, cc);
          be[I] += f[0] * vv[0] + f[1] * vv[1] + f[2] * vv[2];
        }
      }
#pragma unroll
  for (int i = 0; i < L; ++i)
    if (be[i] != 0.0) atomicAdd(b + edofs[e * L + i], be[i]);
}

struct TetPoints {
  int n;
  double xi[16][3];
};
template <int L>
__global__ void tet_curl_points_kernel(int64_t ne, int p, const double* __restrict__ V, const int32_t* __restrict__ sv,
                                       const int32_t* __restrict__ edofs, TetPoints P, const double* __restrict__ A,
                                       double* __restrict__ B) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  TetGeom g;
  tet_geom(V, sv, e, g);
  double ae[L];
  for (int i = 0; i < L; ++i) ae[i] = A[edofs[e * L + i]];
  for (int k = 0; k < P.n; ++k) {
    const double lam[4] = {1.0 - P.xi[k][0] - P.xi[k][1] - P.xi[k][2], P.xi[k][0], P.xi[k][1], P.xi[k][2]};
    double cu[3] = {0.0, 0.0, 0.0};
    for (int I = 0; I < L; ++I) {
      double vv[3], cc[3];
      tet_basis_eval(p, I, g, lam, vv, cc);
      for (int r = 0; r < 3; ++r) cu[r] += ae[I] * cc[r];
    }
    for (int r = 0; r < 3; ++r) B[3 * (e * P.n + k) + r] = cu[r];
  }
}

static TetQuad make_tet_quad(int q, const double* xq, const double* wq) {
  TetQuad Q;
  std::memset(&Q, 0, sizeof(Q));
  Q.q = q;
  for (int k = 0; k < 8; ++k) {
    Q.x[k] = k < q ? xq[k] : 0.0;
    Q.w[k] = (k < q && wq) ? wq[k] : 0.0;
  }
  return Q;
}

cudaError_t tet_quad_points(const hcop* h, int q, const double* xq, double* xyz, cudaStream_t s) {
  if (!h->verts || !h->tet_sv || q < 1 || q > 8) return cudaErrorInvalidValue;
  const TetQuad Q = make_tet_quad(q, xq, nullptr);
  tet_quad_points_kernel<<<(unsigned)((h->ne + 127) / 128), 128, 0, s>>>(h->ne, h->verts, h->tet_sv, Q, xyz);
  return cudaGetLastError();
}

static cudaError_t tet_field_launch(const hcop* h, int mode, int per_point, const double* src, int q,
                                    const double* xq, const double* wq, double* b, cudaStream_t s) {
  if (!h->verts || !h->tet_sv || q < 1 || q > 8) return cudaErrorInvalidValue;
  const TetQuad Q = make_tet_quad(q, xq, wq);
  cudaError_t e = cudaMemsetAsync(b, 0, h->ndof * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((h->ne + 127) / 128);
  if (h->p == 1)
    tet_field_load_kernel<6><<<blocks, 128, 0, s>>>(h->ne, 1, h->verts, h->tet_sv, h->tet_edofs, Q, mode, per_point,
                                                    src, h->nu, b);
  else
    tet_field_load_kernel<20><<<blocks, 128, 0, s>>>(h->ne, 2, h->verts, h->tet_sv, h->tet_edofs, Q, mode, per_point,
                                                     src, h->nu, b);
  return cudaGetLastError();
}

cudaError_t tet_load_field(const hcop* h, int per_point, const double* src, int q, const double* xq,
                           const double* wq, double* b, cudaStream_t s) {
  return tet_field_launch(h, 0, per_point, src, q, xq, wq, b, s);
}

cudaError_t tet_curl_load(const hcop* h, const double* A, int q, const double* xq, const double* wq, double* b,
                          cudaStream_t s) {
  if (!h->nu) return cudaErrorInvalidValue;
  return tet_field_launch(h, 1, 0, A, q, xq, wq, b, s);
}

cudaError_t tet_curl_points(const hcop* h, const double* A, int npts, const double* xi, double* B, cudaStream_t s) {
  if (!h->verts || !h->tet_sv || npts < 1 || npts > 16) return cudaErrorInvalidValue;
  TetPoints P;
  std::memset(&P, 0, sizeof(P));
  P.n = npts;
  for (int k = 0; k < npts; ++k)
    for (int r = 0; r < 3; ++r) P.xi[k][r] = xi[3 * k + r];
  const unsigned blocks = (unsigned)((h->ne + 127) / 128);
  if (h->p == 1)
    tet_curl_points_kernel<6><<<blocks, 128, 0, s>>>(h->ne, 1, h->verts, h->tet_sv, h->tet_edofs, P, A, B);
  else
    tet_curl_points_kernel<20><<<blocks, 128, 0, s>>>(h->ne, 2, h->verts, h->tet_sv, h->tet_edofs, P, A, B);
  return cudaGetLastError();
}

cudaError_t tet_load_coil(const hcop* h, const double coil[7], int q, const double* xq, const double* wq, double* b,
                          cudaStream_t s) {
  if (!h->verts || !h->tet_sv || q < 1 || q > 8) return cudaErrorInvalidValue;
  TetQuad Q;
  Q.q = q;
  for (int k = 0; k < 8; ++k) {
    Q.x[k] = k < q ? xq[k] : 0.0;
    Q.w[k] = k < q ? wq[k] : 0.0;
  }
  for (int k = 0; k < 7; ++k) Q.coil[k] = coil[k];
  cudaError_t e = cudaMemsetAsync(b, 0, h->ndof * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((h->ne + 127) / 128);
  if (h->p == 1)
    tet_load_coil_kernel<6><<<blocks, 128, 0, s>>>(h->ne, 1, h->verts, h->tet_sv, h->tet_edofs, Q, b);
  else
    tet_load_coil_kernel<20><<<blocks, 128, 0, s>>>(h->ne, 2, h->verts, h->tet_sv, h->tet_edofs, Q, b);
  return cudaGetLastError();
}

}  // namespace hc

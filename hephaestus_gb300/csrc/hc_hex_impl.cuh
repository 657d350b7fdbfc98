// hc_hex.cu -- sum-factorised partial-assembly apply of the Nedelec hex operator.
//
// Element operator (reference element [0,1]^3, affine map x = x0 + J xi):
//
//   K_e = sum_{c,b} Mfac_cb (M^x_cb (x) M^y_cb (x) M^z_cb)            mass
//       + Curl^T [ sum_{c,b} Cfac_cb (R^x_cb (x) R^y_cb (x) R^z_cb) ] Curl  curl-curl
//
// where Mfac = sigma |det J| J^-1 J^-T, Cfac = dt nu / |det J| J^T J (the
// covariant Piola map of the values and the contravariant map of the curls),
// the 1-D factors are the closed/open mass matrices picked by component and
// direction, and Curl is the exact element-local discrete curl from the
// Nedelec into the Raviart-Thomas tensor space (one 1-D derivative matrix D
// per term).  No quadrature-point data is stored: for affine elements with
// element-constant coefficients this is the exact Galerkin operator of
// MFEM's CurlCurlIntegrator + VectorFEMassIntegrator
// (src/kernels/curl_curl_kernel.cpp:21-24, vector_fe_mass_kernel.cpp:21-24).
//
// Axis-aligned grids (all off-diagonal factors zero) use the 3 diagonal blocks
// only; general parallelepipeds use all 9.
//
// Work mapping: one thread per element, the element's dofs in registers,
// fully unrolled compile-time 1-D contractions, implicit structured
// element->dof map (no index array), atomic scatter into y.
#pragma once
#include <cstdio>

#include "hc_internal.h"
#include "hc_reduce.cuh"

namespace hc {

// Each translation unit holds its own copy of the 1-D tables (no relocatable
// device code); upload_tables() fills every copy.
static __constant__ Tab1D<double> c_tabd[kMaxP + 1];
static __constant__ Tab1D<float> c_tabf[kMaxP + 1];

static inline cudaError_t upload_tables_here(const void* td, const void* tf) {
  cudaError_t e = cudaMemcpyToSymbol(c_tabd, td, sizeof(c_tabd));
  if (e != cudaSuccess) return e;
  return cudaMemcpyToSymbol(c_tabf, tf, sizeof(c_tabf));
}

template <typename T>
struct TabSel;
template <>
struct TabSel<double> {
  __device__ static const Tab1D<double>& get(int p) { return c_tabd[p]; }
};
template <>
struct TabSel<float> {
  __device__ static const Tab1D<float>& get(int p) { return c_tabf[p]; }
};

enum { kC = 0, kO = 1 };  // closed / open 1-D basis
template <int P>
__host__ __device__ constexpr int nb(int t) {
  return t == kC ? P + 1 : P;
}

// 1-D matrix entry between basis types R (row) and Cc (column)
template <typename T, int P, int R, int Cc>
__device__ __forceinline__ T m1(int i, int j) {
  const Tab1D<T>& t = TabSel<T>::get(P);
  if constexpr (R == kC && Cc == kC) return t.Mcc[i][j];
  else if constexpr (R == kC && Cc == kO) return t.Mco[i][j];
  else if constexpr (R == kO && Cc == kC) return t.Mco[j][i];
  else return t.Moo[i][j];
}
template <typename T, int P>
__device__ __forceinline__ T dm(int a, int j) {
  return TabSel<T>::get(P).D[a][j];
}

// out(n0,n1,n2) += s * (A (x) B (x) Cz) in(m0,m1,m2), index i + n0 (j + n1 k)
template <typename T, int P, int RX, int CX, int RY, int CY, int RZ, int CZ>
__device__ __forceinline__ void kron3_acc(const T* in, T* out, T s) {
  constexpr int m0 = nb<P>(CX), m1n = nb<P>(CY), m2 = nb<P>(CZ);
  constexpr int n0 = nb<P>(RX), n1 = nb<P>(RY), n2 = nb<P>(RZ);
  T t1[m0 * m1n * n2];
#pragma unroll
  for (int k = 0; k < n2; ++k)
#pragma unroll
    for (int j0 = 0; j0 < m1n; ++j0)
#pragma unroll
      for (int i0 = 0; i0 < m0; ++i0) {
        T acc = T(0);
#pragma unroll
        for (int k0 = 0; k0 < m2; ++k0) acc += m1<T, P, RZ, CZ>(k, k0) * in[i0 + m0 * (j0 + m1n * k0)];
        t1[i0 + m0 * (j0 + m1n * k)] = acc;
      }
  T t2[m0 * n1 * n2];
#pragma unroll
  for (int k = 0; k < n2; ++k)
#pragma unroll
    for (int j = 0; j < n1; ++j)
#pragma unroll
      for (int i0 = 0; i0 < m0; ++i0) {
        T acc = T(0);
#pragma unroll
        for (int j0 = 0; j0 < m1n; ++j0) acc += m1<T, P, RY, CY>(j, j0) * t1[i0 + m0 * (j0 + m1n * k)];
        t2[i0 + m0 * (j + n1 * k)] = acc;
      }
#pragma unroll
  for (int k = 0; k < n2; ++k)
#pragma unroll
    for (int j = 0; j < n1; ++j)
#pragma unroll
      for (int i = 0; i < n0; ++i) {
        T acc = T(0);
#pragma unroll
        for (int i0 = 0; i0 < m0; ++i0) acc += m1<T, P, RX, CX>(i, i0) * t2[i0 + m0 * (j + n1 * k)];
        out[i + n0 * (j + n1 * k)] += s * acc;
      }
}

// Nedelec component c: open in direction c, closed elsewhere.
template <int c, int d>
struct NdT {
  static constexpr int v = (c == d) ? kO : kC;
};
// Raviart-Thomas component c: closed in direction c, open elsewhere.
template <int c, int d>
struct RtT {
  static constexpr int v = (c == d) ? kC : kO;
};

template <typename T, int P, int c, int b>
__device__ __forceinline__ void mass_block(const T* u, T* y, T s) {
  kron3_acc<T, P, NdT<c, 0>::v, NdT<b, 0>::v, NdT<c, 1>::v, NdT<b, 1>::v, NdT<c, 2>::v, NdT<b, 2>::v>(
      u, y, s);
}
template <typename T, int P, int c, int b>
__device__ __forceinline__ void rt_block(const T* u, T* y, T s) {
  kron3_acc<T, P, RtT<c, 0>::v, RtT<b, 0>::v, RtT<c, 1>::v, RtT<b, 1>::v, RtT<c, 2>::v, RtT<b, 2>::v>(
      u, y, s);
}

// Exact element-local curl: Nedelec (u0,u1,u2) -> Raviart-Thomas (r0,r1,r2).
//   r0 = D_y u2 - D_z u1,  r1 = D_z u0 - D_x u2,  r2 = D_x u1 - D_y u0
template <typename T, int P>
__device__ __forceinline__ void curl_nd(const T* u0, const T* u1, const T* u2, T* r0, T* r1, T* r2) {
  constexpr int C = P + 1, O = P;
  // r0 dims (C,O,O); u2 dims (C,C,O); u1 dims (C,O,C)
#pragma unroll
  for (int k = 0; k < O; ++k)
#pragma unroll
    for (int j = 0; j < O; ++j)
#pragma unroll
      for (int i = 0; i < C; ++i) {
        T acc = T(0);
#pragma unroll
        for (int q = 0; q < C; ++q) acc += dm<T, P>(j, q) * u2[i + C * (q + C * k)];
#pragma unroll
        for (int q = 0; q < C; ++q) acc -= dm<T, P>(k, q) * u1[i + C * (j + O * q)];
        r0[i + C * (j + O * k)] = acc;
      }
  // r1 dims (O,C,O); u0 dims (O,C,C); u2 dims (C,C,O)
#pragma unroll
  for (int k = 0; k < O; ++k)
#pragma unroll
    for (int j = 0; j < C; ++j)
#pragma unroll
      for (int i = 0; i < O; ++i) {
        T acc = T(0);
#pragma unroll
        for (int q = 0; q < C; ++q) acc += dm<T, P>(k, q) * u0[i + O * (j + C * q)];
#pragma unroll
        for (int q = 0; q < C; ++q) acc -= dm<T, P>(i, q) * u2[q + C * (j + C * k)];
        r1[i + O * (j + C * k)] = acc;
      }
  // r2 dims (O,O,C); u1 dims (C,O,C); u0 dims (O,C,C)
#pragma unroll
  for (int k = 0; k < C; ++k)
#pragma unroll
    for (int j = 0; j < O; ++j)
#pragma unroll
      for (int i = 0; i < O; ++i) {
        T acc = T(0);
#pragma unroll
        for (int q = 0; q < C; ++q) acc += dm<T, P>(i, q) * u1[q + C * (j + O * k)];
#pragma unroll
        for (int q = 0; q < C; ++q) acc -= dm<T, P>(j, q) * u0[i + O * (q + C * k)];
        r2[i + O * (j + O * k)] = acc;
      }
}

// Transpose of curl_nd, accumulated: y0 += D_z^T g1 - D_y^T g2,
// y1 += D_x^T g2 - D_z^T g0, y2 += D_y^T g0 - D_x^T g1.
template <typename T, int P>
__device__ __forceinline__ void curl_nd_t(const T* g0, const T* g1, const T* g2, T* y0, T* y1, T* y2) {
  constexpr int C = P + 1, O = P;
  // y0 dims (O,C,C); g1 (O,C,O); g2 (O,O,C)
#pragma unroll
  for (int k = 0; k < C; ++k)
#pragma unroll
    for (int j = 0; j < C; ++j)
#pragma unroll
      for (int i = 0; i < O; ++i) {
        T acc = T(0);
#pragma unroll
        for (int q = 0; q < O; ++q) acc += dm<T, P>(q, k) * g1[i + O * (j + C * q)];
#pragma unroll
        for (int q = 0; q < O; ++q) acc -= dm<T, P>(q, j) * g2[i + O * (q + O * k)];
        y0[i + O * (j + C * k)] += acc;
      }
  // y1 dims (C,O,C); g2 (O,O,C); g0 (C,O,O)
#pragma unroll
  for (int k = 0; k < C; ++k)
#pragma unroll
    for (int j = 0; j < O; ++j)
#pragma unroll
      for (int i = 0; i < C; ++i) {
        T acc = T(0);
#pragma unroll
        for (int q = 0; q < O; ++q) acc += dm<T, P>(q, i) * g2[q + O * (j + O * k)];
#pragma unroll
        for (int q = 0; q < O; ++q) acc -= dm<T, P>(q, k) * g0[i + C * (j + O * q)];
        y1[i + C * (j + O * k)] += acc;
      }
  // y2 dims (C,C,O); g0 (C,O,O); g1 (O,C,O)
#pragma unroll
  for (int k = 0; k < O; ++k)
#pragma unroll
    for (int j = 0; j < C; ++j)
#pragma unroll
      for (int i = 0; i < C; ++i) {
        T acc = T(0);
#pragma unroll
        for (int q = 0; q < O; ++q) acc += dm<T, P>(q, j) * g0[i + C * (q + O * k)];
#pragma unroll
        for (int q = 0; q < O; ++q) acc -= dm<T, P>(q, i) * g1[q + O * (j + C * k)];
        y2[i + C * (j + C * k)] += acc;
      }
}

// Global index of local dof (a,b,c) of component `comp` of element (ex,ey,ez).
template <int P, int comp>
__device__ __forceinline__ int64_t gdof(const HexDev& d, int ex, int ey, int ez, int a, int b, int c) {
  const int64_t nxo = (int64_t)d.nx * P, nyo = (int64_t)d.ny * P;
  const int64_t i = (int64_t)ex * P + a, j = (int64_t)ey * P + b, k = (int64_t)ez * P + c;
  if constexpr (comp == 0) return d.off[0] + i + nxo * (j + (nyo + 1) * k);
  else if constexpr (comp == 1) return d.off[1] + i + (nxo + 1) * (j + nyo * k);
  else return d.off[2] + i + (nxo + 1) * (j + (nyo + 1) * k);
}
// Tangential-face test (implicit essential mask) for dof (comp, i, j, k).
template <int P, int comp>
__device__ __forceinline__ bool face_ess(const HexDev& d, int ex, int ey, int ez, int a, int b, int c) {
  const int bits = d.ess_bits;
  const int i = ex * P + a, j = ey * P + b, k = ez * P + c;
  const int mx = d.nx * P, my = d.ny * P, mz = d.nz * P;
  bool e = false;
  if (comp != 0) e |= (i == 0 && (bits & 1)) || (i == mx && (bits & 2));
  if (comp != 1) e |= (j == 0 && (bits & 4)) || (j == my && (bits & 8));
  if (comp != 2) e |= (k == 0 && (bits & 16)) || (k == mz && (bits & 32));
  return e;
}
template <int P, int comp>
__device__ __forceinline__ bool is_ess(const HexDev& d, int64_t g, int ex, int ey, int ez, int a, int b,
                                       int c) {
  if (d.ess) return d.ess[g] != 0;
  return face_ess<P, comp>(d, ex, ey, ez, a, b, c);
}

template <typename T, int P, int comp>
__device__ __forceinline__ void gather(const HexDev& d, const T* __restrict__ x, int ex, int ey, int ez,
                                       bool masked, T* u) {
  constexpr int C = P + 1, O = P;
  constexpr int n0 = comp == 0 ? O : C, n1 = comp == 1 ? O : C, n2 = comp == 2 ? O : C;
#pragma unroll
  for (int c = 0; c < n2; ++c)
#pragma unroll
    for (int b = 0; b < n1; ++b)
#pragma unroll
      for (int a = 0; a < n0; ++a) {
        const int64_t g = gdof<P, comp>(d, ex, ey, ez, a, b, c);
        T v = __ldg(x + g);
        if (masked && is_ess<P, comp>(d, g, ex, ey, ez, a, b, c)) v = T(0);
        u[a + n0 * (b + n1 * c)] = v;
      }
}

template <typename T, int P, int comp>
__device__ __forceinline__ void scatter(const HexDev& d, T* __restrict__ y, int ex, int ey, int ez,
                                        bool masked, const T* v) {
  constexpr int C = P + 1, O = P;
  constexpr int n0 = comp == 0 ? O : C, n1 = comp == 1 ? O : C, n2 = comp == 2 ? O : C;
#pragma unroll
  for (int c = 0; c < n2; ++c)
#pragma unroll
    for (int b = 0; b < n1; ++b)
#pragma unroll
      for (int a = 0; a < n0; ++a) {
        const int64_t g = gdof<P, comp>(d, ex, ey, ez, a, b, c);
        if (masked && is_ess<P, comp>(d, g, ex, ey, ez, a, b, c)) continue;
        atomicAdd(y + g, v[a + n0 * (b + n1 * c)]);
      }
}

__device__ __forceinline__ int symk(int a, int b) {
  // packed symmetric (00,01,02,11,12,22)
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return lo == 0 ? hi : (lo == 1 ? 2 + hi : 5);
}

template <typename T, int P, bool FULL>
__global__ void __launch_bounds__(128) hex_apply_kernel(HexDev d, const T* __restrict__ fac,
                                                        const T* __restrict__ x, T* __restrict__ y,
                                                        T mscale, T cscale, int masked,
                                                        KrylovScalars* S, double* partials) {
  // S != nullptr: PCG mode.  Skip when the solve has stopped; accumulate the
  // element energies p_e.K_e p_e onto S->pq (which holds sum_ess p_i^2) and
  // form alpha = rz / pq on the last block.
  if (S && S->done) return;
  const bool want_energy = (S != nullptr);
  constexpr int C = P + 1, O = P;
  constexpr int NDC = O * C * C;  // dofs per component
  constexpr int RTC = C * O * O;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double en = 0.0;
  (void)partials;
  if (e < d.ne) {
    const int ex = (int)(e % d.nx);
    const int ey = (int)((e / d.nx) % d.ny);
    const int ez = (int)(e / ((int64_t)d.nx * d.ny));
    const bool mk = masked != 0;
    T u0[NDC], u1[NDC], u2[NDC];
    gather<T, P, 0>(d, x, ex, ey, ez, mk, u0);
    gather<T, P, 1>(d, x, ex, ey, ez, mk, u1);
    gather<T, P, 2>(d, x, ex, ey, ez, mk, u2);
    T fm[6], fc[6];
    if constexpr (FULL) {
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        fm[k] = mscale * __ldg(fac + (int64_t)k * d.ne + e);
        fc[k] = cscale * __ldg(fac + (int64_t)(6 + k) * d.ne + e);
      }
    } else {
      // axis aligned: only the diagonal tensor entries are read
      constexpr int kd[3] = {0, 3, 5};
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        fm[kd[q]] = mscale * __ldg(fac + (int64_t)kd[q] * d.ne + e);
        fc[kd[q]] = cscale * __ldg(fac + (int64_t)(6 + kd[q]) * d.ne + e);
      }
    }
    T r0[RTC], r1[RTC], r2[RTC];
    curl_nd<T, P>(u0, u1, u2, r0, r1, r2);
    T y0[NDC], y1[NDC], y2[NDC];
#pragma unroll
    for (int i = 0; i < NDC; ++i) y0[i] = y1[i] = y2[i] = T(0);
    if (mscale != T(0)) {
      mass_block<T, P, 0, 0>(u0, y0, fm[0]);
      mass_block<T, P, 1, 1>(u1, y1, fm[3]);
      mass_block<T, P, 2, 2>(u2, y2, fm[5]);
      if constexpr (FULL) {
        mass_block<T, P, 0, 1>(u1, y0, fm[1]);
        mass_block<T, P, 0, 2>(u2, y0, fm[2]);
        mass_block<T, P, 1, 0>(u0, y1, fm[1]);
        mass_block<T, P, 1, 2>(u2, y1, fm[4]);
        mass_block<T, P, 2, 0>(u0, y2, fm[2]);
        mass_block<T, P, 2, 1>(u1, y2, fm[4]);
      }
    }
    T eacc = T(0);
    if (want_energy) {
#pragma unroll
      for (int i = 0; i < NDC; ++i) eacc += u0[i] * y0[i] + u1[i] * y1[i] + u2[i] * y2[i];
    }
    T g0[RTC], g1[RTC], g2[RTC];
#pragma unroll
    for (int i = 0; i < RTC; ++i) g0[i] = g1[i] = g2[i] = T(0);
    rt_block<T, P, 0, 0>(r0, g0, fc[0]);
    rt_block<T, P, 1, 1>(r1, g1, fc[3]);
    rt_block<T, P, 2, 2>(r2, g2, fc[5]);
    if constexpr (FULL) {
      rt_block<T, P, 0, 1>(r1, g0, fc[1]);
      rt_block<T, P, 0, 2>(r2, g0, fc[2]);
      rt_block<T, P, 1, 0>(r0, g1, fc[1]);
      rt_block<T, P, 1, 2>(r2, g1, fc[4]);
      rt_block<T, P, 2, 0>(r0, g2, fc[2]);
      rt_block<T, P, 2, 1>(r1, g2, fc[4]);
    }
    if (want_energy) {
#pragma unroll
      for (int i = 0; i < RTC; ++i) eacc += r0[i] * g0[i] + r1[i] * g1[i] + r2[i] * g2[i];
      en = (double)eacc;
    }
    curl_nd_t<T, P>(g0, g1, g2, y0, y1, y2);
    scatter<T, P, 0>(d, y, ex, ey, ez, mk, y0);
    scatter<T, P, 1>(d, y, ex, ey, ez, mk, y1);
    scatter<T, P, 2>(d, y, ex, ey, ez, mk, y2);
  }
  if (want_energy) {
    double v[1] = {en}, tot[1];
    block_sum_n<1>(v);
    if (grid_sum_n<1>(v, partials, &S->counter[0], tot)) {
      const double pq = S->pq + tot[0];
      S->pq = pq;
      if (!(pq > 0.0) || !isfinite(pq)) {
        S->done = 1;
        S->status = HC_BREAKDOWN;
        S->alpha = 0.0;
      } else {
        S->alpha = S->rz / pq;
      }
    }
  }
}

template <typename T, int P>
cudaError_t hex_launch_p(const HexDev& d, const T* fac, const T* x, T* y, T ms, T cs, bool masked,
                         KrylovScalars* S, double* partials, cudaStream_t s) {
  const int blocks = (int)((d.ne + 127) / 128);
  if (d.full)
    hex_apply_kernel<T, P, true><<<blocks, 128, 0, s>>>(d, fac, x, y, ms, cs, masked, S, partials);
  else
    hex_apply_kernel<T, P, false><<<blocks, 128, 0, s>>>(d, fac, x, y, ms, cs, masked, S, partials);
  return cudaGetLastError();
}

}  // namespace hc

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
#include <algorithm>
#include <cstdio>
#include <vector>

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

// out(n0,n1,n2) (+)= s * (A (x) B (x) Cz) in(m0,m1,m2), index i + n0 (j + n1 k);
// ACC = false assigns (first contribution), avoiding additions of zero.
template <typename T, int P, int RX, int CX, int RY, int CY, int RZ, int CZ, bool ACC = true>
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
        T acc = m1<T, P, RZ, CZ>(k, 0) * in[i0 + m0 * j0];
#pragma unroll
        for (int k0 = 1; k0 < m2; ++k0) acc += m1<T, P, RZ, CZ>(k, k0) * in[i0 + m0 * (j0 + m1n * k0)];
        t1[i0 + m0 * (j0 + m1n * k)] = acc;
      }
  T t2[m0 * n1 * n2];
#pragma unroll
  for (int k = 0; k < n2; ++k)
#pragma unroll
    for (int j = 0; j < n1; ++j)
#pragma unroll
      for (int i0 = 0; i0 < m0; ++i0) {
        T acc = m1<T, P, RY, CY>(j, 0) * t1[i0 + m0 * (m1n * k)];
#pragma unroll
        for (int j0 = 1; j0 < m1n; ++j0) acc += m1<T, P, RY, CY>(j, j0) * t1[i0 + m0 * (j0 + m1n * k)];
        t2[i0 + m0 * (j + n1 * k)] = acc;
      }
#pragma unroll
  for (int k = 0; k < n2; ++k)
#pragma unroll
    for (int j = 0; j < n1; ++j)
#pragma unroll
      for (int i = 0; i < n0; ++i) {
        T acc = m1<T, P, RX, CX>(i, 0) * t2[m0 * (j + n1 * k)];
#pragma unroll
        for (int i0 = 1; i0 < m0; ++i0) acc += m1<T, P, RX, CX>(i, i0) * t2[i0 + m0 * (j + n1 * k)];
        if constexpr (ACC) out[i + n0 * (j + n1 * k)] += s * acc;
        else out[i + n0 * (j + n1 * k)] = s * acc;
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

template <typename T, int P, int c, int b, bool ACC = true>
__device__ __forceinline__ void mass_block(const T* u, T* y, T s) {
  kron3_acc<T, P, NdT<c, 0>::v, NdT<b, 0>::v, NdT<c, 1>::v, NdT<b, 1>::v, NdT<c, 2>::v, NdT<b, 2>::v, ACC>(
      u, y, s);
}
template <typename T, int P, int c, int b, bool ACC = true>
__device__ __forceinline__ void rt_block(const T* u, T* y, T s) {
  kron3_acc<T, P, RtT<c, 0>::v, RtT<b, 0>::v, RtT<c, 1>::v, RtT<b, 1>::v, RtT<c, 2>::v, RtT<b, 2>::v, ACC>(
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
        T acc = dm<T, P>(j, 0) * u2[i + C * (C * k)];
#pragma unroll
        for (int q = 1; q < C; ++q) acc += dm<T, P>(j, q) * u2[i + C * (q + C * k)];
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
        T acc = dm<T, P>(k, 0) * u0[i + O * j];
#pragma unroll
        for (int q = 1; q < C; ++q) acc += dm<T, P>(k, q) * u0[i + O * (j + C * q)];
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
        T acc = dm<T, P>(i, 0) * u1[C * (j + O * k)];
#pragma unroll
        for (int q = 1; q < C; ++q) acc += dm<T, P>(i, q) * u1[q + C * (j + O * k)];
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
        T acc = dm<T, P>(0, k) * g1[i + O * j];
#pragma unroll
        for (int q = 1; q < O; ++q) acc += dm<T, P>(q, k) * g1[i + O * (j + C * q)];
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
        T acc = dm<T, P>(0, i) * g2[O * (j + O * k)];
#pragma unroll
        for (int q = 1; q < O; ++q) acc += dm<T, P>(q, i) * g2[q + O * (j + O * k)];
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
        T acc = dm<T, P>(0, j) * g0[i + C * (O * k)];
#pragma unroll
        for (int q = 1; q < O; ++q) acc += dm<T, P>(q, j) * g0[i + C * (q + O * k)];
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
__global__ void __launch_bounds__(128, 1) hex_apply_kernel(HexDev d, const T* __restrict__ fac,
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
    T y0[NDC], y1[NDC], y2[NDC];
    T eacc = T(0);
    const bool curl = cscale != T(0);  // 0: the mass-only launches of the order-3 complex apply
    if constexpr (!FULL) {
      // axis-aligned: the blocks are diagonal; the curl is taken first, then
      // each u_c dies with its own mass block and each r_c with its own
      // curl-curl block, which keeps the live set small (the order-3
      // element carries 144 dofs)
      T r0[RTC], r1[RTC], r2[RTC];
      if (curl) curl_nd<T, P>(u0, u1, u2, r0, r1, r2);
      auto mass_c = [&](auto cc, const T* u, T* yv) {
        constexpr int c = decltype(cc)::value;
        if (mscale == T(0)) {
#pragma unroll
          for (int i = 0; i < NDC; ++i) yv[i] = T(0);
        } else {
          mass_block<T, P, c, c, false>(u, yv, fm[c == 0 ? 0 : (c == 1 ? 3 : 5)]);
        }
        if (want_energy) {
#pragma unroll
          for (int i = 0; i < NDC; ++i) eacc += u[i] * yv[i];
        }
      };
      mass_c(std::integral_constant<int, 2>{}, u2, y2);
      mass_c(std::integral_constant<int, 1>{}, u1, y1);
      mass_c(std::integral_constant<int, 0>{}, u0, y0);
      if (curl) {
        T g0[RTC], g1[RTC], g2[RTC];
        auto rt_c = [&](auto cc, const T* r, T* gv) {
          constexpr int c = decltype(cc)::value;
          rt_block<T, P, c, c, false>(r, gv, fc[c == 0 ? 0 : (c == 1 ? 3 : 5)]);
          if (want_energy) {
#pragma unroll
            for (int i = 0; i < RTC; ++i) eacc += r[i] * gv[i];
          }
        };
        rt_c(std::integral_constant<int, 0>{}, r0, g0);
        rt_c(std::integral_constant<int, 1>{}, r1, g1);
        rt_c(std::integral_constant<int, 2>{}, r2, g2);
        curl_nd_t<T, P>(g0, g1, g2, y0, y1, y2);
      }
    } else {
#pragma unroll
      for (int i = 0; i < NDC; ++i) y0[i] = y1[i] = y2[i] = T(0);
      if (mscale != T(0)) {
        mass_block<T, P, 0, 0>(u0, y0, fm[0]);
        mass_block<T, P, 1, 1>(u1, y1, fm[3]);
        mass_block<T, P, 2, 2>(u2, y2, fm[5]);
        mass_block<T, P, 0, 1>(u1, y0, fm[1]);
        mass_block<T, P, 0, 2>(u2, y0, fm[2]);
        mass_block<T, P, 1, 0>(u0, y1, fm[1]);
        mass_block<T, P, 1, 2>(u2, y1, fm[4]);
        mass_block<T, P, 2, 0>(u0, y2, fm[2]);
        mass_block<T, P, 2, 1>(u1, y2, fm[4]);
      }
      if (want_energy) {
#pragma unroll
        for (int i = 0; i < NDC; ++i) eacc += u0[i] * y0[i] + u1[i] * y1[i] + u2[i] * y2[i];
      }
      if (curl) {
        T r0[RTC], r1[RTC], r2[RTC];
        curl_nd<T, P>(u0, u1, u2, r0, r1, r2);
        T g0[RTC], g1[RTC], g2[RTC];
#pragma unroll
        for (int i = 0; i < RTC; ++i) g0[i] = g1[i] = g2[i] = T(0);
        rt_block<T, P, 0, 0>(r0, g0, fc[0]);
        rt_block<T, P, 1, 1>(r1, g1, fc[3]);
        rt_block<T, P, 2, 2>(r2, g2, fc[5]);
        rt_block<T, P, 0, 1>(r1, g0, fc[1]);
        rt_block<T, P, 0, 2>(r2, g0, fc[2]);
        rt_block<T, P, 1, 0>(r0, g1, fc[1]);
        rt_block<T, P, 1, 2>(r2, g1, fc[4]);
        rt_block<T, P, 2, 0>(r0, g2, fc[2]);
        rt_block<T, P, 2, 1>(r1, g2, fc[4]);
        if (want_energy) {
#pragma unroll
          for (int i = 0; i < RTC; ++i) eacc += r0[i] * g0[i] + r1[i] * g1[i] + r2[i] * g2[i];
        }
        curl_nd_t<T, P>(g0, g1, g2, y0, y1, y2);
      }
    }
    if (want_energy) en = (double)eacc;
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

// y += cscale C xc + mscale M xm on axis-aligned grids, thread per element,
// essential rows and columns masked: one launch per output of the order-3
// complex apply (y_r = C x_r - w M x_i, y_i = C x_i + w M x_r) instead of two.
// The curl-curl part runs first (its inputs die before the mass inputs are
// gathered), then the mass input one component at a time.
template <typename T, int P>
__global__ void __launch_bounds__(128, 1) hex_apply_pair_kernel(HexDev d, const T* __restrict__ fac,
                                                             const T* __restrict__ xc, const T* __restrict__ xm,
                                                             T* __restrict__ y, T mscale, T cscale) {
  constexpr int C = P + 1, O = P;
  constexpr int NDC = O * C * C;
  constexpr int RTC = C * O * O;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  const int ex = (int)(e % d.nx);
  const int ey = (int)((e / d.nx) % d.ny);
  const int ez = (int)(e / ((int64_t)d.nx * d.ny));
  constexpr int kd[3] = {0, 3, 5};
  T fm[3], fc[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    fm[q] = mscale * __ldg(fac + (int64_t)kd[q] * d.ne + e);
    fc[q] = cscale * __ldg(fac + (int64_t)(6 + kd[q]) * d.ne + e);
  }
  T y0[NDC], y1[NDC], y2[NDC];
#pragma unroll
  for (int i = 0; i < NDC; ++i) y0[i] = y1[i] = y2[i] = T(0);
  {
    T r0[RTC], r1[RTC], r2[RTC];
    {
      T u0[NDC], u1[NDC], u2[NDC];
      gather<T, P, 0>(d, xc, ex, ey, ez, true, u0);
      gather<T, P, 1>(d, xc, ex, ey, ez, true, u1);
      gather<T, P, 2>(d, xc, ex, ey, ez, true, u2);
      curl_nd<T, P>(u0, u1, u2, r0, r1, r2);
    }
    T g0[RTC], g1[RTC], g2[RTC];
    rt_block<T, P, 0, 0, false>(r0, g0, fc[0]);
    rt_block<T, P, 1, 1, false>(r1, g1, fc[1]);
    rt_block<T, P, 2, 2, false>(r2, g2, fc[2]);
    curl_nd_t<T, P>(g0, g1, g2, y0, y1, y2);
  }
  {
    T v[NDC];
    gather<T, P, 0>(d, xm, ex, ey, ez, true, v);
    mass_block<T, P, 0, 0>(v, y0, fm[0]);
  }
  {
    T v[NDC];
    gather<T, P, 1>(d, xm, ex, ey, ez, true, v);
    mass_block<T, P, 1, 1>(v, y1, fm[1]);
  }
  {
    T v[NDC];
    gather<T, P, 2>(d, xm, ex, ey, ez, true, v);
    mass_block<T, P, 2, 2>(v, y2, fm[2]);
  }
  scatter<T, P, 0>(d, y, ex, ey, ez, true, y0);
  scatter<T, P, 1>(d, y, ex, ey, ez, true, y1);
  scatter<T, P, 2>(d, y, ex, ey, ez, true, y2);
}

template <typename T, int P>
cudaError_t hex_launch_pair(const HexDev& d, const T* fac, const T* xc, const T* xm, T* y, T ms, T cs,
                            cudaStream_t s) {
  if (d.full) return cudaErrorInvalidValue;  // axis-aligned grids only
  const int blocks = (int)((d.ne + 127) / 128);
  hex_apply_pair_kernel<T, P><<<blocks, 128, 0, s>>>(d, fac, xc, xm, y, ms, cs);
  return cudaGetLastError();
}
// instantiated in hc_hex_p3.cu
extern template cudaError_t hex_launch_pair<double, 3>(const HexDev&, const double*, const double*, const double*,
                                                       double*, double, double, cudaStream_t);
extern template cudaError_t hex_launch_pair<float, 3>(const HexDev&, const float*, const float*, const float*,
                                                      float*, float, float, cudaStream_t);

// ---------------------------------------------------------------------------
// Brick-tiled apply: one CTA per brick of BX x BY x BZ elements, one thread per
// element.  The brick's dofs (both closed boundary planes included) are
// staged in shared memory by coalesced cooperative loads; each thread runs the
// register-resident element operator on its element, accumulating into a
// shared output tile (shared-memory atomics, at most 4 writers per dof); the
// tile is then flushed with one coalesced global reduction per dof, so a
// dof on a brick face receives one atomic per adjacent brick instead of one
// per adjacent element.
// ---------------------------------------------------------------------------
template <int P, int BX, int BY, int BZ>
struct BrickTile {
  static constexpr int tx(int c) { return BX * P + (c != 0); }
  static constexpr int ty(int c) { return BY * P + (c != 1); }
  static constexpr int tz(int c) { return BZ * P + (c != 2); }
  static constexpr int n(int c) { return tx(c) * ty(c) * tz(c); }
  static constexpr int off(int c) { return c == 0 ? 0 : (c == 1 ? n(0) : n(0) + n(1)); }
  static constexpr int total = n(0) + n(1) + n(2);
};

template <int P, int comp>
__device__ __forceinline__ int64_t gdof_ijk(const HexDev& d, int64_t i, int64_t j, int64_t k) {
  const int64_t nxo = (int64_t)d.nx * P, nyo = (int64_t)d.ny * P;
  if constexpr (comp == 0) return d.off[0] + i + nxo * (j + (nyo + 1) * k);
  else if constexpr (comp == 1) return d.off[1] + i + (nxo + 1) * (j + nyo * k);
  else return d.off[2] + i + (nxo + 1) * (j + (nyo + 1) * k);
}
template <int P, int comp>
__device__ __forceinline__ bool ess_ijk(const HexDev& d, int64_t g, int i, int j, int k) {
  if (d.ess) return d.ess[g] != 0;
  const int bits = d.ess_bits;
  const int mx = d.nx * P, my = d.ny * P, mz = d.nz * P;
  bool e = false;
  if (comp != 0) e |= (i == 0 && (bits & 1)) || (i == mx && (bits & 2));
  if (comp != 1) e |= (j == 0 && (bits & 4)) || (j == my && (bits & 8));
  if (comp != 2) e |= (k == 0 && (bits & 16)) || (k == mz && (bits & 32));
  return e;
}

// Visit the tile entries of component comp owned by thread t in a
// block-strided loop: f(tile_index, global_dof, i, j, k) for entries inside the grid.
template <int P, int BX, int BY, int BZ, int comp, typename F>
__device__ __forceinline__ void tile_loop(const HexDev& d, int X0, int Y0, int Z0, F&& f) {
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int TX = TL::tx(comp), TY = TL::ty(comp), NC = TL::n(comp), OFF = TL::off(comp);
  const int gdx = d.nx * P + (comp != 0), gdy = d.ny * P + (comp != 1), gdz = d.nz * P + (comp != 2);
  for (int r = threadIdx.x; r < NC; r += BX * BY * BZ) {
    const int ti = r % TX, tj = (r / TX) % TY, tk = r / (TX * TY);
    const int i = X0 * P + ti, j = Y0 * P + tj, k = Z0 * P + tk;
    if (i < gdx && j < gdy && k < gdz) f(OFF + r, gdof_ijk<P, comp>(d, i, j, k), i, j, k);
  }
}

template <typename T, int P, int BX, int BY, int BZ, int comp>
__device__ __forceinline__ void sgather(const T* sx, int lx, int ly, int lz, T* u) {
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int C = P + 1, O = P;
  constexpr int n0 = comp == 0 ? O : C, n1 = comp == 1 ? O : C, n2 = comp == 2 ? O : C;
  constexpr int TX = TL::tx(comp), TY = TL::ty(comp), OFF = TL::off(comp);
#pragma unroll
  for (int c = 0; c < n2; ++c)
#pragma unroll
    for (int b = 0; b < n1; ++b)
#pragma unroll
      for (int a = 0; a < n0; ++a)
        u[a + n0 * (b + n1 * c)] = sx[OFF + (lx * P + a) + TX * ((ly * P + b) + TY * (lz * P + c))];
}
template <typename T, int P, int BX, int BY, int BZ, int comp>
__device__ __forceinline__ void sscatter(T* sy, int lx, int ly, int lz, const T* v) {
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int C = P + 1, O = P;
  constexpr int n0 = comp == 0 ? O : C, n1 = comp == 1 ? O : C, n2 = comp == 2 ? O : C;
  constexpr int TX = TL::tx(comp), TY = TL::ty(comp), OFF = TL::off(comp);
#pragma unroll
  for (int c = 0; c < n2; ++c)
#pragma unroll
    for (int b = 0; b < n1; ++b)
#pragma unroll
      for (int a = 0; a < n0; ++a)
        atomicAdd(&sy[OFF + (lx * P + a) + TX * ((ly * P + b) + TY * (lz * P + c))], v[a + n0 * (b + n1 * c)]);
}

// cp.async (4-byte, zero-fill when src_bytes == 0): asynchronous global ->
// shared copies that do not occupy registers, so a whole brick is in flight.
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, int src_bytes) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(sa), "l"(gmem), "r"(src_bytes));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

struct BrickGeom {
  int X0, Y0, Z0;
};
template <int BX, int BY, int BZ>
__device__ __forceinline__ BrickGeom brick_of(const HexDev& d, int b) {
  const int nbx = (d.nx + BX - 1) / BX, nby = (d.ny + BY - 1) / BY;
  BrickGeom g;
  g.X0 = (b % nbx) * BX;
  g.Y0 = ((b / nbx) % nby) * BY;
  g.Z0 = (b / (nbx * nby)) * BZ;
  return g;
}

// Issue the asynchronous copies of one brick's dofs (all three components)
// into sx; entries outside the grid are zero-filled.
template <typename T, int P, int BX, int BY, int BZ, int comp>
__device__ __forceinline__ void prefetch_comp(const HexDev& d, const T* __restrict__ x, T* sx, BrickGeom bg) {
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int TX = TL::tx(comp), TY = TL::ty(comp), TZ = TL::tz(comp), NC = TL::n(comp), OFF = TL::off(comp);
  const int gdx = d.nx * P + (comp != 0), gdy = d.ny * P + (comp != 1), gdz = d.nz * P + (comp != 2);
  const int base = (int)d.off[comp] + bg.X0 * P + gdx * (bg.Y0 * P + gdy * (bg.Z0 * P));
  const bool full = bg.X0 + BX <= d.nx && bg.Y0 + BY <= d.ny && bg.Z0 + BZ <= d.nz;
  if (full) {
    // rows of the tile along x: one warp per row, lane = x index; the
    // (TX - 32) trailing entries of each row are spread one row per thread.
    constexpr int NW = BX * BY * BZ / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tx0 = lane < TX ? lane : 0;
#pragma unroll 2
    for (int row = warp; row < TY * TZ; row += NW) {
      const int tj = row % TY, tk = row / TY;
      const int g = base + gdx * (tj + gdy * tk);
      if (lane < TX) {
        if constexpr (sizeof(T) == 4) cp_async4(sx + OFF + TX * row + tx0, x + g + tx0, 4);
        else cp_async8(sx + OFF + TX * row + tx0, x + g + tx0, 8);
      }
    }
    if constexpr (TX > 32) {
      for (int row = threadIdx.x; row < TY * TZ; row += BX * BY * BZ) {
        const int tj = row % TY, tk = row / TY;
        const int g = base + gdx * (tj + gdy * tk);
#pragma unroll
        for (int ti = 32; ti < TX; ++ti) {
          if constexpr (sizeof(T) == 4) cp_async4(sx + OFF + TX * row + ti, x + g + ti, 4);
          else cp_async8(sx + OFF + TX * row + ti, x + g + ti, 8);
        }
      }
    }
    return;
  }
#pragma unroll 4
  for (int r = threadIdx.x; r < NC; r += BX * BY * BZ) {
    const int ti = r % TX, tj = (r / TX) % TY, tk = r / (TX * TY);
    const bool in = (bg.X0 * P + ti < gdx) && (bg.Y0 * P + tj < gdy) && (bg.Z0 * P + tk < gdz);
    const T* src = in ? x + (base + ti + gdx * (tj + gdy * tk)) : x;
    if constexpr (sizeof(T) == 4) cp_async4(sx + OFF + r, src, in ? 4 : 0);
    else cp_async8(sx + OFF + r, src, in ? 8 : 0);
  }
}

// Zero one boundary plane (direction dir, low or high side) of component comp.
template <typename T, int P, int BX, int BY, int BZ, int comp, int dir>
__device__ __forceinline__ void zero_plane(T* buf, int idx) {
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int TX = TL::tx(comp), TY = TL::ty(comp), TZ = TL::tz(comp), OFF = TL::off(comp);
  constexpr int NA = dir == 0 ? TY : TX, NB = dir == 2 ? TY : TZ;
  for (int r = threadIdx.x; r < NA * NB; r += BX * BY * BZ) {
    const int a = r % NA, b = r / NA;
    int ti, tj, tk;
    if constexpr (dir == 0) { ti = idx; tj = a; tk = b; }
    else if constexpr (dir == 1) { ti = a; tj = idx; tk = b; }
    else { ti = a; tj = b; tk = idx; }
    buf[OFF + ti + TX * (tj + TY * tk)] = T(0);
  }
}
// Zero the essential entries of a staged brick from an explicit mask.
template <typename T, int P, int BX, int BY, int BZ, int comp>
__device__ __forceinline__ void mask_comp(const HexDev& d, T* sx, BrickGeom bg) {
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int TX = TL::tx(comp), TY = TL::ty(comp), NC = TL::n(comp), OFF = TL::off(comp);
  const int gdx = d.nx * P + (comp != 0), gdy = d.ny * P + (comp != 1), gdz = d.nz * P + (comp != 2);
  for (int r = threadIdx.x; r < NC; r += BX * BY * BZ) {
    const int i = bg.X0 * P + r % TX, j = bg.Y0 * P + (r / TX) % TY, k = bg.Z0 * P + r / (TX * TY);
    if (i >= gdx || j >= gdy || k >= gdz) continue;
    const int64_t g = d.off[comp] + i + (int64_t)gdx * (j + (int64_t)gdy * k);
    if (ess_ijk<P, comp>(d, g, i, j, k)) sx[OFF + r] = T(0);
  }
}

// Zero the tangential (essential) entries on the marked grid faces the brick
// touches.  The high face of the grid is at local plane (n - X0) p, which is
// the brick's last plane for full bricks and inside the tile for partial ones.
template <typename T, int P, int BX, int BY, int BZ>
__device__ __forceinline__ void zero_ess_planes(const HexDev& d, T* buf, BrickGeom bg) {
  const int bits = d.ess_bits;
  if (bg.X0 == 0 && (bits & 1)) {
    zero_plane<T, P, BX, BY, BZ, 1, 0>(buf, 0);
    zero_plane<T, P, BX, BY, BZ, 2, 0>(buf, 0);
  }
  if (bg.X0 + BX >= d.nx && (bits & 2)) {
    const int hi = (d.nx - bg.X0) * P;
    zero_plane<T, P, BX, BY, BZ, 1, 0>(buf, hi);
    zero_plane<T, P, BX, BY, BZ, 2, 0>(buf, hi);
  }
  if (bg.Y0 == 0 && (bits & 4)) {
    zero_plane<T, P, BX, BY, BZ, 0, 1>(buf, 0);
    zero_plane<T, P, BX, BY, BZ, 2, 1>(buf, 0);
  }
  if (bg.Y0 + BY >= d.ny && (bits & 8)) {
    const int hi = (d.ny - bg.Y0) * P;
    zero_plane<T, P, BX, BY, BZ, 0, 1>(buf, hi);
    zero_plane<T, P, BX, BY, BZ, 2, 1>(buf, hi);
  }
  if (bg.Z0 == 0 && (bits & 16)) {
    zero_plane<T, P, BX, BY, BZ, 0, 2>(buf, 0);
    zero_plane<T, P, BX, BY, BZ, 1, 2>(buf, 0);
  }
  if (bg.Z0 + BZ >= d.nz && (bits & 32)) {
    const int hi = (d.nz - bg.Z0) * P;
    zero_plane<T, P, BX, BY, BZ, 0, 2>(buf, hi);
    zero_plane<T, P, BX, BY, BZ, 1, 2>(buf, hi);
  }
}

// Flush one component of the output tile.  Entries on a brick face are shared
// with a neighbouring brick and go out as atomic adds; brick-interior entries
// are written with plain stores when y is known to be zero at free dofs
// (OVERWRITE), else added atomically.  Essential rows are skipped when masked.
// fast: full brick and (if masked) face-attribute masking already applied by
// zeroing the essential planes of sy -- every essential dof lies on a brick
// face, so it only ever receives an atomic add of zero.
template <typename T, int P, int BX, int BY, int BZ, int comp, bool OVERWRITE>
__device__ __forceinline__ void flush_comp(const HexDev& d, T* __restrict__ y, T* sy, BrickGeom bg, bool mk,
                                           bool fast) {
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int TX = TL::tx(comp), TY = TL::ty(comp), TZ = TL::tz(comp), NC = TL::n(comp), OFF = TL::off(comp);
  const int gdx = d.nx * P + (comp != 0), gdy = d.ny * P + (comp != 1), gdz = d.nz * P + (comp != 2);
  const int base = (int)d.off[comp] + bg.X0 * P + gdx * (bg.Y0 * P + gdy * (bg.Z0 * P));
  if (fast) {
    constexpr int NW = BX * BY * BZ / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll 2
    for (int row = warp; row < TY * TZ; row += NW) {
      const int tj = row % TY, tk = row / TY;
      const bool rowface = (comp != 1 && (tj == 0 || tj == TY - 1)) || (comp != 2 && (tk == 0 || tk == TZ - 1));
      if (lane < TX) {
        T* src = sy + OFF + TX * row + lane;
        const T v = *src;
        *src = T(0);
        T* dst = y + base + gdx * (tj + gdy * tk) + lane;
        const bool face = rowface || (comp != 0 && (lane == 0 || lane == TX - 1));
        if (OVERWRITE && !face) *dst = v;
        else atomicAdd(dst, v);
      }
    }
    if constexpr (TX > 32) {
      for (int row = threadIdx.x; row < TY * TZ; row += BX * BY * BZ) {
        const int tj = row % TY, tk = row / TY;
#pragma unroll
        for (int ti = 32; ti < TX; ++ti) {
          T* src = sy + OFF + TX * row + ti;
          const T v = *src;
          *src = T(0);
          atomicAdd(y + base + gdx * (tj + gdy * tk) + ti, v);  // last x plane: always a face
        }
      }
    }
    return;
  }
#pragma unroll 2
  for (int r = threadIdx.x; r < NC; r += BX * BY * BZ) {
    const int ti = r % TX, tj = (r / TX) % TY, tk = r / (TX * TY);
    const int i = bg.X0 * P + ti, j = bg.Y0 * P + tj, k = bg.Z0 * P + tk;
    const T v = sy[OFF + r];
    sy[OFF + r] = T(0);
    if (i >= gdx || j >= gdy || k >= gdz) continue;
    const int g = base + ti + gdx * (tj + gdy * tk);
    if (mk && ess_ijk<P, comp>(d, g, i, j, k)) continue;
    // a closed-direction index on the brick's first or last plane is shared
    const bool face = (comp != 0 && (ti == 0 || ti == TX - 1)) || (comp != 1 && (tj == 0 || tj == TY - 1)) ||
                      (comp != 2 && (tk == 0 || tk == TZ - 1));
    if (OVERWRITE && !face) y[g] = v;
    else atomicAdd(y + g, v);
  }
}

template <typename T, int P, bool FULL, int BX, int BY, int BZ, bool OVERWRITE>
__global__ void __launch_bounds__(BX* BY* BZ, sizeof(T) == 4 ? (FULL ? 3 : 4) : 2)
    hex_apply_tiled(HexDev d, const T* __restrict__ fac, const T* __restrict__ x, T* __restrict__ y, T mscale,
                    T cscale, int masked, KrylovScalars* S, double* partials, int nbricks) {
  if (S && S->done) return;
  using TL = BrickTile<P, BX, BY, BZ>;
  constexpr int NT = BX * BY * BZ;
  constexpr int NF = FULL ? 12 : 6;  // factors staged per element
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* sxb[2] = {reinterpret_cast<T*>(smem_raw), reinterpret_cast<T*>(smem_raw) + TL::total};
  T* sy = reinterpret_cast<T*>(smem_raw) + 2 * TL::total;
  T* sfb[2] = {sy + TL::total, sy + TL::total + NF * NT};
  const bool mk = masked != 0;
  const bool mask_needed = mk && (d.ess != nullptr || d.ess_bits != 0);
  constexpr int C = P + 1, O = P;
  constexpr int NDC = O * C * C;
  constexpr int RTC = C * O * O;
  const int lx = threadIdx.x % BX, ly = (threadIdx.x / BX) % BY, lz = threadIdx.x / (BX * BY);
  for (int r = threadIdx.x; r < TL::total; r += BX * BY * BZ) sy[r] = T(0);
  double en = 0.0;
  int b = blockIdx.x;
  // each thread stages its own element's factors (SoA rows are coalesced)
  auto prefetch_fac = [&](BrickGeom g, T* sf) {
    const int ex = g.X0 + lx, ey = g.Y0 + ly, ez = g.Z0 + lz;
    const bool in = ex < d.nx && ey < d.ny && ez < d.nz;
    const int64_t e = in ? ex + (int64_t)d.nx * (ey + (int64_t)d.ny * ez) : 0;
#pragma unroll
    for (int q = 0; q < NF; ++q) {
      const int k = FULL ? q : (q < 3 ? (q == 0 ? 0 : (q == 1 ? 3 : 5)) : (q == 3 ? 6 : (q == 4 ? 9 : 11)));
      if constexpr (sizeof(T) == 4) cp_async4(sf + q * NT + threadIdx.x, fac + (int64_t)k * d.ne + e, in ? 4 : 0);
      else cp_async8(sf + q * NT + threadIdx.x, fac + (int64_t)k * d.ne + e, in ? 8 : 0);
    }
  };
  if (b < nbricks) {
    const BrickGeom g0 = brick_of<BX, BY, BZ>(d, b);
    prefetch_comp<T, P, BX, BY, BZ, 0>(d, x, sxb[0], g0);
    prefetch_comp<T, P, BX, BY, BZ, 1>(d, x, sxb[0], g0);
    prefetch_comp<T, P, BX, BY, BZ, 2>(d, x, sxb[0], g0);
    prefetch_fac(g0, sfb[0]);
  }
  cp_async_commit();
  for (int it = 0; b < nbricks; b += gridDim.x, ++it) {
    T* sx = sxb[it & 1];
    const BrickGeom bg = brick_of<BX, BY, BZ>(d, b);
    const int bn = b + gridDim.x;
    if (bn < nbricks) {  // prefetch the next brick into the other buffer
      const BrickGeom gn = brick_of<BX, BY, BZ>(d, bn);
      T* sn = sxb[(it + 1) & 1];
      prefetch_comp<T, P, BX, BY, BZ, 0>(d, x, sn, gn);
      prefetch_comp<T, P, BX, BY, BZ, 1>(d, x, sn, gn);
      prefetch_comp<T, P, BX, BY, BZ, 2>(d, x, sn, gn);
      prefetch_fac(gn, sfb[(it + 1) & 1]);
    }
    cp_async_commit();
    cp_async_wait<1>();  // this brick's group has landed
    __syncthreads();
    const bool full = bg.X0 + BX <= d.nx && bg.Y0 + BY <= d.ny && bg.Z0 + BZ <= d.nz;
    const bool touches = bg.X0 == 0 || bg.Y0 == 0 || bg.Z0 == 0 || bg.X0 + BX >= d.nx || bg.Y0 + BY >= d.ny ||
                         bg.Z0 + BZ >= d.nz;
    const bool fast = full && d.ess == nullptr;
    if (mask_needed && (d.ess != nullptr || touches)) {
      if (d.ess != nullptr) {
        mask_comp<T, P, BX, BY, BZ, 0>(d, sx, bg);
        mask_comp<T, P, BX, BY, BZ, 1>(d, sx, bg);
        mask_comp<T, P, BX, BY, BZ, 2>(d, sx, bg);
      } else {
        zero_ess_planes<T, P, BX, BY, BZ>(d, sx, bg);
      }
      __syncthreads();
    }
    const int ex = bg.X0 + lx, ey = bg.Y0 + ly, ez = bg.Z0 + lz;
    if (ex < d.nx && ey < d.ny && ez < d.nz) {
      const T* sf = sfb[it & 1];
      T u0[NDC], u1[NDC], u2[NDC];
      sgather<T, P, BX, BY, BZ, 0>(sx, lx, ly, lz, u0);
      sgather<T, P, BX, BY, BZ, 1>(sx, lx, ly, lz, u1);
      sgather<T, P, BX, BY, BZ, 2>(sx, lx, ly, lz, u2);
      T fm[6], fc[6];
      if constexpr (FULL) {
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          fm[k] = mscale * sf[k * NT + threadIdx.x];
          fc[k] = cscale * sf[(6 + k) * NT + threadIdx.x];
        }
      } else {
        constexpr int kd[3] = {0, 3, 5};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
          fm[kd[q]] = mscale * sf[q * NT + threadIdx.x];
          fc[kd[q]] = cscale * sf[(3 + q) * NT + threadIdx.x];
        }
      }
      T r0[RTC], r1[RTC], r2[RTC];
      curl_nd<T, P>(u0, u1, u2, r0, r1, r2);
      T y0[NDC], y1[NDC], y2[NDC];
      T g0[RTC], g1[RTC], g2[RTC];
      T eacc = T(0);
      if constexpr (!FULL) {
        // axis-aligned: the blocks are diagonal, so each u_c and r_c is last
        // used by its own mass block -- computed one component at a time they
        // die early, which keeps the live set (and the register count) down
        auto mass_c = [&](auto cc, const T* u, T* yv) {
          constexpr int c = decltype(cc)::value;
          if (mscale == T(0)) {
#pragma unroll
            for (int i = 0; i < NDC; ++i) yv[i] = T(0);
          } else {
            mass_block<T, P, c, c, false>(u, yv, fm[c == 0 ? 0 : (c == 1 ? 3 : 5)]);
          }
          if (S) {
#pragma unroll
            for (int i = 0; i < NDC; ++i) eacc += u[i] * yv[i];
          }
        };
        mass_c(std::integral_constant<int, 2>{}, u2, y2);
        mass_c(std::integral_constant<int, 1>{}, u1, y1);
        mass_c(std::integral_constant<int, 0>{}, u0, y0);
        auto rt_c = [&](auto cc, const T* r, T* gv) {
          constexpr int c = decltype(cc)::value;
          rt_block<T, P, c, c, false>(r, gv, fc[c == 0 ? 0 : (c == 1 ? 3 : 5)]);
          if (S) {
#pragma unroll
            for (int i = 0; i < RTC; ++i) eacc += r[i] * gv[i];
          }
        };
        rt_c(std::integral_constant<int, 0>{}, r0, g0);
        rt_c(std::integral_constant<int, 1>{}, r1, g1);
        rt_c(std::integral_constant<int, 2>{}, r2, g2);
        if (S) en += (double)eacc;
      } else {
        if (mscale == T(0)) {
#pragma unroll
          for (int i = 0; i < NDC; ++i) y0[i] = y1[i] = y2[i] = T(0);
        } else {
          mass_block<T, P, 0, 0, false>(u0, y0, fm[0]);
          mass_block<T, P, 1, 1, false>(u1, y1, fm[3]);
          mass_block<T, P, 2, 2, false>(u2, y2, fm[5]);
          mass_block<T, P, 0, 1>(u1, y0, fm[1]);
          mass_block<T, P, 0, 2>(u2, y0, fm[2]);
          mass_block<T, P, 1, 0>(u0, y1, fm[1]);
          mass_block<T, P, 1, 2>(u2, y1, fm[4]);
          mass_block<T, P, 2, 0>(u0, y2, fm[2]);
          mass_block<T, P, 2, 1>(u1, y2, fm[4]);
        }
        if (S) {
#pragma unroll
          for (int i = 0; i < NDC; ++i) eacc += u0[i] * y0[i] + u1[i] * y1[i] + u2[i] * y2[i];
        }
        rt_block<T, P, 0, 0, false>(r0, g0, fc[0]);
        rt_block<T, P, 1, 1, false>(r1, g1, fc[3]);
        rt_block<T, P, 2, 2, false>(r2, g2, fc[5]);
        rt_block<T, P, 0, 1>(r1, g0, fc[1]);
        rt_block<T, P, 0, 2>(r2, g0, fc[2]);
        rt_block<T, P, 1, 0>(r0, g1, fc[1]);
        rt_block<T, P, 1, 2>(r2, g1, fc[4]);
        rt_block<T, P, 2, 0>(r0, g2, fc[2]);
        rt_block<T, P, 2, 1>(r1, g2, fc[4]);
        if (S) {
#pragma unroll
          for (int i = 0; i < RTC; ++i) eacc += r0[i] * g0[i] + r1[i] * g1[i] + r2[i] * g2[i];
          en += (double)eacc;
        }
      }
      curl_nd_t<T, P>(g0, g1, g2, y0, y1, y2);
      sscatter<T, P, BX, BY, BZ, 0>(sy, lx, ly, lz, y0);
      sscatter<T, P, BX, BY, BZ, 1>(sy, lx, ly, lz, y1);
      sscatter<T, P, BX, BY, BZ, 2>(sy, lx, ly, lz, y2);
    }
    __syncthreads();
    if (fast && mk && touches && d.ess_bits) {
      zero_ess_planes<T, P, BX, BY, BZ>(d, sy, bg);
      __syncthreads();
    }
    flush_comp<T, P, BX, BY, BZ, 0, OVERWRITE>(d, y, sy, bg, mk, fast);
    flush_comp<T, P, BX, BY, BZ, 1, OVERWRITE>(d, y, sy, bg, mk, fast);
    flush_comp<T, P, BX, BY, BZ, 2, OVERWRITE>(d, y, sy, bg, mk, fast);
    // the next iteration's scatter into sy and prefetch into this buffer
    // happen after every thread passed the barrier at the top of the loop
  }
  cp_async_wait<0>();
  if (S) {
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

// Brick shapes of the tiled kernels (orders 1-2): shape 0 = 16 x 4 x 2
// elements, shape 1 = 8 x 8 x 2 (fewer idle threads where nx is far from a
// multiple of 16); order 3 runs the per-element kernel.  hc_autotune times
// both per problem.
template <int P, int S>
struct BrickShapeS {
  static constexpr int BX = 16, BY = 4, BZ = 2;
};
template <int P>
struct BrickShapeS<P, 1> {
  static constexpr int BX = 8, BY = 8, BZ = 2;
};
template <>
struct BrickShapeS<3, 0> {
  static constexpr int BX = 4, BY = 4, BZ = 4;
};
template <int P>
using BrickShape = BrickShapeS<P, 0>;

// Host: per tile entry the dof offset relative to the brick's base (bit 31 set
// when the entry lies on a brick face, i.e. is shared with a neighbour brick).
template <int P, int S = 0>
inline void build_tile_table(int nx, int ny, std::vector<int>& tab) {
  using B = BrickShapeS<P, S>;
  using TL = BrickTile<P, B::BX, B::BY, B::BZ>;
  tab.assign(TL::total, 0);
  for (int c = 0; c < 3; ++c) {
    const int TX = TL::tx(c), TY = TL::ty(c), TZ = TL::tz(c);
    const int gdx = nx * P + (c != 0), gdy = ny * P + (c != 1);
    for (int r = 0; r < TL::n(c); ++r) {
      const int ti = r % TX, tj = (r / TX) % TY, tk = r / (TX * TY);
      const bool face = (c != 0 && (ti == 0 || ti == TX - 1)) || (c != 1 && (tj == 0 || tj == TY - 1)) ||
                        (c != 2 && (tk == 0 || tk == TZ - 1));
      const int rel = ti + gdx * (tj + gdy * tk);
      tab[TL::off(c) + r] = rel | (face ? (int)0x80000000u : 0);
    }
  }
}

template <int P, int S = 0>
__host__ __device__ inline int brick_blocks(const HexDev& d) {
  using B = BrickShapeS<P, S>;
  return ((d.nx + B::BX - 1) / B::BX) * ((d.ny + B::BY - 1) / B::BY) * ((d.nz + B::BZ - 1) / B::BZ);
}

// CTAs per SM of a persistent brick launch: the caller's (hc_autotune) when
// set, capped by the occupancy; else occ, or one fewer when that needs no
// more rounds over the bricks -- a last round that fills few slots costs as
// much as a full one, and one more resident CTA per SM raises the brick
// throughput by only about 10 % (measured at 64^3: 61.7 us with 3 CTAs per
// SM, 56.0 us with 4).
inline int bricks_per_sm(int occ, int nbricks, int nsm, int want) {
  if (want > 0) return std::min(want, occ);
  const auto rounds = [&](int per) { return (nbricks + per * nsm - 1) / (per * nsm); };
  if (occ > 1 && rounds(occ - 1) * (occ - 1) * 1.1 <= rounds(occ) * occ) return occ - 1;
  return occ;
}

inline int device_sms() {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  return nsm;
}

// The tiled launch for one brick shape (instantiated per order and shape in
// hc_hex_p{1,2}.cu and hc_hex_p{1,2}s.cu).
template <typename T, int P, int S>
cudaError_t hex_launch_ps(const HexDev& d, const T* fac, const T* x, T* y, T ms, T cs, bool masked,
                          KrylovScalars* S_, double* partials, cudaStream_t s, bool y_zero_free) {
  using B = BrickShapeS<P, S>;
  using TL = BrickTile<P, B::BX, B::BY, B::BZ>;
  constexpr int nt = B::BX * B::BY * B::BZ;
  const size_t sm = (3 * TL::total + 2 * (d.full ? 12 : 6) * nt) * sizeof(T);
  const int nbricks = brick_blocks<P, S>(d);
  static int per_sm[2][2][2] = {{{0, 0}, {0, 0}}, {{0, 0}, {0, 0}}};
  const int nsm = device_sms();
  auto go = [&](auto kern, int f, int o) {
    int& occ = per_sm[f][o][sizeof(T) == 8];
    if (!occ) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, nt, sm);
      if (occ < 1) occ = 1;
    }
    const int grid = std::min(nbricks, bricks_per_sm(occ, nbricks, nsm, d.per_sm) * nsm);
    kern<<<grid, nt, sm, s>>>(d, fac, x, y, ms, cs, masked, S_, partials, nbricks);
  };
  if (d.full) {
    if (y_zero_free) go(hex_apply_tiled<T, P, true, B::BX, B::BY, B::BZ, true>, 1, 1);
    else go(hex_apply_tiled<T, P, true, B::BX, B::BY, B::BZ, false>, 1, 0);
  } else {
    if (y_zero_free) go(hex_apply_tiled<T, P, false, B::BX, B::BY, B::BZ, true>, 0, 1);
    else go(hex_apply_tiled<T, P, false, B::BX, B::BY, B::BZ, false>, 0, 0);
  }
  return cudaGetLastError();
}
#define HC_EXTERN_LAUNCH_PS(T, P, S)                                                                   \
  extern template cudaError_t hex_launch_ps<T, P, S>(const HexDev&, const T*, const T*, T*, T, T, bool, \
                                                     KrylovScalars*, double*, cudaStream_t, bool);
HC_EXTERN_LAUNCH_PS(double, 1, 1)
HC_EXTERN_LAUNCH_PS(double, 2, 1)
HC_EXTERN_LAUNCH_PS(float, 1, 1)
HC_EXTERN_LAUNCH_PS(float, 2, 1)
#undef HC_EXTERN_LAUNCH_PS

template <typename T, int P>
cudaError_t hex_launch_p(const HexDev& d, const T* fac, const T* x, T* y, T ms, T cs, bool masked,
                         KrylovScalars* S, double* partials, cudaStream_t s, bool y_zero_free) {
  if constexpr (P <= 2) {
    if (d.shape == 1) return hex_launch_ps<T, P, 1>(d, fac, x, y, ms, cs, masked, S, partials, s, y_zero_free);
    return hex_launch_ps<T, P, 0>(d, fac, x, y, ms, cs, masked, S, partials, s, y_zero_free);
  } else {
    const int blocks = (int)((d.ne + 127) / 128);
    if (d.full)
      hex_apply_kernel<T, P, true><<<blocks, 128, 0, s>>>(d, fac, x, y, ms, cs, masked, S, partials);
    else
      hex_apply_kernel<T, P, false><<<blocks, 128, 0, s>>>(d, fac, x, y, ms, cs, masked, S, partials);
    return cudaGetLastError();
  }
}

}  // namespace hc

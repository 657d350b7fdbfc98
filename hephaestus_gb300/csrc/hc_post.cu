// hc_post.cu -- operators around the solve on the structured hex space:
//  * B = curl A into the Raviart-Thomas tensor space: the exact discrete curl
//    that CurlAuxSolver applies with MFEM's CurlInterpolator
//    (src/auxsolvers/curl_aux.cpp:13-30).  Component c of the RT space is
//    closed (Gauss-Lobatto) in direction c and open (Gauss-Legendre) in the
//    other two; a shared RT dof gets the identical value from both elements.
//  * the load vector b_i = (J, w_i) of a loop coil: the right-hand side that
//    DivFreeSource adds (M g with g = M^-1 (J, w), src/sources/div_free_source.cpp:72-114,
//    i.e. (J, w) up to its inner solve tolerance).
#include <cmath>
#include <cstring>
#include <vector>

#include "hc_hex_impl.cuh"

namespace hc {

cudaError_t upload_tables_post(const void* td, const void* tf) { return upload_tables_here(td, tf); }

// ---- curl ---------------------------------------------------------------------
template <int P>
__global__ void hex_curl_kernel(HexDev d, const double* __restrict__ A, double* __restrict__ B, int64_t rt_off1,
                                int64_t rt_off2) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  constexpr int C = P + 1, O = P, NDC = O * C * C, RTC = C * O * O;
  const int ex = (int)(e % d.nx), ey = (int)((e / d.nx) % d.ny), ez = (int)(e / ((int64_t)d.nx * d.ny));
  double u0[NDC], u1[NDC], u2[NDC], r0[RTC], r1[RTC], r2[RTC];
  gather<double, P, 0>(d, A, ex, ey, ez, false, u0);
  gather<double, P, 1>(d, A, ex, ey, ez, false, u1);
  gather<double, P, 2>(d, A, ex, ey, ez, false, u2);
  curl_nd<double, P>(u0, u1, u2, r0, r1, r2);
  const int64_t mx = (int64_t)d.nx * P, my = (int64_t)d.ny * P;
  // RT comp 0: (C,O,O) dims (mx+1, my, mz); comp 1: (O,C,O) (mx, my+1, mz); comp 2: (O,O,C) (mx, my, mz+1)
#pragma unroll
  for (int k = 0; k < O; ++k)
#pragma unroll
    for (int j = 0; j < O; ++j)
#pragma unroll
      for (int i = 0; i < C; ++i)
        B[(ex * P + i) + (mx + 1) * ((ey * P + j) + my * (int64_t)(ez * P + k))] = r0[i + C * (j + O * k)];
#pragma unroll
  for (int k = 0; k < O; ++k)
#pragma unroll
    for (int j = 0; j < C; ++j)
#pragma unroll
      for (int i = 0; i < O; ++i)
        B[rt_off1 + (ex * P + i) + mx * ((ey * P + j) + (my + 1) * (int64_t)(ez * P + k))] = r1[i + O * (j + C * k)];
#pragma unroll
  for (int k = 0; k < C; ++k)
#pragma unroll
    for (int j = 0; j < O; ++j)
#pragma unroll
      for (int i = 0; i < O; ++i)
        B[rt_off2 + (ex * P + i) + mx * ((ey * P + j) + my * (int64_t)(ez * P + k))] = r2[i + O * (j + O * k)];
}

void hex_rt_layout(const HexDev& d, int64_t* off1, int64_t* off2, int64_t* n) {
  const int64_t mx = (int64_t)d.nx * d.p, my = (int64_t)d.ny * d.p, mz = (int64_t)d.nz * d.p;
  *off1 = (mx + 1) * my * mz;
  *off2 = *off1 + mx * (my + 1) * mz;
  *n = *off2 + mx * my * (mz + 1);
}

cudaError_t hex_curl(const HexDev& d, const double* A, double* B, cudaStream_t s) {
  int64_t o1, o2, n;
  hex_rt_layout(d, &o1, &o2, &n);
  const int blocks = (int)((d.ne + 127) / 128);
  switch (d.p) {
    case 1: hex_curl_kernel<1><<<blocks, 128, 0, s>>>(d, A, B, o1, o2); break;
    case 2: hex_curl_kernel<2><<<blocks, 128, 0, s>>>(d, A, B, o1, o2); break;
    case 3: hex_curl_kernel<3><<<blocks, 128, 0, s>>>(d, A, B, o1, o2); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---- coil load vector -------------------------------------------------------------
// Gauss-Legendre points per direction (<= 8) and the 1-D basis values there;
// passed to the kernel by value, so concurrent loads on different streams
// never share it.
struct LoadTab {
  int q;
  double w[8];
  double x[8];
  double bc[8][kMaxP + 1];  // closed basis at the points
  double bo[8][kMaxP];      // open basis at the points
};
struct CoilDev {
  double I0, xc, yc, r0, r1, z0, z1;
};

template <int P>
__global__ void hex_load_coil_kernel(HexDev d, const double* __restrict__ V, CoilDev coil, LoadTab c_load,
                                     double* __restrict__ b) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  constexpr int C = P + 1, O = P, NDC = O * C * C;
  const int ex = (int)(e % d.nx), ey = (int)((e / d.nx) % d.ny), ez = (int)(e / ((int64_t)d.nx * d.ny));
  auto vtx = [&](int a, int bb, int c) {
    return V + 3 * ((ex + a) + (int64_t)(d.nx + 1) * ((ey + bb) + (int64_t)(d.ny + 1) * (ez + c)));
  };
  const double *v0 = vtx(0, 0, 0), *vx = vtx(1, 0, 0), *vy = vtx(0, 1, 0), *vz = vtx(0, 0, 1);
  double J[9];
  for (int r = 0; r < 3; ++r) {
    J[3 * r] = vx[r] - v0[r];
    J[3 * r + 1] = vy[r] - v0[r];
    J[3 * r + 2] = vz[r] - v0[r];
  }
  const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
  double Ji[9];
  Ji[0] = (J[4] * J[8] - J[5] * J[7]) / det;
  Ji[1] = (J[2] * J[7] - J[1] * J[8]) / det;
  Ji[2] = (J[1] * J[5] - J[2] * J[4]) / det;
  Ji[3] = (J[5] * J[6] - J[3] * J[8]) / det;
  Ji[4] = (J[0] * J[8] - J[2] * J[6]) / det;
  Ji[5] = (J[2] * J[3] - J[0] * J[5]) / det;
  Ji[6] = (J[3] * J[7] - J[4] * J[6]) / det;
  Ji[7] = (J[1] * J[6] - J[0] * J[7]) / det;
  Ji[8] = (J[0] * J[4] - J[1] * J[3]) / det;
  const double adet = fabs(det);
  double be0[NDC], be1[NDC], be2[NDC];
  for (int i = 0; i < NDC; ++i) be0[i] = be1[i] = be2[i] = 0.0;
  const int q = c_load.q;
  for (int kz = 0; kz < q; ++kz)
    for (int ky = 0; ky < q; ++ky)
      for (int kx = 0; kx < q; ++kx) {
        const double xi[3] = {c_load.x[kx], c_load.x[ky], c_load.x[kz]};
        double x[3];
        for (int r = 0; r < 3; ++r) x[r] = v0[r] + J[3 * r] * xi[0] + J[3 * r + 1] * xi[1] + J[3 * r + 2] * xi[2];
        const double dx = x[0] - coil.xc, dy = x[1] - coil.yc;
        const double rr = sqrt(dx * dx + dy * dy);
        if (!(rr >= coil.r0 && rr <= coil.r1 && x[2] >= coil.z0 && x[2] <= coil.z1)) continue;
        const double jc[3] = {-coil.I0 * dy, coil.I0 * dx, 0.0};
        const double wq = c_load.w[kx] * c_load.w[ky] * c_load.w[kz] * adet;
        // reference-frame source: J^-1 jc
        double f[3];
        for (int r = 0; r < 3; ++r) f[r] = wq * (Ji[3 * r] * jc[0] + Ji[3 * r + 1] * jc[1] + Ji[3 * r + 2] * jc[2]);
        for (int c = 0; c < C; ++c)
          for (int bb = 0; bb < C; ++bb)
            for (int a = 0; a < O; ++a)
              be0[a + O * (bb + C * c)] += f[0] * c_load.bo[kx][a] * c_load.bc[ky][bb] * c_load.bc[kz][c];
        for (int c = 0; c < C; ++c)
          for (int bb = 0; bb < O; ++bb)
            for (int a = 0; a < C; ++a)
              be1[a + C * (bb + O * c)] += f[1] * c_load.bc[kx][a] * c_load.bo[ky][bb] * c_load.bc[kz][c];
        for (int c = 0; c < O; ++c)
          for (int bb = 0; bb < C; ++bb)
            for (int a = 0; a < C; ++a)
              be2[a + C * (bb + C * c)] += f[2] * c_load.bc[kx][a] * c_load.bc[ky][bb] * c_load.bo[kz][c];
      }
  scatter<double, P, 0>(d, b, ex, ey, ez, false, be0);
  scatter<double, P, 1>(d, b, ex, ey, ez, false, be1);
  scatter<double, P, 2>(d, b, ex, ey, ez, false, be2);
}

static LoadTab make_load_tab(const HexDev& d, int q, const double* xq, const double* wq, const double* bc,
                             const double* bo) {
  LoadTab t;
  std::memset(&t, 0, sizeof(t));
  t.q = q;
  for (int k = 0; k < q; ++k) {
    t.x[k] = xq[k];
    t.w[k] = wq[k];
    for (int j = 0; j <= d.p; ++j) t.bc[k][j] = bc[k * (d.p + 1) + j];
    for (int j = 0; j < d.p; ++j) t.bo[k][j] = bo[k * d.p + j];
  }
  return t;
}

// Affine map of element e: corner v0, Jacobian J (columns = edge vectors),
// inverse Ji, det.
struct HexMap {
  double v0[3], J[9], Ji[9], det;
};
__device__ __forceinline__ void hex_map(const HexDev& d, const double* __restrict__ V, int ex, int ey, int ez,
                                        HexMap& m) {
  auto vtx = [&](int a, int bb, int c) {
    return V + 3 * ((ex + a) + (int64_t)(d.nx + 1) * ((ey + bb) + (int64_t)(d.ny + 1) * (ez + c)));
  };
  const double *v0 = vtx(0, 0, 0), *vx = vtx(1, 0, 0), *vy = vtx(0, 1, 0), *vz = vtx(0, 0, 1);
  for (int r = 0; r < 3; ++r) {
    m.v0[r] = v0[r];
    m.J[3 * r] = vx[r] - v0[r];
    m.J[3 * r + 1] = vy[r] - v0[r];
    m.J[3 * r + 2] = vz[r] - v0[r];
  }
  const double* J = m.J;
  m.det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) + J[2] * (J[3] * J[7] - J[4] * J[6]);
  double* Ji = m.Ji;
  Ji[0] = (J[4] * J[8] - J[5] * J[7]) / m.det;
  Ji[1] = (J[2] * J[7] - J[1] * J[8]) / m.det;
  Ji[2] = (J[1] * J[5] - J[2] * J[4]) / m.det;
  Ji[3] = (J[5] * J[6] - J[3] * J[8]) / m.det;
  Ji[4] = (J[0] * J[8] - J[2] * J[6]) / m.det;
  Ji[5] = (J[2] * J[3] - J[0] * J[5]) / m.det;
  Ji[6] = (J[3] * J[7] - J[4] * J[6]) / m.det;
  Ji[7] = (J[1] * J[6] - J[0] * J[7]) / m.det;
  Ji[8] = (J[0] * J[4] - J[1] * J[3]) / m.det;
}

// ---- points of the q^3 Gauss-Legendre rule, x = v0 + J xi -------------------------
__global__ void hex_quad_points_kernel(HexDev d, const double* __restrict__ V, LoadTab t, double* __restrict__ xyz) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  const int ex = (int)(e % d.nx), ey = (int)((e / d.nx) % d.ny), ez = (int)(e / ((int64_t)d.nx * d.ny));
  HexMap m;
  hex_map(d, V, ex, ey, ez, m);
  const int q = t.q, q3 = q * q * q;
  for (int kz = 0; kz < q; ++kz)
    for (int ky = 0; ky < q; ++ky)
      for (int kx = 0; kx < q; ++kx) {
        const double xi[3] = {t.x[kx], t.x[ky], t.x[kz]};
        double* out = xyz + 3 * (e * q3 + kx + q * (ky + q * kz));
        for (int r = 0; r < 3; ++r) out[r] = m.v0[r] + m.J[3 * r] * xi[0] + m.J[3 * r + 1] * xi[1] + m.J[3 * r + 2] * xi[2];
      }
}

// ---- b = (J, w_i) for a caller-supplied source ------------------------------------
// per_point = 0: J is one vector per element; 1: J at the q^3 points of the rule.
// Covariant Piola: (j, w) = int (J^-1 j) . w_ref |det J|.
template <int P>
__global__ void hex_load_field_kernel(HexDev d, const double* __restrict__ V, LoadTab t, int per_point,
                                      const double* __restrict__ src, double* __restrict__ b) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  constexpr int C = P + 1, O = P, NDC = O * C * C;
  const int ex = (int)(e % d.nx), ey = (int)((e / d.nx) % d.ny), ez = (int)(e / ((int64_t)d.nx * d.ny));
  HexMap m;
  hex_map(d, V, ex, ey, ez, m);
  const double adet = fabs(m.det);
  double be0[NDC], be1[NDC], be2[NDC];
  for (int i = 0; i < NDC; ++i) be0[i] = be1[i] = be2[i] = 0.0;
  const int q = t.q, q3 = q * q * q;
  for (int kz = 0; kz < q; ++kz)
    for (int ky = 0; ky < q; ++ky)
      for (int kx = 0; kx < q; ++kx) {
        const double* jc = per_point ? src + 3 * (e * q3 + kx + q * (ky + q * kz)) : src + 3 * e;
        const double wq = t.w[kx] * t.w[ky] * t.w[kz] * adet;
        double f[3];
        for (int r = 0; r < 3; ++r) f[r] = wq * (m.Ji[3 * r] * jc[0] + m.Ji[3 * r + 1] * jc[1] + m.Ji[3 * r + 2] * jc[2]);
        for (int c = 0; c < C; ++c)
          for (int bb = 0; bb < C; ++bb)
            for (int a = 0; a < O; ++a)
              be0[a + O * (bb + C * c)] += f[0] * t.bo[kx][a] * t.bc[ky][bb] * t.bc[kz][c];
        for (int c = 0; c < C; ++c)
          for (int bb = 0; bb < O; ++bb)
            for (int a = 0; a < C; ++a)
              be1[a + C * (bb + O * c)] += f[1] * t.bc[kx][a] * t.bo[ky][bb] * t.bc[kz][c];
        for (int c = 0; c < O; ++c)
          for (int bb = 0; bb < C; ++bb)
            for (int a = 0; a < C; ++a)
              be2[a + C * (bb + C * c)] += f[2] * t.bc[kx][a] * t.bc[ky][bb] * t.bo[kz][c];
      }
  scatter<double, P, 0>(d, b, ex, ey, ez, false, be0);
  scatter<double, P, 1>(d, b, ex, ey, ez, false, be1);
  scatter<double, P, 2>(d, b, ex, ey, ez, false, be2);
}

// ---- b_i = (nu curl A, w_i) ---------------------------------------------------------
// curl A is the Raviart-Thomas field J r / det J (r the element-local curl of
// the reference dofs) and w = J^-T w_ref, so the Piola factors cancel:
// (curl A, w)_e = int r . w_ref over the reference cube.  Component c pairs RT
// component c (closed in c, open across) with Nedelec component c (open in c,
// closed across): one mixed 1-D mass per direction, exact.
template <int P>
__global__ void hex_curl_load_kernel(HexDev d, const double* __restrict__ nu, const double* __restrict__ A,
                                     double* __restrict__ b) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  constexpr int C = P + 1, O = P, NDC = O * C * C, RTC = C * O * O;
  const int ex = (int)(e % d.nx), ey = (int)((e / d.nx) % d.ny), ez = (int)(e / ((int64_t)d.nx * d.ny));
  double u0[NDC], u1[NDC], u2[NDC], r0[RTC], r1[RTC], r2[RTC];
  gather<double, P, 0>(d, A, ex, ey, ez, false, u0);
  gather<double, P, 1>(d, A, ex, ey, ez, false, u1);
  gather<double, P, 2>(d, A, ex, ey, ez, false, u2);
  curl_nd<double, P>(u0, u1, u2, r0, r1, r2);
  const double s = nu[e];
  kron3_acc<double, P, NdT<0, 0>::v, RtT<0, 0>::v, NdT<0, 1>::v, RtT<0, 1>::v, NdT<0, 2>::v, RtT<0, 2>::v, false>(
      r0, u0, s);
  kron3_acc<double, P, NdT<1, 0>::v, RtT<1, 0>::v, NdT<1, 1>::v, RtT<1, 1>::v, NdT<1, 2>::v, RtT<1, 2>::v, false>(
      r1, u1, s);
  kron3_acc<double, P, NdT<2, 0>::v, RtT<2, 0>::v, NdT<2, 1>::v, RtT<2, 1>::v, NdT<2, 2>::v, RtT<2, 2>::v, false>(
      r2, u2, s);
  scatter<double, P, 0>(d, b, ex, ey, ez, false, u0);
  scatter<double, P, 1>(d, b, ex, ey, ez, false, u1);
  scatter<double, P, 2>(d, b, ex, ey, ez, false, u2);
}

cudaError_t hex_quad_points(const HexDev& d, const double* V, int q, const double* xq, const double* wq,
                            const double* bc, const double* bo, double* xyz, cudaStream_t s) {
  const LoadTab t = make_load_tab(d, q, xq, wq, bc, bo);
  const int blocks = (int)((d.ne + 127) / 128);
  hex_quad_points_kernel<<<blocks, 128, 0, s>>>(d, V, t, xyz);
  return cudaGetLastError();
}

cudaError_t hex_load_field(const HexDev& d, const double* V, int per_point, const double* src, int q,
                           const double* xq, const double* wq, const double* bc, const double* bo, double* b,
                           cudaStream_t s) {
  const LoadTab t = make_load_tab(d, q, xq, wq, bc, bo);
  cudaError_t e = cudaMemsetAsync(b, 0, d.ndof * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const int blocks = (int)((d.ne + 127) / 128);
  switch (d.p) {
    case 1: hex_load_field_kernel<1><<<blocks, 128, 0, s>>>(d, V, t, per_point, src, b); break;
    case 2: hex_load_field_kernel<2><<<blocks, 128, 0, s>>>(d, V, t, per_point, src, b); break;
    case 3: hex_load_field_kernel<3><<<blocks, 128, 0, s>>>(d, V, t, per_point, src, b); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t hex_curl_load(const HexDev& d, const double* nu, const double* A, double* b, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(b, 0, d.ndof * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const int blocks = (int)((d.ne + 127) / 128);
  switch (d.p) {
    case 1: hex_curl_load_kernel<1><<<blocks, 128, 0, s>>>(d, nu, A, b); break;
    case 2: hex_curl_load_kernel<2><<<blocks, 128, 0, s>>>(d, nu, A, b); break;
    case 3: hex_curl_load_kernel<3><<<blocks, 128, 0, s>>>(d, nu, A, b); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t hex_load_coil(const HexDev& d, const double* V, const double coil[7], int q, const double* xq,
                          const double* wq, const double* bc, const double* bo, double* b, cudaStream_t s) {
  const LoadTab t = make_load_tab(d, q, xq, wq, bc, bo);
  cudaError_t e = cudaMemsetAsync(b, 0, d.ndof * sizeof(double), s);
  if (e != cudaSuccess) return e;
  const CoilDev cd{coil[0], coil[1], coil[2], coil[3], coil[4], coil[5], coil[6]};
  const int blocks = (int)((d.ne + 127) / 128);
  switch (d.p) {
    case 1: hex_load_coil_kernel<1><<<blocks, 128, 0, s>>>(d, V, cd, t, b); break;
    case 2: hex_load_coil_kernel<2><<<blocks, 128, 0, s>>>(d, V, cd, t, b); break;
    case 3: hex_load_coil_kernel<3><<<blocks, 128, 0, s>>>(d, V, cd, t, b); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace hc

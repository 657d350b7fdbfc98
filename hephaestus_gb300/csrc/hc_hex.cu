// hc_hex.cu -- dispatch of the hex apply kernels, the operator diagonal, and
// the 1-D tables in constant memory.  The apply kernel itself is in
// hc_hex_impl.cuh (instantiated per order in hc_hex_p{1,2,3}.cu).
#include <algorithm>

#include "hc_hex_impl.cuh"

namespace hc {

cudaError_t upload_tables_p1(const void* td, const void* tf);
cudaError_t upload_tables_p2(const void* td, const void* tf);
cudaError_t upload_tables_p3(const void* td, const void* tf);
cudaError_t upload_tables_p1s(const void* td, const void* tf);
cudaError_t upload_tables_p2s(const void* td, const void* tf);
cudaError_t upload_tables_post(const void* td, const void* tf);

// upper bound on the blocks of any apply launch (sizes the reduction partials)
int hex_apply_blocks(const HexDev& d) {
  const int legacy = (int)((d.ne + 127) / 128);
  const int b1 = brick_blocks<1>(d), b2 = brick_blocks<2>(d), b3 = brick_blocks<3>(d);
  const int s1 = brick_blocks<1, 1>(d), s2 = brick_blocks<2, 1>(d);
  return std::max(std::max(std::max(legacy, b1), std::max(b2, b3)), std::max(s1, s2));
}

// instantiated in hc_hex_p{1,2,3}.cu
#define HC_EXTERN_LAUNCH(T, P)                                                                          \
  extern template cudaError_t hex_launch_p<T, P>(const HexDev&, const T*, const T*, T*, T, T, bool,     \
                                                 KrylovScalars*, double*, cudaStream_t, bool);
HC_EXTERN_LAUNCH(double, 1)
HC_EXTERN_LAUNCH(double, 2)
HC_EXTERN_LAUNCH(double, 3)
HC_EXTERN_LAUNCH(float, 1)
HC_EXTERN_LAUNCH(float, 2)
HC_EXTERN_LAUNCH(float, 3)
#undef HC_EXTERN_LAUNCH

template <typename T>
cudaError_t hex_apply(const HexDev& d, const T* fac, const T* x, T* y, double ms, double cs, bool masked,
                      KrylovScalars* S, double* partials, cudaStream_t s, bool yz) {
  switch (d.p) {
    case 1: return hex_launch_p<T, 1>(d, fac, x, y, (T)ms, (T)cs, masked, S, partials, s, yz);
    case 2: return hex_launch_p<T, 2>(d, fac, x, y, (T)ms, (T)cs, masked, S, partials, s, yz);
    case 3: return hex_launch_p<T, 3>(d, fac, x, y, (T)ms, (T)cs, masked, S, partials, s, yz);
    default: return cudaErrorInvalidValue;
  }
}
template cudaError_t hex_apply<double>(const HexDev&, const double*, const double*, double*, double, double,
                                       bool, KrylovScalars*, double*, cudaStream_t, bool);
template cudaError_t hex_apply<float>(const HexDev&, const float*, const float*, float*, double, double,
                                      bool, KrylovScalars*, double*, cudaStream_t, bool);

// ---------------------------------------------------------------------------
// Diagonal of K (FP64).  For a unit dof vector the element curl is a sum of
// two rank-1 tensors (one per Raviart-Thomas component it feeds), so each
// diagonal entry is a short sum of products of 1-D bilinear forms.
// ---------------------------------------------------------------------------
template <int P>
__device__ double q1d(int tr, int tc, const double* vr, const double* vc) {
  // vr^T M_{tr,tc} vc with M the 1-D mass matrix between basis types
  const Tab1D<double>& t = c_tabd[P];
  const int nr = tr == kC ? P + 1 : P, nc = tc == kC ? P + 1 : P;
  double s = 0.0;
  for (int i = 0; i < nr; ++i)
    for (int j = 0; j < nc; ++j) {
      double m;
      if (tr == kC && tc == kC) m = t.Mcc[i][j];
      else if (tr == kC && tc == kO) m = t.Mco[i][j];
      else if (tr == kO && tc == kC) m = t.Mco[j][i];
      else m = t.Moo[i][j];
      s += vr[i] * m * vc[j];
    }
  return s;
}

template <int P>
__global__ void hex_diag_kernel(HexDev d, double* __restrict__ diag, double ms, double cs) {
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= d.ne) return;
  constexpr int C = P + 1, O = P;
  const int ex = (int)(e % d.nx), ey = (int)((e / d.nx) % d.ny), ez = (int)(e / ((int64_t)d.nx * d.ny));
  double fm[6], fc[6];
  for (int k = 0; k < 6; ++k) {
    fm[k] = d.fac[(int64_t)k * d.ne + e];
    fc[k] = d.fac[(int64_t)(6 + k) * d.ne + e];
  }
  const Tab1D<double>& t = c_tabd[P];
#pragma unroll 1
  for (int comp = 0; comp < 3; ++comp) {
    const int n0 = comp == 0 ? O : C, n1 = comp == 1 ? O : C, n2 = comp == 2 ? O : C;
#pragma unroll 1
    for (int c = 0; c < n2; ++c)
#pragma unroll 1
      for (int b = 0; b < n1; ++b)
#pragma unroll 1
        for (int a = 0; a < n0; ++a) {
          const int idx[3] = {a, b, c};
          // mass: diagonal block (comp, comp)
          double mv = fm[symk(comp, comp)];
          for (int dd = 0; dd < 3; ++dd) {
            const int i = idx[dd];
            mv *= (dd == comp) ? t.Moo[i][i] : t.Mcc[i][i];
          }
          // curl of the unit dof: two RT components B1, B2 with rank-1 factors
          // vectors per direction (length by RT type), sign
          double v[2][3][kMaxP + 1];
          int comps[2], types[2][3];
          double sg[2];
          const int c1 = (comp + 1) % 3, c2 = (comp + 2) % 3;
          // r_{c1} = +D_{c2} u_comp ; r_{c2} = -D_{c1} u_comp   (cyclic curl)
          comps[0] = c1;
          sg[0] = 1.0;
          comps[1] = c2;
          sg[1] = -1.0;
          for (int q = 0; q < 2; ++q) {
            const int B = comps[q];
            const int ddir = (q == 0) ? c2 : c1;  // differentiated direction
            for (int dd = 0; dd < 3; ++dd) {
              types[q][dd] = (dd == B) ? kC : kO;
              for (int k = 0; k <= kMaxP; ++k) v[q][dd][k] = 0.0;
              if (dd == ddir) {
                for (int k = 0; k < O; ++k) v[q][dd][k] = t.D[k][idx[dd]];
              } else {
                v[q][dd][idx[dd]] = 1.0;
              }
            }
          }
          double cv = 0.0;
#pragma unroll 1
          for (int q = 0; q < 2; ++q)
#pragma unroll 1
            for (int r = 0; r < 2; ++r) {
              const double f = fc[symk(comps[q], comps[r])];
              if (f == 0.0) continue;
              double prod = sg[q] * sg[r] * f;
              for (int dd = 0; dd < 3; ++dd) {
                const int tr = types[q][dd], tc = types[r][dd];
                double s = 0.0;
                if (tr == kC && tc == kC) s = q1d<P>(kC, kC, v[q][dd], v[r][dd]);
                else if (tr == kC && tc == kO) s = q1d<P>(kC, kO, v[q][dd], v[r][dd]);
                else if (tr == kO && tc == kC) s = q1d<P>(kO, kC, v[q][dd], v[r][dd]);
                else s = q1d<P>(kO, kO, v[q][dd], v[r][dd]);
                prod *= s;
              }
              cv += prod;
            }
          int64_t g;
          if (comp == 0) g = gdof<P, 0>(d, ex, ey, ez, a, b, c);
          else if (comp == 1) g = gdof<P, 1>(d, ex, ey, ez, a, b, c);
          else g = gdof<P, 2>(d, ex, ey, ez, a, b, c);
          atomicAdd(diag + g, ms * mv + cs * cv);
        }
  }
}

cudaError_t hex_diag_scaled(const HexDev& d, double* diag, double ms, double cs, cudaStream_t s) {
  const int blocks = (int)((d.ne + 127) / 128);
  switch (d.p) {
    case 1: hex_diag_kernel<1><<<blocks, 128, 0, s>>>(d, diag, ms, cs); break;
    case 2: hex_diag_kernel<2><<<blocks, 128, 0, s>>>(d, diag, ms, cs); break;
    case 3: hex_diag_kernel<3><<<blocks, 128, 0, s>>>(d, diag, ms, cs); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t hex_diag(const HexDev& d, double* diag, cudaStream_t s) { return hex_diag_scaled(d, diag, 1.0, 1.0, s); }

void hex_tile_table(int p, int shape, int nx, int ny, std::vector<int>& tab) {
  if (p == 1) shape ? build_tile_table<1, 1>(nx, ny, tab) : build_tile_table<1, 0>(nx, ny, tab);
  else if (p == 2) shape ? build_tile_table<2, 1>(nx, ny, tab) : build_tile_table<2, 0>(nx, ny, tab);
  else tab.assign(1, 0);
}

cudaError_t upload_tables() {
  Tab1D<double> td[kMaxP + 1];
  Tab1D<float> tf[kMaxP + 1];
  memset(td, 0, sizeof(td));
  memset(tf, 0, sizeof(tf));
  for (int p = 1; p <= kMaxP; ++p) {
    build_tab1d(p, &td[p]);
    const double* a = reinterpret_cast<const double*>(&td[p]);
    float* b = reinterpret_cast<float*>(&tf[p]);
    for (size_t i = 0; i < sizeof(Tab1D<double>) / sizeof(double); ++i) b[i] = (float)a[i];
  }
  cudaError_t e = upload_tables_here(td, tf);
  if (e == cudaSuccess) e = upload_tables_p1(td, tf);
  if (e == cudaSuccess) e = upload_tables_p2(td, tf);
  if (e == cudaSuccess) e = upload_tables_p3(td, tf);
  if (e == cudaSuccess) e = upload_tables_p1s(td, tf);
  if (e == cudaSuccess) e = upload_tables_p2s(td, tf);
  if (e == cudaSuccess) e = upload_tables_post(td, tf);
  return e;
}

}  // namespace hc

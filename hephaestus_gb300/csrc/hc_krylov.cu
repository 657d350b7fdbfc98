// hc_krylov.cu -- device PCG, Chebyshev-Jacobi preconditioner, Lanczos bound,
// and FP32-inner / FP64-outer iterative refinement.
//
// Replaces, for this operator, the HyprePCG solve of the reference
// (src/formulations/HCurl/hcurl_formulation.cpp:81-85,
// src/problem_builders/problem_builder_base.cpp:221-253,
// src/solvers/hephaestus_solvers.hpp:34-57).  All scalars (alpha, beta, dots,
// the stopping test) live in device memory; the host reads them once per batch
// of iterations.  Vector kernels are grid-stride streams over 2 x 152 blocks;
// every dot is a deterministic two-level FP64 reduction (FP32 products are
// summed in FP32 over runs of 8 before entering FP64).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "hc_internal.h"
#include "hc_reduce.cuh"

namespace hc {

#define GS_LOOP(i, n) \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// Vector stride of the Krylov work space: every work vector starts on a
// 256-byte boundary, so the 16-byte vector kernels apply to all of them.
static inline int64_t vstride(int64_t n) { return (n + 63) & ~(int64_t)63; }

static inline unsigned vgrid(int64_t n) {
  int64_t b = (n + kRedThreads - 1) / kRedThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, kRedBlocks));
}

// ---------------------------------------------------------------------------
// setup kernels
// ---------------------------------------------------------------------------
__global__ void k_diag_finish(int64_t n, const uint8_t* __restrict__ ess, double* d, double* dinv, float* dinvf,
                              double* sd, float* sdf, int* bad) {
  GS_LOOP(i, n) {
    double v = ess[i] ? 1.0 : d[i];
    if (!(v > 0.0) || !isfinite(v)) {
      atomicExch(bad, 1);
      v = 1.0;
    }
    d[i] = v;
    const double iv = 1.0 / v;
    dinv[i] = iv;
    dinvf[i] = (float)iv;
    const double s = sqrt(iv);
    sd[i] = s;
    sdf[i] = (float)s;
  }
}

cudaError_t diag_finish(int64_t n, const uint8_t* ess, double* d, double* dinv, float* dinvf, double* sd,
                        float* sdf, cudaStream_t s) {
  int* bad = nullptr;
  cudaError_t e = cudaMallocAsync(&bad, sizeof(int), s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(bad, 0, sizeof(int), s);
  k_diag_finish<<<vgrid(n), kRedThreads, 0, s>>>(n, ess, d, dinv, dinvf, sd, sdf, bad);
  int hb = 0;
  cudaMemcpyAsync(&hb, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  cudaFreeAsync(bad, s);
  if (e != cudaSuccess) return e;
  return hb ? cudaErrorInvalidValue : cudaGetLastError();
}

template <typename T>
__global__ void k_init_masked(int64_t n, const uint8_t* __restrict__ ess, const T* __restrict__ x,
                              T* __restrict__ y) {
  GS_LOOP(i, n) y[i] = ess[i] ? x[i] : T(0);
}
template <typename T>
cudaError_t init_masked(int64_t n, const uint8_t* ess, const T* x, T* y, cudaStream_t s) {
  k_init_masked<T><<<vgrid(n), kRedThreads, 0, s>>>(n, ess, x, y);
  return cudaGetLastError();
}
template cudaError_t init_masked<double>(int64_t, const uint8_t*, const double*, double*, cudaStream_t);
template <typename T>
__global__ void k_init_masked_multi(int64_t n, int nrhs, const uint8_t* __restrict__ ess, const T* __restrict__ x,
                                    T* __restrict__ y) {
  GS_LOOP(i, n * nrhs) y[i] = ess[i / nrhs] ? x[i] : T(0);
}
// 16-byte chunks of a [dof][rhs] block with 4 | nrhs (a power of two): the
// row of chunk i is i >> shift, no division per element
template <typename T>
__global__ void k_init_masked_multi_v(int64_t nchunks, int shift, const uint8_t* __restrict__ ess,
                                      const uint4* __restrict__ x, uint4* __restrict__ y) {
  GS_LOOP(i, nchunks) y[i] = ess[i >> shift] ? x[i] : make_uint4(0u, 0u, 0u, 0u);
}
template <typename T>
cudaError_t init_masked_multi(int64_t n, int nrhs, const uint8_t* ess, const T* x, T* y, cudaStream_t s) {
  const int per = (int)(16 / sizeof(T));  // values per 16-byte chunk
  if (nrhs % per == 0 && ((uintptr_t)x | (uintptr_t)y) % 16 == 0 && (nrhs & (nrhs - 1)) == 0) {
    int shift = 0;
    while ((1 << shift) < nrhs / per) ++shift;
    const int64_t nch = n * (nrhs / per);
    const int64_t blocks = std::min<int64_t>((nch + 255) / 256, 152 * 16);
    k_init_masked_multi_v<T><<<(unsigned)std::max<int64_t>(1, blocks), 256, 0, s>>>(
        nch, shift, ess, reinterpret_cast<const uint4*>(x), reinterpret_cast<uint4*>(y));
    return cudaGetLastError();
  }
  k_init_masked_multi<T><<<vgrid(n * nrhs), kRedThreads, 0, s>>>(n, nrhs, ess, x, y);
  return cudaGetLastError();
}
template cudaError_t init_masked_multi<double>(int64_t, int, const uint8_t*, const double*, double*, cudaStream_t);
template cudaError_t init_masked_multi<float>(int64_t, int, const uint8_t*, const float*, float*, cudaStream_t);
template cudaError_t init_masked<float>(int64_t, const uint8_t*, const float*, float*, cudaStream_t);

// q.p over all dofs; alpha = rz / pq with the breakdown test (PCG mode of an
// operator without a fused energy reduction)
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_dot_alpha(int64_t n, const T* __restrict__ p, const T* __restrict__ q, KrylovScalars* S, double* partials) {
  if (S->done) return;
  double v[1] = {0.0}, tot[1];
  T acc = T(0);  // per-thread sum in T: no per-element FP64 work (GB300's FP64 rate is low)
  GS_LOOP(i, n) acc += p[i] * q[i];
  v[0] += (double)acc;
  block_sum_n<1>(v);
  if (grid_sum_n<1>(v, partials, &S->counter[0], tot)) {
    const double pq = tot[0];
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
template <typename T>
cudaError_t dot_alpha(int64_t n, const T* p, const T* q, KrylovScalars* S, double* partials, cudaStream_t s) {
  k_dot_alpha<T><<<vgrid(n), kRedThreads, 0, s>>>(n, p, q, S, partials);
  return cudaGetLastError();
}
template cudaError_t dot_alpha<double>(int64_t, const double*, const double*, KrylovScalars*, double*, cudaStream_t);
template cudaError_t dot_alpha<float>(int64_t, const float*, const float*, KrylovScalars*, double*, cudaStream_t);

template <typename T>
static const T* tetK_of(const hcop* h);
template <>
const double* tetK_of<double>(const hcop* h) {
  return h->tetK64;
}
template <>
const float* tetK_of<float>(const hcop* h) {
  return h->tetK32;
}

// y += P K P x on top of the caller's initialisation of y ((I-P)x for J).
template <typename T>
cudaError_t OpJ<T>::apply(const T* x, T* y, KrylovScalars* S, double* partials, cudaStream_t s,
                          bool y_zero_free) const {
  if (h->type == HC_TET) {
    cudaError_t e = tet_apply_launch<T>(h, tetK_of<T>(h), x, y, 1, true, 1.0, S ? &S->done : nullptr, s);
    if (e == cudaSuccess && S) e = dot_alpha<T>(h->ndof, x, y, S, partials, s);
    return e;
  }
  const HexDev d = h->hexdev();
  return hex_apply<T>(d, fac, x, y, h->has_mass ? 1.0 : 0.0, 1.0, true, S, partials, s, y_zero_free);
}
template struct OpJ<double>;
template struct OpJ<float>;

// ---------------------------------------------------------------------------
// PCG kernels
// ---------------------------------------------------------------------------
// r = b - q (q = J x0); bb, rr and (Jacobi) rz; initial stopping test
template <typename T, bool JAC>
__global__ void __launch_bounds__(kRedThreads)
    k_pcg_setup(int64_t n, const T* __restrict__ b, const T* __restrict__ q, T* __restrict__ r,
                const T* __restrict__ dinv, KrylovScalars* S, double* partials) {
  double v[3] = {0.0, 0.0, 0.0}, tot[3];
  T a0 = T(0), a1 = T(0), a2 = T(0);  // per-thread sums in T (no per-element FP64 work)
  GS_LOOP(i, n) {
    const T bi = b[i];
    const T ri = bi - q[i];
    r[i] = ri;
    a0 += bi * bi;
    a1 += ri * ri;
    if (JAC) a2 += ri * ri * (dinv ? dinv[i] : T(1));
  }
  v[0] = (double)a0;
  v[1] = (double)a1;
  v[2] = (double)a2;
  block_sum_n<3>(v);
  if (grid_sum_n<3>(v, partials, &S->counter[4], tot)) {
    S->bb = tot[0];
    S->rr = tot[1];
    S->tol2 = fmax(S->rtol2 * tot[0], S->atol2);
    if (JAC) S->rz = tot[2];
    S->it = 0;
    S->beta = 0.0;
    S->done = 0;
    S->status = HC_NOT_CONVERGED;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      S->done = 1;
      S->status = HC_BREAKDOWN;
    } else if (tot[1] <= S->tol2) {
      S->done = 1;
      S->status = HC_OK;
    }
  }
}

// x += alpha p; r -= alpha q; rr (and Jacobi rz = r.D^-1 r); stopping test; beta.
// zout != nullptr: also z = D^-1 r (the Jacobi part of the auxiliary-space preconditioner)
template <typename T, bool JAC>
__global__ void __launch_bounds__(kRedThreads)
    k_pcg_update(int64_t n, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                 const T* __restrict__ q, const T* __restrict__ dinv, KrylovScalars* S, double* partials,
                 T* __restrict__ zout = nullptr) {
  if (S->done) return;
  const T a = (T)S->alpha;
  double v[2] = {0.0, 0.0}, tot[2];
  T rrt = T(0), rzt = T(0);  // per-thread sums in T (no per-element FP64 work)
  GS_LOOP(i, n) {
    x[i] += a * p[i];
    const T ri = r[i] - a * q[i];
    r[i] = ri;
    if (zout) zout[i] = dinv[i] * ri;
    rrt += ri * ri;
    if (JAC) rzt += ri * ri * (dinv ? dinv[i] : T(1));
  }
  v[0] += (double)rrt;
  v[1] += (double)rzt;
  block_sum_n<2>(v);
  if (grid_sum_n<2>(v, partials, &S->counter[2], tot)) {
    S->rr = tot[0];
    S->it += 1;
    if (!isfinite(tot[0])) {
      S->done = 1;
      S->status = HC_BREAKDOWN;
    } else if (tot[0] <= S->tol2) {
      S->done = 1;
      S->status = HC_OK;
    } else if (S->it >= S->maxit) {
      S->done = 1;
      S->status = HC_NOT_CONVERGED;
    }
    if (JAC) {
      S->beta = tot[1] / S->rz;
      S->rz = tot[1];
    }
  }
}

// p = z + beta p (z = D^-1 r for Jacobi); q = (I-P) p; S->pq = sum_ess p_i^2
template <typename T, bool JAC>
__global__ void __launch_bounds__(kRedThreads)
    k_pcg_dir(int64_t n, const T* __restrict__ zr, const T* __restrict__ dinv, T* __restrict__ p,
              T* __restrict__ q, const uint8_t* __restrict__ ess, KrylovScalars* S, double* partials) {
  if (S->done) return;
  const T b = (T)S->beta;
  double v[1] = {0.0}, tot[1];
  GS_LOOP(i, n) {
    const T z = JAC ? (dinv ? dinv[i] * zr[i] : zr[i]) : zr[i];
    const T pi = z + b * p[i];
    p[i] = pi;
    const bool e = ess[i] != 0;
    q[i] = e ? pi : T(0);
    if (e) v[0] += (double)pi * (double)pi;
  }
  block_sum_n<1>(v);
  if (grid_sum_n<1>(v, partials, &S->counter[3], tot)) S->pq = tot[0];
}

// rz = r.z ; first: beta = 0, else beta = rz_new / rz
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_rz_beta(int64_t n, const T* __restrict__ r, const T* __restrict__ z, int first, KrylovScalars* S,
              double* partials) {
  if (S->done) return;
  double v[1] = {0.0}, tot[1];
  T acc = T(0);  // per-thread sum in T (no per-element FP64 work)
  GS_LOOP(i, n) acc += r[i] * z[i];
  v[0] += (double)acc;
  block_sum_n<1>(v);
  if (grid_sum_n<1>(v, partials, &S->counter[5], tot)) {
    if (first) {
      S->beta = 0.0;
    } else {
      S->beta = tot[0] / S->rz;
    }
    S->rz = tot[0];
  }
}

// ---- 16-byte forms of the per-iteration kernels ---------------------------
// Same arithmetic as k_pcg_update / k_pcg_dir / k_rz_beta, on 16-byte chunks
// (4 floats or 2 doubles) so that each thread keeps 5-6 wide loads in flight:
// the scalar forms, one 4-byte load per vector per loop trip, are bound by
// memory latency at 2 x 152 blocks.  All vectors 16-byte aligned; the last
// n % W elements go through a scalar tail.
template <typename T>
struct Chunk16 {
  static constexpr int W = (int)(16 / sizeof(T));
  T v[W];
  __device__ __forceinline__ void load(const T* __restrict__ p, int64_t c) {
    const uint4 u = reinterpret_cast<const uint4*>(p)[c];
    memcpy(v, &u, 16);
  }
  __device__ __forceinline__ void store(T* __restrict__ p, int64_t c) const {
    uint4 u;
    memcpy(&u, v, 16);
    reinterpret_cast<uint4*>(p)[c] = u;
  }
};

template <typename T, bool JAC>
__global__ void __launch_bounds__(kRedThreads)
    k_pcg_update_v(int64_t n, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                   const T* __restrict__ q, const T* __restrict__ dinv, KrylovScalars* S, double* partials,
                   T* __restrict__ zout) {
  if (S->done) return;
  constexpr int W = Chunk16<T>::W;
  const T a = (T)S->alpha;
  const int64_t nc = n / W, t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                st = (int64_t)gridDim.x * blockDim.x;
  const bool needd = zout != nullptr || (JAC && dinv != nullptr);
  T rrt = T(0), rzt = T(0);
#pragma unroll 2
  for (int64_t c = t0; c < nc; c += st) {
    Chunk16<T> xv, rv, pv, qv, dv;
    xv.load(x, c);
    rv.load(r, c);
    pv.load(p, c);
    qv.load(q, c);
    if (needd) dv.load(dinv, c);
#pragma unroll
    for (int w = 0; w < W; ++w) {
      xv.v[w] += a * pv.v[w];
      const T ri = rv.v[w] - a * qv.v[w];
      rv.v[w] = ri;
      rrt += ri * ri;
      if (JAC) rzt += ri * ri * (dinv ? dv.v[w] : T(1));
      if (zout) dv.v[w] *= ri;
    }
    xv.store(x, c);
    rv.store(r, c);
    if (zout) dv.store(zout, c);
  }
  for (int64_t i = nc * W + t0; i < n; i += st) {
    x[i] += a * p[i];
    const T ri = r[i] - a * q[i];
    r[i] = ri;
    if (zout) zout[i] = dinv[i] * ri;
    rrt += ri * ri;
    if (JAC) rzt += ri * ri * (dinv ? dinv[i] : T(1));
  }
  double v[2] = {(double)rrt, (double)rzt}, tot[2];
  block_sum_n<2>(v);
  if (grid_sum_n<2>(v, partials, &S->counter[2], tot)) {
    S->rr = tot[0];
    S->it += 1;
    if (!isfinite(tot[0])) {
      S->done = 1;
      S->status = HC_BREAKDOWN;
    } else if (tot[0] <= S->tol2) {
      S->done = 1;
      S->status = HC_OK;
    } else if (S->it >= S->maxit) {
      S->done = 1;
      S->status = HC_NOT_CONVERGED;
    }
    if (JAC) {
      S->beta = tot[1] / S->rz;
      S->rz = tot[1];
    }
  }
}

template <typename T, bool JAC>
__global__ void __launch_bounds__(kRedThreads)
    k_pcg_dir_v(int64_t n, const T* __restrict__ zr, const T* __restrict__ dinv, T* __restrict__ p,
                T* __restrict__ q, const uint8_t* __restrict__ ess, KrylovScalars* S, double* partials) {
  if (S->done) return;
  constexpr int W = Chunk16<T>::W;
  const T b = (T)S->beta;
  const int64_t nc = n / W, t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                st = (int64_t)gridDim.x * blockDim.x;
  double v[1] = {0.0}, tot[1];
#pragma unroll 2
  for (int64_t c = t0; c < nc; c += st) {
    Chunk16<T> zv, pv, dv;
    zv.load(zr, c);
    pv.load(p, c);
    if (JAC && dinv) dv.load(dinv, c);
    uint8_t m[W];
    if constexpr (W == 4) {
      const uchar4 e4 = reinterpret_cast<const uchar4*>(ess)[c];
      m[0] = e4.x, m[1] = e4.y, m[2] = e4.z, m[3] = e4.w;
    } else {
      const uchar2 e2 = reinterpret_cast<const uchar2*>(ess)[c];
      m[0] = e2.x, m[1] = e2.y;
    }
    Chunk16<T> qv;
#pragma unroll
    for (int w = 0; w < W; ++w) {
      const T z = JAC ? (dinv ? dv.v[w] * zv.v[w] : zv.v[w]) : zv.v[w];
      const T pi = z + b * pv.v[w];
      pv.v[w] = pi;
      qv.v[w] = m[w] ? pi : T(0);
      if (m[w]) v[0] += (double)pi * (double)pi;
    }
    pv.store(p, c);
    qv.store(q, c);
  }
  for (int64_t i = nc * W + t0; i < n; i += st) {
    const T z = JAC ? (dinv ? dinv[i] * zr[i] : zr[i]) : zr[i];
    const T pi = z + b * p[i];
    p[i] = pi;
    const bool e = ess[i] != 0;
    q[i] = e ? pi : T(0);
    if (e) v[0] += (double)pi * (double)pi;
  }
  block_sum_n<1>(v);
  if (grid_sum_n<1>(v, partials, &S->counter[3], tot)) S->pq = tot[0];
}

template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_rz_beta_v(int64_t n, const T* __restrict__ r, const T* __restrict__ z, int first, KrylovScalars* S,
                double* partials) {
  if (S->done) return;
  constexpr int W = Chunk16<T>::W;
  const int64_t nc = n / W, t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x,
                st = (int64_t)gridDim.x * blockDim.x;
  T acc = T(0);
#pragma unroll 4
  for (int64_t c = t0; c < nc; c += st) {
    Chunk16<T> rv, zv;
    rv.load(r, c);
    zv.load(z, c);
#pragma unroll
    for (int w = 0; w < W; ++w) acc += rv.v[w] * zv.v[w];
  }
  for (int64_t i = nc * W + t0; i < n; i += st) acc += r[i] * z[i];
  double v[1] = {(double)acc}, tot[1];
  block_sum_n<1>(v);
  if (grid_sum_n<1>(v, partials, &S->counter[5], tot)) {
    S->beta = first ? 0.0 : tot[0] / S->rz;
    S->rz = tot[0];
  }
}

static inline bool al16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// z = D^-1 r with no solver state (hc_precond_apply_device)
__global__ void k_jacobi(int64_t n, const double* __restrict__ dinv, const double* __restrict__ r,
                         double* __restrict__ z) {
  GS_LOOP(i, n) z[i] = dinv[i] * r[i];
}
cudaError_t jacobi_apply(int64_t n, const double* dinv, const double* r, double* z, cudaStream_t s) {
  k_jacobi<<<vgrid(n), kRedThreads, 0, s>>>(n, dinv, r, z);
  return cudaGetLastError();
}

// z = D^-1 r (the Jacobi part of the auxiliary-space preconditioner)
template <typename T>
__global__ void k_jz(int64_t n, const T* __restrict__ r, const T* __restrict__ dinv, T* __restrict__ z,
                     const KrylovScalars* S) {
  if (S->done) return;
  GS_LOOP(i, n) z[i] = dinv[i] * r[i];
}

// Chebyshev iteration (Saad, Iterative Methods for Sparse Linear Systems,
// Alg. 12.1) on D^-1 J z = D^-1 r with a fixed degree: a fixed SPD
// polynomial preconditioner when lmax bounds the spectrum of D^-1 J (and the
// smoother of HC_PRECOND_AUX_MULT).  One step:
//     d = c1 d_prev + c2 D^-1 (r - w),  z += d     (w = J z on entry)
// flags: kCbZ0   z = 0 on entry (first step: r - w = r, z = d, w unread)
//        kCbDkZ  d_prev = z (the step after a first step from z = 0)
//        kCbDk   d_prev = dk (read)            kCbStoreDk  dk = d
//        kCbInitW w = (I - P) z afterwards (the next operator apply's start)
// VEC: 16-byte loads and stores (every vector 16-byte aligned, ess aligned
// to the chunk width), with a scalar tail.
enum { kCbZ0 = 1, kCbDkZ = 2, kCbDk = 4, kCbStoreDk = 8, kCbInitW = 16 };
template <typename T>
__device__ __forceinline__ void cheb_elem(T& zi, T& wi, T& di, T ri, T dvi, T dki, bool e, T c1, T c2, int f) {
  const T res = (f & kCbZ0) ? ri : ri - wi;
  const T prev = (f & kCbDkZ) ? zi : ((f & kCbDk) ? dki : T(0));
  di = c1 * prev + c2 * dvi * res;
  zi = (f & kCbZ0) ? di : zi + di;
  if (f & kCbInitW) wi = e ? zi : T(0);
}
template <typename T, bool VEC>
__global__ void __launch_bounds__(kRedThreads)
    k_cheb_step(int64_t n, const T* __restrict__ r, const T* __restrict__ dinv, T* __restrict__ z,
                T* __restrict__ dk, T* __restrict__ w, const uint8_t* __restrict__ ess, T c1, T c2, int f,
                const KrylovScalars* S) {
  if (S->done) return;
  constexpr int W = Chunk16<T>::W;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, st = (int64_t)gridDim.x * blockDim.x;
  const int64_t nc = VEC ? n / W : 0;
  if (VEC) {
#pragma unroll 2
    for (int64_t c = t0; c < nc; c += st) {
      Chunk16<T> rv, dv, zv, wv, kv, ov;
      rv.load(r, c);
      dv.load(dinv, c);
      if (!(f & kCbZ0)) {
        zv.load(z, c);
        wv.load(w, c);
      }
      if (f & kCbDk) kv.load(dk, c);
      uint8_t m[W];
      if constexpr (W == 4) {
        const uchar4 e4 = reinterpret_cast<const uchar4*>(ess)[c];
        m[0] = e4.x, m[1] = e4.y, m[2] = e4.z, m[3] = e4.w;
      } else {
        const uchar2 e2 = reinterpret_cast<const uchar2*>(ess)[c];
        m[0] = e2.x, m[1] = e2.y;
      }
#pragma unroll
      for (int q = 0; q < W; ++q)
        cheb_elem<T>(zv.v[q], wv.v[q], ov.v[q], rv.v[q], dv.v[q], kv.v[q], m[q] != 0, c1, c2, f);
      zv.store(z, c);
      if (f & kCbStoreDk) ov.store(dk, c);
      if (f & kCbInitW) wv.store(w, c);
    }
  }
  for (int64_t i = nc * W + t0; i < n; i += st) {
    T zi = (f & kCbZ0) ? T(0) : z[i], wi = (f & kCbZ0) ? T(0) : w[i], di;
    cheb_elem<T>(zi, wi, di, r[i], dinv[i], (f & kCbDk) ? dk[i] : T(0), ess[i] != 0, c1, c2, f);
    z[i] = zi;
    if (f & kCbStoreDk) dk[i] = di;
    if (f & kCbInitW) w[i] = wi;
  }
}

// HC_PRECOND_AUX_MULT: t = r - w (w = J z after the pre-smoothing)
template <typename T, bool VEC>
__global__ void __launch_bounds__(kRedThreads)
    k_amul_t(int64_t n, const T* __restrict__ r, const T* __restrict__ w, T* __restrict__ t,
             const KrylovScalars* S) {
  if (S->done) return;
  constexpr int W = Chunk16<T>::W;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, st = (int64_t)gridDim.x * blockDim.x;
  const int64_t nc = VEC ? n / W : 0;
  if (VEC) {
#pragma unroll 2
    for (int64_t c = t0; c < nc; c += st) {
      Chunk16<T> rv, wv;
      rv.load(r, c);
      wv.load(w, c);
#pragma unroll
      for (int q = 0; q < W; ++q) rv.v[q] -= wv.v[q];
      rv.store(t, c);
    }
  }
  for (int64_t i = nc * W + t0; i < n; i += st) t[i] = r[i] - w[i];
}
// w = (I - P) z (the start of an operator apply)
template <typename T, bool VEC>
__global__ void __launch_bounds__(kRedThreads)
    k_init_w(int64_t n, const T* __restrict__ z, T* __restrict__ w, const uint8_t* __restrict__ ess,
             const KrylovScalars* S) {
  if (S->done) return;
  constexpr int W = Chunk16<T>::W;
  const int64_t t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, st = (int64_t)gridDim.x * blockDim.x;
  const int64_t nc = VEC ? n / W : 0;
  if (VEC) {
#pragma unroll 2
    for (int64_t c = t0; c < nc; c += st) {
      Chunk16<T> zv;
      zv.load(z, c);
      uint8_t m[W];
      if constexpr (W == 4) {
        const uchar4 e4 = reinterpret_cast<const uchar4*>(ess)[c];
        m[0] = e4.x, m[1] = e4.y, m[2] = e4.z, m[3] = e4.w;
      } else {
        const uchar2 e2 = reinterpret_cast<const uchar2*>(ess)[c];
        m[0] = e2.x, m[1] = e2.y;
      }
#pragma unroll
      for (int q = 0; q < W; ++q) zv.v[q] = m[q] ? zv.v[q] : T(0);
      zv.store(w, c);
    }
  }
  for (int64_t i = nc * W + t0; i < n; i += st) w[i] = ess[i] ? z[i] : T(0);
}

// ---------------------------------------------------------------------------
// Lanczos kernels on D^-1/2 J D^-1/2
// ---------------------------------------------------------------------------
template <typename T>
__global__ void k_lz_start(int64_t n, T* __restrict__ v, KrylovScalars* S, double* partials) {
  double a[1] = {0.0}, tot[1];
  GS_LOOP(i, n) {
    const double t = (double)i * 0.6180339887498949;
    const T vi = (T)(t - floor(t) - 0.5);
    v[i] = vi;
    a[0] += (double)vi * (double)vi;
  }
  block_sum_n<1>(a);
  if (grid_sum_n<1>(a, partials, &S->counter[6], tot)) S->rr = tot[0];
}
template <typename T>
__global__ void k_lz_scale0(int64_t n, T* __restrict__ v, T* __restrict__ vp, const KrylovScalars* S) {
  const T s = (T)(1.0 / sqrt(S->rr));
  GS_LOOP(i, n) {
    v[i] *= s;
    vp[i] = T(0);
  }
}
template <typename T>
__global__ void k_lz_pre(int64_t n, const T* __restrict__ v, const T* __restrict__ sd, T* __restrict__ tmp,
                         T* __restrict__ w, const uint8_t* __restrict__ ess) {
  GS_LOOP(i, n) {
    const T t = sd[i] * v[i];
    tmp[i] = t;
    w[i] = ess[i] ? t : T(0);
  }
}
template <typename T>
__global__ void k_lz_alpha(int64_t n, T* __restrict__ w, const T* __restrict__ sd, const T* __restrict__ v,
                           KrylovScalars* S, double* partials, int j) {
  double a[1] = {0.0}, tot[1];
  GS_LOOP(i, n) {
    const T wi = sd[i] * w[i];
    w[i] = wi;
    a[0] += (double)wi * (double)v[i];
  }
  block_sum_n<1>(a);
  if (grid_sum_n<1>(a, partials, &S->counter[6], tot)) S->lz[j] = tot[0];
}
template <typename T>
__global__ void k_lz_update(int64_t n, T* __restrict__ w, const T* __restrict__ v, const T* __restrict__ vp,
                            KrylovScalars* S, double* partials, int j) {
  const T a = (T)S->lz[j], b = (T)S->lz[kMaxLanczos + j];
  double s[1] = {0.0}, tot[1];
  GS_LOOP(i, n) {
    const T wi = w[i] - a * v[i] - b * vp[i];
    w[i] = wi;
    s[0] += (double)wi * (double)wi;
  }
  block_sum_n<1>(s);
  if (grid_sum_n<1>(s, partials, &S->counter[6], tot)) S->lz[kMaxLanczos + j + 1] = sqrt(tot[0]);
}
template <typename T>
__global__ void k_lz_shift(int64_t n, const T* __restrict__ w, T* __restrict__ v, T* __restrict__ vp,
                           const KrylovScalars* S, int j) {
  const double bn = S->lz[kMaxLanczos + j + 1];
  const T ib = bn > 0.0 ? (T)(1.0 / bn) : T(0);
  GS_LOOP(i, n) {
    vp[i] = v[i];
    v[i] = w[i] * ib;
  }
}

// ---------------------------------------------------------------------------
// refinement kernels (FP64 outer)
// ---------------------------------------------------------------------------
// r = b - r (r holds J x); returns ||r||^2 and ||b||^2 into S->rr, S->bb
__global__ void __launch_bounds__(kRedThreads)
    k_resid64(int64_t n, const double* __restrict__ b, double* __restrict__ r, KrylovScalars* S, double* partials) {
  double v[2] = {0.0, 0.0}, tot[2];
  GS_LOOP(i, n) {
    const double bi = b[i];
    const double ri = bi - r[i];
    r[i] = ri;
    v[0] += ri * ri;
    v[1] += bi * bi;
  }
  block_sum_n<2>(v);
  if (grid_sum_n<2>(v, partials, &S->counter[7], tot)) {
    S->rr = tot[0];
    S->bb = tot[1];
  }
}
__global__ void k_d2f_scaled(int64_t n, const double* __restrict__ r, float* __restrict__ rf, double s) {
  GS_LOOP(i, n) rf[i] = (float)(r[i] * s);
}
__global__ void k_axpy_f2d(int64_t n, const float* __restrict__ c, double* __restrict__ x, double s) {
  GS_LOOP(i, n) x[i] += s * (double)c[i];
}

// ---------------------------------------------------------------------------
// host drivers
// ---------------------------------------------------------------------------
static_assert(sizeof(KrylovScalars) <= 4096, "pinned scalar blocks are 4 KB");
cudaError_t ensure_scalars(hcop* h) {
  if (h->scal) return cudaSuccess;
  cudaError_t e = dmalloc(h, (void**)&h->scal, sizeof(KrylovScalars));
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(h->scal, 0, sizeof(KrylovScalars), h->stream);
  if (e != cudaSuccess) return e;
  h->hscal = static_cast<KrylovScalars*>(pinned_get(sizeof(KrylovScalars)));
  if (!h->hscal) return cudaErrorMemoryAllocation;
  const HexDev d = h->hexdev();
  const size_t np = (size_t)std::max(kRedBlocks, hex_apply_blocks(d)) * 4;
  return dmalloc(h, (void**)&h->partials, np * sizeof(double));
}

hc_status ensure_work(hcop* h, size_t bytes) {
  if (h->work_bytes >= bytes) return HC_OK;
  dfree(h, h->work);  // stream-ordered: queued work on the handle's stream finishes first
  h->work = nullptr;
  h->work_bytes = 0;
  cudaError_t e = dmalloc(h, &h->work, bytes);
  if (e != cudaSuccess) {
    h->err = std::string("work space allocation failed: ") + cudaGetErrorString(e);
    return HC_ENOMEM;
  }
  h->work_bytes = bytes;
  return HC_OK;
}

// largest eigenvalue of the symmetric tridiagonal (a, b) by Sturm bisection
static double tridiag_lmax(const std::vector<double>& a, const std::vector<double>& b) {
  const int m = (int)a.size();
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < m; ++i) {
    const double rad = (i > 0 ? std::fabs(b[i - 1]) : 0.0) + (i + 1 < m ? std::fabs(b[i]) : 0.0);
    lo = std::min(lo, a[i] - rad);
    hi = std::max(hi, a[i] + rad);
  }
  for (int it = 0; it < 200; ++it) {
    const double mid = 0.5 * (lo + hi);
    int below = 0;
    double q = 1.0;
    for (int i = 0; i < m; ++i) {
      q = a[i] - mid - (i > 0 ? b[i - 1] * b[i - 1] / q : 0.0);
      if (q == 0.0) q = 1e-300;
      if (q < 0.0) ++below;
    }
    if (below >= m) hi = mid;
    else lo = mid;
  }
  return hi;
}

template <typename T>
static const T* sd_of(hcop* h);
template <>
const double* sd_of<double>(hcop* h) {
  return h->sdinv;
}
template <>
const float* sd_of<float>(hcop* h) {
  return h->sdinvf;
}
template <typename T>
static const T* dinv_of(hcop* h);
template <>
const double* dinv_of<double>(hcop* h) {
  return h->dinv;
}
template <>
const float* dinv_of<float>(hcop* h) {
  return h->dinvf;
}
template <typename T>
static const T* fac_of(hcop* h);
template <>
const double* fac_of<double>(hcop* h) {
  return h->fac;
}
template <>
const float* fac_of<float>(hcop* h) {
  return h->facf;
}

template <typename T>
hc_status lanczos_device(hcop* h, int steps, double* lmax, T* wk) {
  if (steps < 2 || steps > kMaxLanczos) {
    h->err = "Lanczos steps must be in [2, 64]";
    return HC_EINVAL;
  }
  HC_CUDA_TRY(h, ensure_scalars(h));
  const int64_t n = h->ndof;
  cudaStream_t s = h->stream;
  const int64_t np = vstride(n);
  T *v = wk, *vp = wk + np, *w = wk + 2 * np, *tmp = wk + 3 * np;
  KrylovScalars* S = h->scal;
  const unsigned g = vgrid(n);
  const OpJ<T> op{h, fac_of<T>(h)};
  HC_CUDA_TRY(h, cudaMemsetAsync(S->lz, 0, sizeof(S->lz), s));
  k_lz_start<T><<<g, kRedThreads, 0, s>>>(n, v, S, h->partials);
  k_lz_scale0<T><<<g, kRedThreads, 0, s>>>(n, v, vp, S);
  for (int j = 0; j < steps; ++j) {
    k_lz_pre<T><<<g, kRedThreads, 0, s>>>(n, v, sd_of<T>(h), tmp, w, h->ess);
    HC_CUDA_TRY(h, op.apply(tmp, w, nullptr, nullptr, s));
    k_lz_alpha<T><<<g, kRedThreads, 0, s>>>(n, w, sd_of<T>(h), v, S, h->partials, j);
    k_lz_update<T><<<g, kRedThreads, 0, s>>>(n, w, v, vp, S, h->partials, j);
    k_lz_shift<T><<<g, kRedThreads, 0, s>>>(n, w, v, vp, S, j);
  }
  HC_CUDA_TRY(h, cudaGetLastError());
  HC_CUDA_TRY(h, cudaMemcpyAsync(h->hscal, S, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, s));
  HC_CUDA_TRY(h, cudaStreamSynchronize(s));
  std::vector<double> a, b;
  for (int j = 0; j < steps; ++j) {
    a.push_back(h->hscal->lz[j]);
    const double bj = h->hscal->lz[kMaxLanczos + j + 1];
    if (j + 1 < steps) b.push_back(bj);
    if (!(bj > 0.0)) break;  // invariant subspace found
  }
  b.resize(a.size() - 1);
  *lmax = tridiag_lmax(a, b);
  if (!std::isfinite(*lmax) || *lmax <= 0.0) {
    h->err = "Lanczos bound is not positive";
    return HC_BREAKDOWN;
  }
  return HC_OK;
}

template <typename T>
hc_status lanczos_device(hcop* h, int steps, double* lmax) {
  hc_status st = ensure_work(h, (size_t)4 * vstride(h->ndof) * sizeof(T));
  if (st != HC_OK) return st;
  return lanczos_device<T>(h, steps, lmax, (T*)h->work);
}
template hc_status lanczos_device<double>(hcop*, int, double*);
template hc_status lanczos_device<float>(hcop*, int, double*);

// Host callback of pcg_run at each batch boundary, after the scalars were
// read back into hs.  Returns kHookGoOn (stop or go on as hs says),
// kHookResumed (the callback changed the iterate and cleared S->done and
// hs->done: iterate on) or kHookStop.
enum { kHookGoOn = 0, kHookResumed = 1, kHookStop = 2 };
struct ChunkHook {
  virtual int at_batch(KrylovScalars* hs) = 0;
  virtual ~ChunkHook() = default;
};

// Preconditioned CG; wk holds 6 n-vectors of T.
template <typename T>
static hc_status pcg_run(hcop* h, const SolveCfg& cfg, const T* b, T* x, T* wk, int* iters, int* applies,
                         ChunkHook* hook = nullptr) {
  HC_CUDA_TRY(h, ensure_scalars(h));
  const int64_t n = h->ndof;
  cudaStream_t s = h->stream;
  KrylovScalars* S = h->scal;
  const int64_t np = vstride(n);
  T *r = wk, *p = wk + np, *q = wk + 2 * np, *z = wk + 3 * np, *dk = wk + 4 * np, *w = wk + 5 * np;
  const unsigned g = vgrid(n);
  const OpJ<T> op{h, fac_of<T>(h)};
  const T* dinv = dinv_of<T>(h);
  double* part = h->partials;
  int napply = 0;

  // scalars
  KrylovScalars* hs = h->hscal;
  std::memset(hs, 0, sizeof(KrylovScalars));
  hs->rtol2 = cfg.rtol * cfg.rtol;
  hs->atol2 = cfg.atol * cfg.atol;
  hs->maxit = cfg.maxit;
  HC_CUDA_TRY(h, cudaMemcpyAsync(S, hs, sizeof(KrylovScalars), cudaMemcpyHostToDevice, s));
  HC_CUDA_TRY(h, cudaMemsetAsync(p, 0, n * sizeof(T), s));

  const bool jac = cfg.precond == HC_PRECOND_JACOBI || cfg.precond == HC_PRECOND_NONE;
  const bool none = cfg.precond == HC_PRECOND_NONE;
  const bool aux = cfg.precond == HC_PRECOND_AUX;
  const bool amult = cfg.precond == HC_PRECOND_AUX_MULT;
  // z = C(r) for the Chebyshev preconditioner (and the smoother of AUX_MULT)
  double theta = 0, delta = 0, sigma1 = 0;
  std::vector<double> c1s, c2s;
  if (cfg.precond == HC_PRECOND_CHEBYSHEV || amult) {
    const double lmin = cfg.lmax / cfg.cheb_ratio;
    theta = 0.5 * (cfg.lmax + lmin);
    delta = 0.5 * (cfg.lmax - lmin);
    sigma1 = theta / delta;
    double rho = 1.0 / sigma1;
    for (int k = 1; k < cfg.cheb_degree; ++k) {
      const double rn = 1.0 / (2.0 * sigma1 - rho);
      c1s.push_back(rn * rho);
      c2s.push_back(2.0 * rn / delta);
      rho = rn;
    }
  }
  // Chebyshev smoothing of z toward J z = r (cfg.cheb_degree steps).  from0:
  // z = 0 on entry; else w = J z on entry.  init_last: leave w = (I - P) z for
  // the caller's next apply.  dk is stored only where a later step reads it.
  const bool vec = al16(r) && al16(z) && al16(dk) && al16(w) && al16(dinv) &&
                   (reinterpret_cast<uintptr_t>(h->ess) % (16 / sizeof(T))) == 0;
  const unsigned gw = vgrid((n + Chunk16<T>::W - 1) / Chunk16<T>::W);
  auto cheb_launch = [&](T c1, T c2, int f) {
    if (vec)
      k_cheb_step<T, true><<<gw, kRedThreads, 0, s>>>(n, r, dinv, z, dk, w, h->ess, c1, c2, f, S);
    else
      k_cheb_step<T, false><<<g, kRedThreads, 0, s>>>(n, r, dinv, z, dk, w, h->ess, c1, c2, f, S);
  };
  auto smooth = [&](bool from0, bool init_last) -> cudaError_t {
    const int deg = cfg.cheb_degree;
    for (int j = 0; j < deg; ++j) {
      if (j > 0) {
        cudaError_t e = op.apply(z, w, nullptr, nullptr, s);
        if (e != cudaSuccess) return e;
        ++napply;
      }
      int f = 0;
      if (j == 0 && from0) f |= kCbZ0;
      if (j == 1) f |= from0 ? kCbDkZ : kCbDk;
      if (j >= 2) f |= kCbDk;
      if (j + 1 < deg && (j >= 1 || !from0)) f |= kCbStoreDk;
      if (j + 1 < deg || init_last) f |= kCbInitW;
      const T c1 = j == 0 ? T(0) : (T)c1s[j - 1];
      const T c2 = j == 0 ? (T)(1.0 / theta) : (T)c2s[j - 1];
      cheb_launch(c1, c2, f);
    }
    return cudaGetLastError();
  };
  // AUX_MULT: z = S r; z += c G V G^T (r - J z); z += S (r - J z) with S the
  // Chebyshev-Jacobi polynomial: a symmetric multiplicative (smoother,
  // gradient-space correction, smoother) cycle, as AMS cycles are.
  auto aux_mult = [&]() -> cudaError_t {
    cudaError_t e = smooth(true, true);
    if (e != cudaSuccess) return e;
    if ((e = op.apply(z, w, nullptr, nullptr, s)) != cudaSuccess) return e;
    ++napply;
    if (vec)
      k_amul_t<T, true><<<gw, kRedThreads, 0, s>>>(n, r, w, dk, S);
    else
      k_amul_t<T, false><<<g, kRedThreads, 0, s>>>(n, r, w, dk, S);
    const float coef[4] = {kAuxMultWeight, 0.0f, 0.0f, 0.0f};
    if ((e = auxmg_apply<T, 1>(h, dk, nullptr, z, nullptr, coef, &S->done, s)) != cudaSuccess) return e;
    if (vec)
      k_init_w<T, true><<<gw, kRedThreads, 0, s>>>(n, z, w, h->ess, S);
    else
      k_init_w<T, false><<<g, kRedThreads, 0, s>>>(n, z, w, h->ess, S);
    if ((e = op.apply(z, w, nullptr, nullptr, s)) != cudaSuccess) return e;
    ++napply;
    return smooth(false, false);
  };
  // z = B r for the non-Jacobi preconditioners
  auto precond = [&](bool z_ready) -> cudaError_t {
    if (aux) {
      if (!z_ready) k_jz<T><<<g, kRedThreads, 0, s>>>(n, r, dinv, z, S);
      const float coef[4] = {1.0f, 0.0f, 0.0f, 0.0f};
      return auxmg_apply<T, 1>(h, r, nullptr, z, nullptr, coef, &S->done, s);
    }
    if (amult) return aux_mult();
    return smooth(true, false);
  };

  // r = b - J x
  HC_CUDA_TRY(h, init_masked<T>(n, h->ess, x, q, s));
  HC_CUDA_TRY(h, op.apply(x, q, nullptr, nullptr, s));
  ++napply;
  // no preconditioner: the Jacobi kernels with a null diagonal (z = r)
  const T* dj = none ? nullptr : dinv;
  if (jac) {
    k_pcg_setup<T, true><<<g, kRedThreads, 0, s>>>(n, b, q, r, dj, S, part);
    k_pcg_dir<T, true><<<g, kRedThreads, 0, s>>>(n, r, dj, p, q, h->ess, S, part);
  } else {
    k_pcg_setup<T, false><<<g, kRedThreads, 0, s>>>(n, b, q, r, dinv, S, part);
    HC_CUDA_TRY(h, precond(false));
    k_rz_beta<T><<<g, kRedThreads, 0, s>>>(n, r, z, 1, S, part);
    k_pcg_dir<T, false><<<g, kRedThreads, 0, s>>>(n, z, dinv, p, q, h->ess, S, part);
  }
  HC_CUDA_TRY(h, cudaGetLastError());

  // 16-byte kernels when every vector they touch is aligned (the work
  // vectors always are; x is the caller's)
  const bool wide = al16(x) && al16(dinv) && (reinterpret_cast<uintptr_t>(h->ess) % (16 / sizeof(T))) == 0;
  const unsigned gv = vgrid((n + Chunk16<T>::W - 1) / Chunk16<T>::W);
  const int chunk = 25;
  int launched = 0;
  for (;;) {
    for (int k = 0; k < chunk && launched < cfg.maxit; ++k, ++launched) {
      HC_CUDA_TRY(h, op.apply(p, q, S, part, s));
      ++napply;
      if (jac && wide) {
        k_pcg_update_v<T, true><<<gv, kRedThreads, 0, s>>>(n, x, r, p, q, dj, S, part, nullptr);
        k_pcg_dir_v<T, true><<<gv, kRedThreads, 0, s>>>(n, r, dj, p, q, h->ess, S, part);
      } else if (jac) {
        k_pcg_update<T, true><<<g, kRedThreads, 0, s>>>(n, x, r, p, q, dj, S, part);
        k_pcg_dir<T, true><<<g, kRedThreads, 0, s>>>(n, r, dj, p, q, h->ess, S, part);
      } else if (wide) {
        k_pcg_update_v<T, false><<<gv, kRedThreads, 0, s>>>(n, x, r, p, q, dinv, S, part, aux ? z : nullptr);
        HC_CUDA_TRY(h, precond(aux));
        k_rz_beta_v<T><<<gv, kRedThreads, 0, s>>>(n, r, z, 0, S, part);
        k_pcg_dir_v<T, false><<<gv, kRedThreads, 0, s>>>(n, z, dinv, p, q, h->ess, S, part);
      } else {
        k_pcg_update<T, false><<<g, kRedThreads, 0, s>>>(n, x, r, p, q, dinv, S, part, aux ? z : nullptr);
        HC_CUDA_TRY(h, precond(aux));
        k_rz_beta<T><<<g, kRedThreads, 0, s>>>(n, r, z, 0, S, part);
        k_pcg_dir<T, false><<<g, kRedThreads, 0, s>>>(n, z, dinv, p, q, h->ess, S, part);
      }
    }
    HC_CUDA_TRY(h, cudaGetLastError());
    HC_CUDA_TRY(h, cudaMemcpyAsync(hs, S, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, s));
    HC_CUDA_TRY(h, cudaStreamSynchronize(s));
    if (hook) {
      const int a = hook->at_batch(hs);
      if (a == kHookStop) break;
      if (a == kHookResumed && launched < cfg.maxit) continue;
    }
    if (hs->done || launched >= cfg.maxit) break;
  }
  *iters = hs->it;
  if (applies) *applies = napply;
  if (!hs->done) return HC_NOT_CONVERGED;
  return (hc_status)hs->status;
}

template <typename T>
hc_status pcg_device(hcop* h, const SolveCfg& cfg, const T* b, T* x, int* iters, int* applies,
                     double* unused) {
  (void)unused;
  hc_status st = ensure_work(h, (size_t)6 * vstride(h->ndof) * sizeof(T));
  if (st != HC_OK) return st;
  return pcg_run<T>(h, cfg, b, x, (T*)h->work, iters, applies);
}
template hc_status pcg_device<double>(hcop*, const SolveCfg&, const double*, double*, int*, int*, double*);
template hc_status pcg_device<float>(hcop*, const SolveCfg&, const float*, float*, int*, int*, double*);

// r64 = b - J x in FP64; ||r64||^2 and ||b||^2 read back to the host.
static hc_status resid64(hcop* h, const double* b, const double* x, double* r64, double* rn2, double* bn2) {
  const int64_t n = h->ndof;
  cudaStream_t s = h->stream;
  const OpJ<double> op64{h, h->fac};
  HC_CUDA_TRY(h, init_masked<double>(n, h->ess, x, r64, s));
  HC_CUDA_TRY(h, op64.apply(x, r64, nullptr, nullptr, s));
  k_resid64<<<vgrid(n), kRedThreads, 0, s>>>(n, b, r64, h->scal, h->partials);
  HC_CUDA_TRY(h, cudaGetLastError());
  HC_CUDA_TRY(h, cudaMemcpyAsync(h->hscal, h->scal, sizeof(KrylovScalars), cudaMemcpyDeviceToHost, s));
  HC_CUDA_TRY(h, cudaStreamSynchronize(s));
  *rn2 = h->hscal->rr;
  *bn2 = h->hscal->bb;
  return HC_OK;
}

// The FP32 inner solver's settings (Chebyshev bound estimated in FP32 once per handle).
static hc_status inner_cfg(hcop* h, const hc_solve_params* prm, double rtol, float* wk, SolveCfg* in) {
  in->precond = prm->precond;
  in->cheb_degree = prm->cheb_degree > 0 ? prm->cheb_degree : 2;
  in->cheb_ratio = prm->cheb_ratio > 0 ? prm->cheb_ratio : 30.0;
  in->rtol = rtol;
  in->atol = 0.0;
  in->lmax = prm->cheb_lmax;
  if ((in->precond == HC_PRECOND_CHEBYSHEV || in->precond == HC_PRECOND_AUX_MULT) && in->lmax <= 0) {
    if (h->lmax32 <= 0) {
      double lm = 0;
      const hc_status st = lanczos_device<float>(h, 20, &lm, wk);
      if (st != HC_OK) return st;
      h->lmax32 = 1.1 * lm;
    }
    in->lmax = h->lmax32;
  }
  return HC_OK;
}

// FP64 polish: PCG on J x = b from the current x, after the FP32 iteration
// reached its accuracy floor.  The work layout grows to
// r64 | 8n floats | 6n doubles (the FP64 PCG vectors, also Lanczos space).
// Returns the solve's status, judged on the true residual (rn2, bn2 out).
static hc_status polish64(hcop* h, const hc_solve_params* prm, const SolveCfg& in, const double* b, double* x,
                          double tol, int* iters, int* applies, int* outer, double* rn2, double* bn2) {
  const int64_t n = h->ndof;
  const int64_t np = vstride(n);
  hc_status st = ensure_work(h, (size_t)np * sizeof(double) + (size_t)8 * np * sizeof(float) +
                                    (size_t)6 * np * sizeof(double));
  if (st != HC_OK) return st;
  double* r64 = (double*)h->work;
  double* wk64 = (double*)((char*)h->work + (size_t)np * sizeof(double) + (size_t)8 * np * sizeof(float));
  SolveCfg c64;
  c64.precond = prm->precond;
  c64.cheb_degree = in.cheb_degree;
  c64.cheb_ratio = in.cheb_ratio;
  c64.lmax = prm->cheb_lmax;
  if ((c64.precond == HC_PRECOND_CHEBYSHEV || c64.precond == HC_PRECOND_AUX_MULT) && c64.lmax <= 0) {
    if (h->lmax64 <= 0) {
      double lm = 0;
      st = lanczos_device<double>(h, 20, &lm, wk64);
      if (st != HC_OK) return st;
      h->lmax64 = 1.1 * lm;
    }
    c64.lmax = h->lmax64;
  }
  // aim below the tolerance: the polish stops on its recursive residual,
  // the status is judged on the true residual.  Where the two drift apart
  // (operators at the FP64 floor), a restart from the current x -- whose
  // set-up recomputes b - J x -- is one FP64 refinement step: up to three
  // rounds, while each at least halves the true residual.
  c64.rtol = 0.5 * prm->rtol;
  c64.atol = 0.5 * prm->atol;
  double rn_prev = std::sqrt(*rn2);
  for (int round = 0; round < 3; ++round) {
    c64.maxit = prm->maxit - *iters;
    if (c64.maxit < 1) return HC_NOT_CONVERGED;
    int it = 0, ap = 0;
    const hc_status pst = pcg_run<double>(h, c64, b, x, wk64, &it, &ap);
    *iters += it;
    *applies += ap + 1;
    ++*outer;
    if (pst == HC_ECUDA || pst == HC_ENOMEM) return pst;
    st = resid64(h, b, x, r64, rn2, bn2);
    if (st != HC_OK) return st;
    const double rn = std::sqrt(*rn2);
    if (!std::isfinite(rn)) return HC_BREAKDOWN;
    if (pst == HC_BREAKDOWN) return pst;
    if (rn <= tol) return HC_OK;
    if (rn > 0.5 * rn_prev) break;
    rn_prev = rn;
  }
  return HC_NOT_CONVERGED;
}

static void fill_info(hc_solve_info* info, hc_status result, int iters, int outer, int applies, double rn2,
                      double bn2, double lmax) {
  if (!info) return;
  info->status = result;
  info->iterations = iters;
  info->outer_iterations = outer;
  info->applies = applies;
  const double bn = std::sqrt(bn2);
  info->rel_residual = bn > 0 ? std::sqrt(rn2) / bn : std::sqrt(rn2);
  info->lmax = lmax;
}

// FP32 inner PCG inside FP64 iterative refinement.
hc_status mixed_device(hcop* h, const hc_solve_params* prm, const double* b, double* x, hc_solve_info* info) {
  const int64_t n = h->ndof;
  // layout: r64 (n doubles) | rf, cf (2n floats) | 6n floats of PCG work
  const int64_t np = vstride(n);
  const size_t bytes = (size_t)np * sizeof(double) + (size_t)8 * np * sizeof(float);
  hc_status st = ensure_work(h, bytes);
  if (st != HC_OK) return st;
  HC_CUDA_TRY(h, ensure_scalars(h));
  double* r64 = (double*)h->work;
  float* rf = (float*)(r64 + np);
  float* cf = rf + np;
  float* wk = cf + np;
  cudaStream_t s = h->stream;
  const unsigned g = vgrid(n);
  int applies = 0, iters = 0, outer = 0;

  SolveCfg in;
  st = inner_cfg(h, prm, prm->inner_rtol > 0 ? prm->inner_rtol : 1e-4, wk, &in);
  if (st != HC_OK) return st;
  const int max_outer = prm->max_outer > 0 ? prm->max_outer : 50;

  double rn2 = 0, bn2 = 0;
  st = resid64(h, b, x, r64, &rn2, &bn2);
  if (st != HC_OK) return st;
  ++applies;
  const double bn = std::sqrt(bn2);
  const double tol = std::max(prm->rtol * bn, prm->atol);
  hc_status result = HC_NOT_CONVERGED;
  // A refinement step that no longer cuts the FP64 residual by 4x has hit the
  // FP32 accuracy floor of this operator (kappa eps_32 ~ 1 on its smooth
  // modes): stop refining and finish with FP64 PCG from the current x.
  bool stalled = false;
  double rn_prev = 0.0;
  const int inner_cap = std::max(100, prm->maxit / 4);
  while (true) {
    const double rn = std::sqrt(rn2);
    if (!std::isfinite(rn)) {
      result = HC_BREAKDOWN;
      break;
    }
    if (rn <= tol) {
      result = HC_OK;
      break;
    }
    if (outer >= max_outer || iters >= prm->maxit) break;
    if (outer >= 2 && rn > 0.25 * rn_prev) {
      stalled = true;
      break;
    }
    rn_prev = rn;
    ++outer;
    k_d2f_scaled<<<g, kRedThreads, 0, s>>>(n, r64, rf, 1.0 / rn);
    HC_CUDA_TRY(h, cudaMemsetAsync(cf, 0, n * sizeof(float), s));
    in.maxit = std::min(prm->maxit - iters, inner_cap);
    int it = 0, ap = 0;
    hc_status ist = pcg_run<float>(h, in, rf, cf, wk, &it, &ap);
    iters += it;
    applies += ap;
    if (ist == HC_BREAKDOWN || ist == HC_ECUDA || ist == HC_ENOMEM) {
      result = ist;
      break;
    }
    k_axpy_f2d<<<g, kRedThreads, 0, s>>>(n, cf, x, rn);
    HC_CUDA_TRY(h, cudaGetLastError());
    st = resid64(h, b, x, r64, &rn2, &bn2);
    if (st != HC_OK) return st;
    ++applies;
  }
  if (stalled && iters < prm->maxit)
    result = polish64(h, prm, in, b, x, tol, &iters, &applies, &outer, &rn2, &bn2);
  if (result == HC_ECUDA || result == HC_ENOMEM) return result;
  fill_info(info, result, iters, outer, applies, rn2, bn2, in.lmax);
  return result;
}

// S->rr = rr (the replaced residual's norm); the iteration goes on.
__global__ void k_resume(KrylovScalars* S, double rr) {
  S->rr = rr;
  S->done = 0;
  S->status = HC_NOT_CONVERGED;
}

// One FP32 PCG with FP64 residual replacement and grouped solution updates
// (H. A. van der Vorst and Q. Ye, "Residual replacement strategies for Krylov
// subspace iterative methods for the convergence of true residuals", SIAM J.
// Sci. Comput. 22 (2000) 835-852; used for mixed precision as the "reliable
// updates" of M. A. Clark et al., Comput. Phys. Commun. 181 (2010) 1517-1528).
// At a batch boundary where the FP32 recursive residual fell by `delta` since
// the last replacement, or met the tolerance: the FP32 correction (scaled by
// the initial residual norm) is added to the FP64 solution, b - J x is
// computed in FP64 and replaces the FP32 recursive residual.  The search
// direction and r.z are kept: unlike iterative refinement, the Krylov space
// is not restarted.  Two replacements in a row that do not halve the true
// residual mark the FP32 accuracy floor of the operator.
struct ReplaceHook : ChunkHook {
  hcop* h;
  const double* b;
  double* x;
  double* r64;
  float* rp;  // the FP32 PCG's residual vector
  float* cf;  // the FP32 correction since the last replacement
  double scale, tol, delta2, rr_last, rn_prev;
  int slow = 0, replacements = 0, applies = 0, since = 0;
  bool converged = false, stalled = false;
  bool pending = true;  // cf holds a correction not yet added to x
  hc_status err = HC_OK;
  double rn2 = 0, bn2 = 0;

  int at_batch(KrylovScalars* hs) override {
    if (hs->done && hs->status == HC_BREAKDOWN) return kHookGoOn;
    // due: converged or capped, the recursive residual fell by delta, or 8
    // batches (200 iterations) without that (an FP32 iteration that stopped
    // converging is caught by the stall test below)
    if (!hs->done && !(hs->rr <= delta2 * rr_last) && ++since < 8) return kHookGoOn;
    since = 0;
    const int64_t n = h->ndof;
    cudaStream_t s = h->stream;
    const unsigned g = vgrid(n);
    k_axpy_f2d<<<g, kRedThreads, 0, s>>>(n, cf, x, scale);
    cudaError_t e = cudaMemsetAsync(cf, 0, n * sizeof(float), s);
    if (e != cudaSuccess) {
      h->err = cudaGetErrorString(e);
      err = HC_ECUDA;
      return kHookStop;
    }
    err = resid64(h, b, x, r64, &rn2, &bn2);
    if (err != HC_OK) return kHookStop;
    pending = false;
    ++applies;
    ++replacements;
    const double rn = std::sqrt(rn2);
    if (!std::isfinite(rn)) {
      err = HC_BREAKDOWN;
      return kHookStop;
    }
    if (rn <= tol) {
      converged = true;
      return kHookStop;
    }
    if (hs->done && hs->it >= hs->maxit) return kHookStop;
    slow = rn > 0.5 * rn_prev ? slow + 1 : 0;
    rn_prev = rn;
    if (slow >= 2) {
      stalled = true;
      return kHookStop;
    }
    k_d2f_scaled<<<g, kRedThreads, 0, s>>>(n, r64, rp, 1.0 / scale);
    const double rr = rn2 / (scale * scale);
    k_resume<<<1, 1, 0, s>>>(h->scal, rr);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
      h->err = cudaGetErrorString(e);
      err = HC_ECUDA;
      return kHookStop;
    }
    pending = true;
    hs->rr = rr;
    hs->done = 0;
    hs->status = HC_NOT_CONVERGED;
    rr_last = rr;
    return kHookResumed;
  }
};

hc_status mixed_rr_device(hcop* h, const hc_solve_params* prm, const double* b, double* x, hc_solve_info* info) {
  const int64_t n = h->ndof;
  // layout: r64 (n doubles) | rf, cf (2n floats) | 6n floats of PCG work (r first)
  const int64_t np = vstride(n);
  const size_t bytes = (size_t)np * sizeof(double) + (size_t)8 * np * sizeof(float);
  hc_status st = ensure_work(h, bytes);
  if (st != HC_OK) return st;
  HC_CUDA_TRY(h, ensure_scalars(h));
  double* r64 = (double*)h->work;
  float* rf = (float*)(r64 + np);
  float* cf = rf + np;
  float* wk = cf + np;
  cudaStream_t s = h->stream;
  int applies = 0, iters = 0, outer = 0;

  double rn2 = 0, bn2 = 0;
  st = resid64(h, b, x, r64, &rn2, &bn2);
  if (st != HC_OK) return st;
  ++applies;
  const double rn0 = std::sqrt(rn2), bn = std::sqrt(bn2);
  const double tol = std::max(prm->rtol * bn, prm->atol);
  SolveCfg in;
  // the FP32 stopping test, on the recursive residual in units of ||r0||
  st = inner_cfg(h, prm, rn0 > 0 ? 0.5 * tol / rn0 : 0.0, wk, &in);
  if (st != HC_OK) return st;
  if (!std::isfinite(rn0)) {
    fill_info(info, HC_BREAKDOWN, 0, 0, applies, rn2, bn2, in.lmax);
    return HC_BREAKDOWN;
  }
  if (rn0 <= tol) {
    fill_info(info, HC_OK, 0, 0, applies, rn2, bn2, in.lmax);
    return HC_OK;
  }
  const double delta = prm->inner_rtol > 0 ? std::min(prm->inner_rtol, 0.5) : 0.1;
  ReplaceHook hk;
  hk.h = h;
  hk.b = b;
  hk.x = x;
  hk.r64 = r64;
  hk.rp = wk;
  hk.cf = cf;
  hk.scale = rn0;
  hk.tol = tol;
  hk.delta2 = delta * delta;
  hk.rr_last = 1.0;
  hk.rn_prev = rn0;
  k_d2f_scaled<<<vgrid(n), kRedThreads, 0, s>>>(n, r64, rf, 1.0 / rn0);
  HC_CUDA_TRY(h, cudaMemsetAsync(cf, 0, n * sizeof(float), s));
  in.maxit = prm->maxit;
  int it = 0, ap = 0;
  const hc_status ist = pcg_run<float>(h, in, rf, cf, wk, &it, &ap, &hk);
  iters += it;
  applies += ap + hk.applies;
  outer = hk.replacements;
  if (hk.err != HC_OK) {
    if (hk.err == HC_ECUDA || hk.err == HC_ENOMEM) return hk.err;
    fill_info(info, hk.err, iters, outer, applies, hk.rn2, hk.bn2, in.lmax);
    return hk.err;
  }
  if (ist == HC_ECUDA || ist == HC_ENOMEM) return ist;
  rn2 = hk.rn2;
  bn2 = hk.bn2;
  if (hk.pending) {
    // the FP32 correction since the last replacement (iteration cap, breakdown)
    k_axpy_f2d<<<vgrid(n), kRedThreads, 0, s>>>(n, cf, x, rn0);
    HC_CUDA_TRY(h, cudaGetLastError());
    st = resid64(h, b, x, r64, &rn2, &bn2);
    if (st != HC_OK) return st;
    ++applies;
  }
  hc_status result = HC_NOT_CONVERGED;
  if (!std::isfinite(std::sqrt(rn2))) result = HC_BREAKDOWN;
  else if (std::sqrt(rn2) <= tol) result = HC_OK;
  else if (ist == HC_BREAKDOWN) result = HC_BREAKDOWN;
  else if (hk.stalled && iters < prm->maxit)
    result = polish64(h, prm, in, b, x, tol, &iters, &applies, &outer, &rn2, &bn2);
  if (result == HC_ECUDA || result == HC_ENOMEM) return result;
  fill_info(info, result, iters, outer, applies, rn2, bn2, in.lmax);
  return result;
}

double vec_norm2_host(hcop* h, const double* x, int64_t n) {
  (void)h;
  (void)x;
  (void)n;
  return 0.0;
}

}  // namespace hc

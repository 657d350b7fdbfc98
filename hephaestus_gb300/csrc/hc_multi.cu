// hc_multi.cu -- block PCG for R right-hand sides sharing every operator
// application (the batched element-matrix apply of tet meshes, or R applies
// on hex grids), with per-right-hand-side alpha, beta, dots and stopping
// tests, in FP64 or as FP32 inner block PCG inside FP64 iterative refinement.
//
// Vectors are row-major [dof][rhs] (R in {1, 2, 4, 8, 16, 32}).  Reductions are
// segmented by right-hand side and deterministic: with a grid stride that is a
// multiple of R every thread touches a single right-hand side (tid % R); warp
// shuffles over lane offsets >= R, fixed-order block and last-block grid sums.
// Preconditioner: Jacobi (the operator diagonal), or Jacobi plus the
// gradient-space AMG correction of hc_tetaux.cu applied to all columns at once.
// A converged right-hand side is frozen (alpha = 0, direction zeroed) while the
// others continue.
#include <algorithm>
#include <functional>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "hc_internal.h"

namespace hc {

constexpr int kMaxRhs = 32;
constexpr int kMThreads = 256;
constexpr int kMBlocks = 1216;  // 8 x 152 SMs: 64 resident warps per SM

struct MScalars {
  double rz[kMaxRhs], rr[kMaxRhs], bb[kMaxRhs], tol2[kMaxRhs], alpha[kMaxRhs], beta[kMaxRhs];
  int done[kMaxRhs], status[kMaxRhs], it[kMaxRhs];
  int all_done, maxit, iter;
  double rtol2, atol2;
  unsigned int counter[4];
};
static_assert(sizeof(MScalars) <= 4096, "pinned scalar blocks are 4 KB");

// Segmented (per right-hand side) sum of NV x W values per thread; thread t
// owns the W columns (W t) % R .. + W - 1 (W = 1: rhs t % R).  Returns, on
// thread 0 of the last block, the grid totals in shared memory (total of value
// k for rhs r at [k * kMaxRhs + r]); nullptr elsewhere.
template <int NV, int W>
__device__ const double* mgrid_sum(double (&v)[NV][W], int R, double* partials, unsigned int* counter) {
  __shared__ double sh[NV][kMThreads / 32][kMaxRhs];
  __shared__ double tot[NV * kMaxRhs];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int G = R / W;  // lanes l and l + G own the same columns
#pragma unroll
  for (int k = 0; k < NV; ++k)
#pragma unroll
    for (int q = 0; q < W; ++q)
      for (int o = 16; o >= G; o >>= 1) v[k][q] += __shfl_down_sync(0xffffffffu, v[k][q], o);
  if (lane < G)
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
      for (int q = 0; q < W; ++q) sh[k][w][W * lane + q] = v[k][q];
  __syncthreads();
  // block partial per rhs, written by thread r < R
  if (threadIdx.x < R) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int i = 0; i < kMThreads / 32; ++i) s += sh[k][i][threadIdx.x];
      partials[((size_t)k * R + threadIdx.x) * gridDim.x + blockIdx.x] = s;
    }
    __threadfence();  // the partial writers publish before the ticket
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(counter, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return nullptr;
  __threadfence();
  // one warp per (value, rhs) pair: lanes stride over the block partials in a
  // fixed order, then a fixed shuffle tree
  for (int pr = w; pr < NV * R; pr += kMThreads / 32) {
    const int k = pr / R, rr = pr % R;
    const volatile double* src = partials + ((size_t)k * R + rr) * gridDim.x;
    double s = 0.0;
    for (unsigned int b = lane; b < gridDim.x; b += 32) s += src[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) tot[k * kMaxRhs + rr] = s;
  }
  __syncthreads();
  if (threadIdx.x != 0) return nullptr;
  *counter = 0u;
  return tot;
}

// Loop over this thread's entries, W consecutive ones at a time (i = dof * R +
// rhs; W = 4 for R >= 4: 128-bit accesses).  The grid stride is a multiple of
// R, so a thread keeps its columns K_COL .. K_COL + W - 1, K_COL = (W tid) % R,
// and the dof is i >> lgR (R a power of two).
#define M_THREAD(R, W)                                                       \
  const int64_t m_t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;       \
  const int64_t m_stride = (int64_t)gridDim.x * blockDim.x * (W);            \
  const int K_COL = (int)((m_t0 * (W)) & ((R) - 1));                         \
  const int m_lg = __ffs(R) - 1;                                             \
  (void)K_COL;                                                               \
  (void)m_lg
#define M_LOOP(i, n, R, W) _Pragma("unroll 4") for (int64_t i = m_t0 * (W); i < (n) * (R); i += m_stride)

template <int W>
__device__ __forceinline__ void mld(const float* __restrict__ p, float (&o)[W]) {
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
__device__ __forceinline__ void mld(const double* __restrict__ p, double (&o)[W]) {
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
__device__ __forceinline__ void mst(float* __restrict__ p, const float (&o)[W]) {
  if constexpr (W == 4)
    *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
  else
    *p = o[0];
}
template <int W>
__device__ __forceinline__ void mst(double* __restrict__ p, const double (&o)[W]) {
  if constexpr (W == 4) {
    *reinterpret_cast<double2*>(p) = make_double2(o[0], o[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(o[2], o[3]);
  } else {
    *p = o[0];
  }
}

// Per-thread partial sums in the vectors' precision (a thread sums at most a
// few hundred terms: n R / (W x 311,296 threads)), combined across threads,
// blocks and the grid in FP64.  GB300's FP64 rate is a small fraction of its
// FP32 rate, so FP32 vectors must not do per-element FP64 work.
template <typename T, int NV, int W>
struct MAcc {
  double v[NV][W];
  T a[NV][W];
  __device__ MAcc() {
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
      for (int q = 0; q < W; ++q) {
        v[k][q] = 0.0;
        a[k][q] = T(0);
      }
  }
  __device__ __forceinline__ void flush() {
#pragma unroll
    for (int k = 0; k < NV; ++k)
#pragma unroll
      for (int q = 0; q < W; ++q) {
        v[k][q] += (double)a[k][q];
        a[k][q] = T(0);
      }
  }
  __device__ __forceinline__ void step() {}
};

// r = b - q; bb, rr, rz per rhs; tolerances and the first stopping test
template <typename T, int W>
__global__ void __launch_bounds__(kMThreads)
    k_m_setup(int64_t n, int R, const T* __restrict__ b, const T* __restrict__ q, T* __restrict__ r,
              const T* __restrict__ dinv, MScalars* S, double* partials) {
  M_THREAD(R, W);
  MAcc<T, 3, W> acc;
  M_LOOP(i, n, R, W) {
    T bv[W], qv[W];
    mld<W>(b + i, bv);
    mld<W>(q + i, qv);
    const T di = dinv[i >> m_lg];
#pragma unroll
    for (int w = 0; w < W; ++w) {
      qv[w] = bv[w] - qv[w];
      acc.a[0][w] += bv[w] * bv[w];
      acc.a[1][w] += qv[w] * qv[w];
      acc.a[2][w] += qv[w] * qv[w] * di;
    }
    mst<W>(r + i, qv);
    acc.step();
  }
  acc.flush();
  if (const double* tot = mgrid_sum<3, W>(acc.v, R, partials, &S->counter[0])) {
    int all = 1;
    for (int k = 0; k < R; ++k) {
      S->bb[k] = tot[k];
      S->rr[k] = tot[kMaxRhs + k];
      S->rz[k] = tot[2 * kMaxRhs + k];
      S->tol2[k] = fmax(S->rtol2 * tot[k], S->atol2);
      S->beta[k] = 0.0;
      S->it[k] = 0;
      S->status[k] = HC_NOT_CONVERGED;
      S->done[k] = 0;
      if (!isfinite(tot[k]) || !isfinite(tot[kMaxRhs + k])) {
        S->done[k] = 1;
        S->status[k] = HC_BREAKDOWN;
      } else if (tot[kMaxRhs + k] <= S->tol2[k]) {
        S->done[k] = 1;
        S->status[k] = HC_OK;
      }
      all &= S->done[k];
    }
    S->all_done = all;
    S->iter = 0;
  }
}

// p = z + beta p with z = B r (z == nullptr: z = D^-1 r; p = 0 for a stopped rhs); q = (I - P) p
template <typename T, int W>
__global__ void __launch_bounds__(kMThreads)
    k_m_dir(int64_t n, int R, const T* __restrict__ r, const T* __restrict__ z, const T* __restrict__ dinv,
            T* __restrict__ p, T* __restrict__ q, const uint8_t* __restrict__ ess, const MScalars* S) {
  if (S->all_done) return;
  M_THREAD(R, W);
  T beta[W];
  bool stop[W];
#pragma unroll
  for (int w = 0; w < W; ++w) {
    stop[w] = S->done[K_COL + w] != 0;
    beta[w] = (T)S->beta[K_COL + w];
  }
  M_LOOP(i, n, R, W) {
    const int64_t d = i >> m_lg;
    T zv[W], pv[W];
    if (z) {
      mld<W>(z + i, zv);
    } else {
      mld<W>(r + i, zv);
      const T di = dinv[d];
#pragma unroll
      for (int w = 0; w < W; ++w) zv[w] *= di;
    }
    mld<W>(p + i, pv);
#pragma unroll
    for (int w = 0; w < W; ++w) pv[w] = stop[w] ? T(0) : zv[w] + beta[w] * pv[w];
    mst<W>(p + i, pv);
    if (!ess[d]) {
#pragma unroll
      for (int w = 0; w < W; ++w) pv[w] = T(0);
    }
    mst<W>(q + i, pv);
  }
}

// alpha = rz / p.q per rhs (q = J p)
template <typename T, int W>
__global__ void __launch_bounds__(kMThreads)
    k_m_alpha(int64_t n, int R, const T* __restrict__ p, const T* __restrict__ q, MScalars* S, double* partials) {
  if (S->all_done) return;
  M_THREAD(R, W);
  MAcc<T, 1, W> acc;
  M_LOOP(i, n, R, W) {
    T pv[W], qv[W];
    mld<W>(p + i, pv);
    mld<W>(q + i, qv);
#pragma unroll
    for (int w = 0; w < W; ++w) acc.a[0][w] += pv[w] * qv[w];
    acc.step();
  }
  acc.flush();
  if (const double* tot = mgrid_sum<1, W>(acc.v, R, partials, &S->counter[1])) {
    for (int k = 0; k < R; ++k) {
      if (S->done[k]) {
        S->alpha[k] = 0.0;
        continue;
      }
      const double pq = tot[k];
      if (!(pq > 0.0) || !isfinite(pq)) {
        S->alpha[k] = 0.0;
        S->done[k] = 1;
        S->status[k] = HC_BREAKDOWN;
      } else {
        S->alpha[k] = S->rz[k] / pq;
      }
    }
  }
}

// x += alpha p; r -= alpha q; rr per rhs and stopping tests; jac: rz = r.D^-1 r and beta
template <typename T, int W>
__global__ void __launch_bounds__(kMThreads)
    k_m_update(int64_t n, int R, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
               const T* __restrict__ q, const T* __restrict__ dinv, int jac, MScalars* S, double* partials) {
  if (S->all_done) return;
  M_THREAD(R, W);
  T a[W];
#pragma unroll
  for (int w = 0; w < W; ++w) a[w] = (T)S->alpha[K_COL + w];
  MAcc<T, 2, W> acc;
  M_LOOP(i, n, R, W) {
    T xv[W], rv[W], pv[W], qv[W];
    mld<W>(x + i, xv);
    mld<W>(r + i, rv);
    mld<W>(p + i, pv);
    mld<W>(q + i, qv);
    const T di = jac ? dinv[i >> m_lg] : T(0);
#pragma unroll
    for (int w = 0; w < W; ++w) {
      xv[w] += a[w] * pv[w];
      rv[w] -= a[w] * qv[w];
      acc.a[0][w] += rv[w] * rv[w];
      acc.a[1][w] += rv[w] * rv[w] * di;
    }
    mst<W>(x + i, xv);
    mst<W>(r + i, rv);
    acc.step();
  }
  acc.flush();
  if (const double* tot = mgrid_sum<2, W>(acc.v, R, partials, &S->counter[2])) {
    S->iter += 1;
    int all = 1;
    for (int k = 0; k < R; ++k) {
      if (!S->done[k]) {
        S->it[k] += 1;
        S->rr[k] = tot[k];
        if (jac) {
          S->beta[k] = tot[kMaxRhs + k] / S->rz[k];
          S->rz[k] = tot[kMaxRhs + k];
        }
        if (!isfinite(tot[k])) {
          S->done[k] = 1;
          S->status[k] = HC_BREAKDOWN;
        } else if (tot[k] <= S->tol2[k]) {
          S->done[k] = 1;
          S->status[k] = HC_OK;
        } else if (S->it[k] >= S->maxit) {
          S->done[k] = 1;
          S->status[k] = HC_NOT_CONVERGED;
        }
      }
      all &= S->done[k];
    }
    S->all_done = all;
  }
}

// rz = r.z per rhs; first: beta = 0, else beta = rz_new / rz_old (columns still running)
template <typename T, int W>
__global__ void __launch_bounds__(kMThreads)
    k_m_rz(int64_t n, int R, const T* __restrict__ r, const T* __restrict__ z, int first, MScalars* S,
           double* partials) {
  if (S->all_done) return;
  M_THREAD(R, W);
  MAcc<T, 1, W> acc;
  M_LOOP(i, n, R, W) {
    T rv[W], zv[W];
    mld<W>(r + i, rv);
    mld<W>(z + i, zv);
#pragma unroll
    for (int w = 0; w < W; ++w) acc.a[0][w] += rv[w] * zv[w];
    acc.step();
  }
  acc.flush();
  if (const double* tot = mgrid_sum<1, W>(acc.v, R, partials, &S->counter[1])) {
    for (int k = 0; k < R; ++k) {
      if (first) {
        S->rz[k] = tot[k];
        S->beta[k] = 0.0;
      } else if (!S->done[k]) {
        S->beta[k] = tot[k] / S->rz[k];
        S->rz[k] = tot[k];
      }
    }
  }
}

// FP64 residual of the refinement: r = b - r (r holds J x); |r|^2 and |b|^2 per rhs
__global__ void __launch_bounds__(kMThreads)
    k_m_resid64(int64_t n, int R, const double* __restrict__ b, double* __restrict__ r, MScalars* S,
                double* partials) {
  M_THREAD(R, 1);
  double v[2][1] = {{0}, {0}};
  M_LOOP(i, n, R, 1) {
    const double bi = b[i], ri = bi - r[i];
    r[i] = ri;
    v[0][0] += ri * ri;
    v[1][0] += bi * bi;
  }
  if (const double* tot = mgrid_sum<2, 1>(v, R, partials, &S->counter[3]))
    for (int k = 0; k < R; ++k) {
      S->rr[k] = tot[k];
      S->bb[k] = tot[kMaxRhs + k];
    }
}
// rf = r / |r_k| per column (FP32); c = 0
__global__ void __launch_bounds__(kMThreads)
    k_m_d2f(int64_t n, int R, const double* __restrict__ r, const double* __restrict__ inv, float* __restrict__ rf,
            float* __restrict__ c) {
  M_THREAD(R, 1);
  const double s = inv[K_COL];
  M_LOOP(i, n, R, 1) {
    rf[i] = (float)(r[i] * s);
    c[i] = 0.0f;
  }
}
// x += |r_k| c per column
__global__ void __launch_bounds__(kMThreads)
    k_m_axpy(int64_t n, int R, const float* __restrict__ c, const double* __restrict__ scale, double* __restrict__ x) {
  M_THREAD(R, 1);
  const double s = scale[K_COL];
  M_LOOP(i, n, R, 1) x[i] += s * (double)c[i];
}

static inline unsigned mgrid(int64_t n, int R, int W = 1) {
  // the grid stride (W x blocks x threads) is a multiple of R: fixed columns per thread
  const int64_t b = (n * R / W + kMThreads - 1) / kMThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, kMBlocks));
}
// launch kernel<T, W> with W = 4 (128-bit accesses) when R >= 4
#define M_LAUNCH(kern, ...)                                                    \
  do {                                                                        \
    if (R >= 4)                                                               \
      kern<T, 4><<<mgrid(n, R, 4), kMThreads, 0, s>>>(__VA_ARGS__);           \
    else                                                                      \
      kern<T, 1><<<mgrid(n, R, 1), kMThreads, 0, s>>>(__VA_ARGS__);           \
  } while (0)

// Y = J X for R right-hand sides (masked): tets batch the element matrices,
// hex grids apply column by column
template <typename T>
static cudaError_t multi_apply(hcop* h, int R, const T* X, T* Y, cudaStream_t s);
template <>
cudaError_t multi_apply<double>(hcop* h, int R, const double* X, double* Y, cudaStream_t s) {
  cudaError_t e = init_masked_multi<double>(h->ndof, R, h->ess, X, Y, s);
  if (e != cudaSuccess) return e;
  return tet_apply_launch<double>(h, h->tetK64, X, Y, R, true, 1.0, nullptr, s);
}
template <>
cudaError_t multi_apply<float>(hcop* h, int R, const float* X, float* Y, cudaStream_t s) {
  cudaError_t e = init_masked_multi<float>(h->ndof, R, h->ess, X, Y, s);
  if (e != cudaSuccess) return e;
  return tet_apply_launch<float>(h, h->tetK32, X, Y, R, true, 1.0, nullptr, s);
}

struct MultiWork {
  MScalars* S = nullptr;
  MScalars* hS = nullptr;
  double* partials = nullptr;
  double* col = nullptr;  // 2 x kMaxRhs per-column scales (device)
  void* vec = nullptr;
  size_t vec_bytes = 0;
};

static MultiWork* mwork(hcop* h) {
  if (!h->mwork) h->mwork = new MultiWork();
  return static_cast<MultiWork*>(h->mwork);
}

void multi_free(hcop* h) {
  MultiWork* w = static_cast<MultiWork*>(h->mwork);
  if (!w) return;
  dfree(h, w->S);
  dfree(h, w->partials);
  dfree(h, w->col);
  dfree(h, w->vec);
  pinned_put(w->hS);
  delete w;
  h->mwork = nullptr;
}

static hc_status multi_prepare(hcop* h, size_t vec_bytes) {
  MultiWork* w = mwork(h);
  if (!w->S) {
    if (dmalloc(h, (void**)&w->S, sizeof(MScalars)) != cudaSuccess ||
        dmalloc(h, (void**)&w->partials, (size_t)3 * kMaxRhs * kMBlocks * sizeof(double)) != cudaSuccess ||
        dmalloc(h, (void**)&w->col, 2 * kMaxRhs * sizeof(double)) != cudaSuccess ||
        !(w->hS = static_cast<MScalars*>(pinned_get(sizeof(MScalars))))) {
      h->err = "multi-RHS work space allocation failed";
      return HC_ENOMEM;
    }
    HC_CUDA_TRY(h, cudaMemsetAsync(w->S, 0, sizeof(MScalars), h->stream));
  }
  if (w->vec_bytes < vec_bytes) {
    dfree(h, w->vec);
    w->vec = nullptr;
    w->vec_bytes = 0;
    if (dmalloc(h, &w->vec, vec_bytes) != cudaSuccess) {
      h->err = "multi-RHS work vectors allocation failed";
      return HC_ENOMEM;
    }
    w->vec_bytes = vec_bytes;
  }
  return HC_OK;
}

// Block PCG on J X = B (X: initial guess); wk holds r, p, q (and z with aux): 3 (4) n R of T.
// Host callback of mpcg_run at each batch boundary (after the scalars were
// read into hs): go on as hs says, iterate on after the callback changed the
// iterate and the device scalars (and hs), or stop.
enum { kMHookGoOn = 0, kMHookResumed = 1, kMHookStop = 2 };
struct MultiHook {
  virtual int at_batch(MScalars* hs) = 0;
  virtual ~MultiHook() = default;
};

template <typename T>
static hc_status mpcg_run(hcop* h, int R, double rtol, double atol, int maxit, const T* B, T* X, T* wk,
                          const T* dinv, bool aux, MultiHook* hook) {
  MultiWork* w = mwork(h);
  cudaStream_t s = h->stream;
  const int64_t n = h->ndof;
  T *r = wk, *p = wk + n * R, *q = wk + 2 * n * R;
  T* z = aux ? wk + 3 * n * R : nullptr;
  const int* all_done = &w->S->all_done;
  auto precond = [&](int first) -> hc_status {
    if (!aux) return HC_OK;
    HC_CUDA_TRY(h, tetaux_apply<T>(h, R, r, z, dinv, all_done, s));
    M_LAUNCH(k_m_rz, n, R, r, z, first, w->S, w->partials);
    return HC_OK;
  };
  MScalars* hs = w->hS;
  std::memset(hs, 0, sizeof(MScalars));
  hs->rtol2 = rtol * rtol;
  hs->atol2 = atol * atol;
  hs->maxit = maxit;
  HC_CUDA_TRY(h, cudaMemcpyAsync(w->S, hs, sizeof(MScalars), cudaMemcpyHostToDevice, s));
  HC_CUDA_TRY(h, multi_apply<T>(h, R, X, q, s));
  M_LAUNCH(k_m_setup, n, R, B, q, r, dinv, w->S, w->partials);
  HC_CUDA_TRY(h, cudaMemsetAsync(p, 0, n * R * sizeof(T), s));
  hc_status pst = precond(1);
  if (pst != HC_OK) return pst;
  M_LAUNCH(k_m_dir, n, R, r, z, dinv, p, q, h->ess, w->S);
  HC_CUDA_TRY(h, cudaGetLastError());
  const int chunk = 25;
  for (int launched = 0;;) {
    for (int k = 0; k < chunk && launched < maxit; ++k, ++launched) {
      // q holds (I-P) p; the apply adds P K P p
      HC_CUDA_TRY(h, tet_apply_launch<T>(h, sizeof(T) == 8 ? (const T*)h->tetK64 : (const T*)h->tetK32, p, q, R,
                                         true, 1.0, &w->S->all_done, s));
      M_LAUNCH(k_m_alpha, n, R, p, q, w->S, w->partials);
      M_LAUNCH(k_m_update, n, R, X, r, p, q, dinv, aux ? 0 : 1, w->S, w->partials);
      pst = precond(0);
      if (pst != HC_OK) return pst;
      M_LAUNCH(k_m_dir, n, R, r, z, dinv, p, q, h->ess, w->S);
    }
    HC_CUDA_TRY(h, cudaGetLastError());
    HC_CUDA_TRY(h, cudaMemcpyAsync(hs, w->S, sizeof(MScalars), cudaMemcpyDeviceToHost, s));
    HC_CUDA_TRY(h, cudaStreamSynchronize(s));
    if (hook) {
      const int a = hook->at_batch(hs);
      if (a == kMHookStop) break;
      if (a == kMHookResumed && launched < maxit) continue;
    }
    if (hs->all_done || launched >= maxit) break;
  }
  return HC_OK;
}

hc_status multi_solve_device(hcop* h, const hc_solve_params* prm, int R, const double* B, double* X,
                             hc_solve_info* info) {
  if (h->type != HC_TET) {
    h->err = "multi-RHS solves: tet meshes (batched element matrices) only in this build";
    return HC_ENOTSUP;
  }
  const int64_t n = h->ndof;
  const size_t nr = (size_t)n * R;
  MultiWork* w = nullptr;
  for (int k = 0; k < R; ++k) std::memset(&info[k], 0, sizeof(hc_solve_info));
  const bool aux = prm->precond == HC_PRECOND_AUX;
  const size_t nk = aux ? 4 : 3;  // Krylov vectors: r, p, q (, z)
  if (aux) {
    hc_status st = tetaux_setup(h);
    if (st == HC_OK) st = tetaux_reserve(h, R);
    if (st != HC_OK) return st;
  }
  if (prm->precision == HC_FP64) {
    hc_status st = multi_prepare(h, nk * nr * sizeof(double));
    if (st != HC_OK) return st;
    w = mwork(h);
    st = mpcg_run<double>(h, R, prm->rtol, prm->atol, prm->maxit, B, X, (double*)w->vec, h->dinv, aux, nullptr);
    if (st != HC_OK) return st;
    hc_status worst = HC_OK;
    for (int k = 0; k < R; ++k) {
      info[k].status = w->hS->done[k] ? w->hS->status[k] : HC_NOT_CONVERGED;
      info[k].iterations = w->hS->it[k];
      info[k].outer_iterations = 1;
      info[k].rel_residual = w->hS->bb[k] > 0 ? std::sqrt(w->hS->rr[k] / w->hS->bb[k]) : std::sqrt(w->hS->rr[k]);
      if (info[k].status != HC_OK && worst == HC_OK) worst = (hc_status)info[k].status;
    }
    return worst;
  }
  // mixed: r64 (n R doubles) | rf, c (2 n R floats) | r, p, q (, z) (nk n R floats)
  hc_status st = multi_prepare(h, nr * sizeof(double) + (2 + nk) * nr * sizeof(float));
  if (st != HC_OK) return st;
  w = mwork(h);
  double* r64 = (double*)w->vec;
  float* rf = (float*)(r64 + nr);
  float* c = rf + nr;
  float* wk = c + nr;
  cudaStream_t s = h->stream;
  const unsigned g = mgrid(n, R);
  std::vector<double> rn(R), bn(R), tol(R), inv(2 * kMaxRhs, 0.0);
  std::vector<int> total(R, 0), outer(R, 0);
  auto residual = [&]() -> hc_status {
    HC_CUDA_TRY(h, multi_apply<double>(h, R, X, r64, s));
    k_m_resid64<<<g, kMThreads, 0, s>>>(n, R, B, r64, w->S, w->partials);
    HC_CUDA_TRY(h, cudaGetLastError());
    HC_CUDA_TRY(h, cudaMemcpyAsync(w->hS, w->S, sizeof(MScalars), cudaMemcpyDeviceToHost, s));
    HC_CUDA_TRY(h, cudaStreamSynchronize(s));
    for (int k = 0; k < R; ++k) rn[k] = std::sqrt(w->hS->rr[k]);
    return HC_OK;
  };
  st = residual();
  if (st != HC_OK) return st;
  for (int k = 0; k < R; ++k) {
    bn[k] = std::sqrt(w->hS->bb[k]);
    tol[k] = std::max(prm->rtol * bn[k], prm->atol);
  }
  const double inner = prm->inner_rtol > 0 ? prm->inner_rtol : 1e-4;
  const int max_outer = prm->max_outer > 0 ? prm->max_outer : 50;
  std::vector<double> rn_prev(R, 0.0);
  bool stalled = false;
  if (prm->precision == HC_MIXED_RR) {
    // One FP32 block PCG with FP64 residual replacement, per column: the
    // block form of the single-column solve (van der Vorst & Ye residual
    // replacement; direction and r.z kept across a replacement).
    struct BlockReplace : MultiHook {
      hcop* h;
      MultiWork* w;
      int R;
      int64_t n;
      unsigned g;
      double *r64, *X;
      float *rpcg, *c;
      double delta2;
      std::vector<double>*rn, *tol, scale, rr_last, rnp, inv;
      std::vector<int> stop, slow, *total;
      std::function<hc_status()> residual;
      int since = 0, replacements = 0, maxit = 0;
      bool any_stalled = false;
      hc_status err = HC_OK;
      int at_batch(MScalars* hs) override {
        bool due = hs->all_done != 0;
        for (int k = 0; k < R; ++k) {
          if (stop[k]) continue;
          if (hs->done[k] && hs->status[k] == HC_BREAKDOWN) continue;
          if (hs->done[k] || hs->rr[k] <= delta2 * rr_last[k]) due = true;
        }
        if (!due && ++since < 8) return kMHookGoOn;
        since = 0;
        cudaStream_t s = h->stream;
        // x += scale_k c_k, c = 0, then the FP64 residual of every column
        for (int k = 0; k < R; ++k) inv[kMaxRhs + k] = scale[k];
        cudaError_t e = cudaMemcpyAsync(w->col, inv.data(), 2 * kMaxRhs * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
          k_m_axpy<<<g, kMThreads, 0, s>>>(n, R, c, w->col + kMaxRhs, X);
          e = cudaMemsetAsync(c, 0, (size_t)n * R * sizeof(float), s);
        }
        if (e != cudaSuccess) {
          h->err = cudaGetErrorString(e);
          err = HC_ECUDA;
          return kMHookStop;
        }
        std::vector<int> it_now(R), done_now(R), st_now(R);
        for (int k = 0; k < R; ++k) {
          it_now[k] = hs->it[k];
          done_now[k] = hs->done[k];
          st_now[k] = hs->status[k];
        }
        err = residual();  // overwrites hs (= w->hS) with the device scalars and rr, bb
        if (err != HC_OK) return kMHookStop;
        ++replacements;
        bool all = true;
        for (int k = 0; k < R; ++k) {
          const double r = (*rn)[k];
          if (!stop[k]) {
            (*total)[k] = it_now[k];
            if (!std::isfinite(r)) {
              stop[k] = HC_BREAKDOWN + 100;
            } else if (r <= (*tol)[k]) {
              stop[k] = HC_OK + 100;
            } else if (done_now[k] && st_now[k] == HC_BREAKDOWN) {
              stop[k] = HC_BREAKDOWN + 100;
            } else if (it_now[k] >= maxit) {
              stop[k] = HC_NOT_CONVERGED + 100;
            } else {
              slow[k] = r > 0.5 * rnp[k] ? slow[k] + 1 : 0;
              rnp[k] = r;
              if (slow[k] >= 2) {  // this column's FP32 floor: finish it in FP64
                stop[k] = HC_NOT_CONVERGED + 100;
                any_stalled = true;
              }
            }
          }
          const bool on = !stop[k];
          inv[k] = on ? 1.0 / scale[k] : 0.0;
          hs->rr[k] = on ? r * r / (scale[k] * scale[k]) : 0.0;
          hs->done[k] = on ? 0 : 1;
          hs->status[k] = on ? HC_NOT_CONVERGED : stop[k] - 100;
          hs->it[k] = it_now[k];
          if (on) rr_last[k] = hs->rr[k];
          all &= !on;
        }
        hs->all_done = all ? 1 : 0;
        if (all) return kMHookStop;
        // the FP32 recursive residuals := (b - J x) / scale (zero for stopped columns)
        e = cudaMemcpyAsync(w->col, inv.data(), 2 * kMaxRhs * sizeof(double), cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess) {
          k_m_d2f<<<g, kMThreads, 0, s>>>(n, R, r64, w->col, rpcg, c);
          e = cudaMemcpyAsync(w->S, hs, sizeof(MScalars), cudaMemcpyHostToDevice, s);
        }
        if (e != cudaSuccess) {
          h->err = cudaGetErrorString(e);
          err = HC_ECUDA;
          return kMHookStop;
        }
        return kMHookResumed;
      }
    };
    BlockReplace hk;
    hk.h = h;
    hk.w = w;
    hk.R = R;
    hk.n = n;
    hk.g = g;
    hk.r64 = r64;
    hk.X = X;
    hk.rpcg = wk;  // the block PCG's residual is its first work block
    hk.c = c;
    const double delta = prm->inner_rtol > 0 ? std::min(prm->inner_rtol, 0.5) : 0.1;
    hk.delta2 = delta * delta;
    hk.rn = &rn;
    hk.tol = &tol;
    hk.total = &total;
    hk.residual = residual;
    hk.maxit = prm->maxit;
    hk.scale.assign(R, 1.0);
    hk.rr_last.assign(R, 1.0);
    hk.rnp = rn;
    hk.inv.assign(2 * kMaxRhs, 0.0);
    hk.stop.assign(R, 0);
    hk.slow.assign(R, 0);
    double rin = 1.0;  // the FP32 stopping test, in units of each column's |r0|
    for (int k = 0; k < R; ++k) {
      if (!(rn[k] > tol[k]) || !std::isfinite(rn[k])) {
        hk.stop[k] = (std::isfinite(rn[k]) ? HC_OK : HC_BREAKDOWN) + 100;
        hk.scale[k] = 1.0;
        hk.inv[k] = 0.0;
      } else {
        hk.scale[k] = rn[k];
        hk.inv[k] = 1.0 / rn[k];
        rin = std::min(rin, 0.5 * tol[k] / rn[k]);
      }
      hk.inv[kMaxRhs + k] = hk.scale[k];
    }
    HC_CUDA_TRY(h, cudaMemcpyAsync(w->col, hk.inv.data(), 2 * kMaxRhs * sizeof(double), cudaMemcpyHostToDevice, s));
    k_m_d2f<<<g, kMThreads, 0, s>>>(n, R, r64, w->col, rf, c);
    HC_CUDA_TRY(h, cudaGetLastError());
    st = mpcg_run<float>(h, R, rin, 0.0, prm->maxit, rf, c, wk, h->dinvf, aux, &hk);
    if (st != HC_OK) return st;
    if (hk.err != HC_OK) return hk.err;
    // the correction since the last replacement (iteration cap) and the final residuals
    for (int k = 0; k < R; ++k) hk.inv[kMaxRhs + k] = hk.scale[k];
    HC_CUDA_TRY(h, cudaMemcpyAsync(w->col, hk.inv.data(), 2 * kMaxRhs * sizeof(double), cudaMemcpyHostToDevice, s));
    k_m_axpy<<<g, kMThreads, 0, s>>>(n, R, c, w->col + kMaxRhs, X);
    HC_CUDA_TRY(h, cudaGetLastError());
    for (int k = 0; k < R; ++k)
      if (!hk.stop[k]) total[k] = w->hS->it[k];
    st = residual();
    if (st != HC_OK) return st;
    for (int k = 0; k < R; ++k) outer[k] = hk.replacements;
    stalled = hk.any_stalled;
  }
  for (int step = 0; prm->precision != HC_MIXED_RR; ++step) {
    bool all = true, any_bad = false;
    for (int k = 0; k < R; ++k) {
      if (!std::isfinite(rn[k])) any_bad = true;
      if (rn[k] > tol[k]) all = false;
    }
    if (all || any_bad || step >= max_outer) break;
    bool progress = step < 2;
    for (int k = 0; k < R; ++k)
      if (rn[k] > tol[k] && rn[k] <= 0.25 * rn_prev[k]) progress = true;
    if (!progress) {
      stalled = true;
      break;
    }
    int used = 0;
    for (int k = 0; k < R; ++k) used = std::max(used, total[k]);
    if (used >= prm->maxit) break;
    // column scales: converged columns get zero right-hand sides (their correction stays 0)
    for (int k = 0; k < R; ++k) {
      inv[k] = rn[k] > tol[k] ? 1.0 / rn[k] : 0.0;
      inv[kMaxRhs + k] = rn[k] > tol[k] ? rn[k] : 0.0;
      rn_prev[k] = rn[k];
      if (rn[k] > tol[k]) ++outer[k];
    }
    HC_CUDA_TRY(h, cudaMemcpyAsync(w->col, inv.data(), 2 * kMaxRhs * sizeof(double), cudaMemcpyHostToDevice, s));
    k_m_d2f<<<g, kMThreads, 0, s>>>(n, R, r64, w->col, rf, c);
    st = mpcg_run<float>(h, R, inner, 0.0, std::min(prm->maxit - used, std::max(100, prm->maxit / 4)), rf, c, wk,
                         h->dinvf, aux, nullptr);
    if (st != HC_OK) return st;
    for (int k = 0; k < R; ++k) total[k] += w->hS->it[k];
    k_m_axpy<<<g, kMThreads, 0, s>>>(n, R, c, w->col + kMaxRhs, X);
    HC_CUDA_TRY(h, cudaGetLastError());
    st = residual();
    if (st != HC_OK) return st;
  }
  if (stalled) {
    // FP64 block PCG from the refined X
    const size_t off = nr * sizeof(double) + (2 + nk) * nr * sizeof(float);
    st = multi_prepare(h, off + nk * nr * sizeof(double));
    if (st != HC_OK) return st;
    w = mwork(h);
    r64 = (double*)w->vec;
    double* wk64 = (double*)((char*)w->vec + off);
    // aim below the tolerance: the polish stops on its recursive residual,
    // the status below is judged on the true one.  A restart from X (its
    // set-up recomputes B - J X per column) is one FP64 refinement step: up
    // to three rounds while the worst unconverged column at least halves.
    double worst_prev = 0.0;
    for (int k = 0; k < R; ++k)
      if (rn[k] > tol[k]) worst_prev = std::max(worst_prev, rn[k] / std::max(tol[k], 1e-300));
    for (int round = 0; round < 3; ++round) {
      int used = 0;
      for (int k = 0; k < R; ++k) used = std::max(used, total[k]);
      if (used >= prm->maxit) break;
      st = mpcg_run<double>(h, R, 0.5 * prm->rtol, 0.5 * prm->atol, std::max(1, prm->maxit - used), B, X, wk64,
                            h->dinv, aux, nullptr);
      if (st != HC_OK) return st;
      for (int k = 0; k < R; ++k) {
        total[k] += w->hS->it[k];
        ++outer[k];
      }
      st = residual();
      if (st != HC_OK) return st;
      double worst = 0.0;
      bool bad = false;
      for (int k = 0; k < R; ++k) {
        if (!std::isfinite(rn[k])) bad = true;
        if (rn[k] > tol[k]) worst = std::max(worst, rn[k] / std::max(tol[k], 1e-300));
      }
      if (bad || worst == 0.0 || worst > 0.5 * worst_prev) break;
      worst_prev = worst;
    }
  }
  hc_status worst = HC_OK;
  for (int k = 0; k < R; ++k) {
    const bool ok = std::isfinite(rn[k]) && rn[k] <= tol[k];
    info[k].status = std::isfinite(rn[k]) ? (ok ? HC_OK : HC_NOT_CONVERGED) : HC_BREAKDOWN;
    info[k].iterations = total[k];
    info[k].outer_iterations = outer[k];
    info[k].rel_residual = bn[k] > 0 ? rn[k] / bn[k] : rn[k];
    if (info[k].status != HC_OK && worst == HC_OK) worst = (hc_status)info[k].status;
  }
  return worst;
}

}  // namespace hc

using namespace hc;

extern "C" hc_status hc_solve_multi_device(hcop_t* h, const hc_solve_params* prm, int32_t nrhs, const double* B,
                                           double* X, hc_solve_info* info) {
  if (!h || !prm || !B || !X || !info) return HC_EINVAL;
  if (nrhs != 1 && nrhs != 2 && nrhs != 4 && nrhs != 8 && nrhs != 16 && nrhs != 32) {
    h->err = "hc_solve_multi_device: nrhs must be 1, 2, 4, 8, 16 or 32";
    return HC_EINVAL;
  }
  if (prm->precision != HC_FP64 && prm->precision != HC_MIXED && prm->precision != HC_MIXED_RR) {
    h->err = "precision must be HC_FP64, HC_MIXED or HC_MIXED_RR";
    return HC_EINVAL;
  }
  if ((reinterpret_cast<uintptr_t>(B) | reinterpret_cast<uintptr_t>(X)) % 16 != 0) {
    h->err = "hc_solve_multi_device: B and X must be 16-byte aligned";  // 128-bit vector accesses
    return HC_EINVAL;
  }
  if (prm->precond != HC_PRECOND_JACOBI && prm->precond != HC_PRECOND_AUX) {
    h->err = "multi-RHS solves take the Jacobi or the auxiliary-space preconditioner";
    return HC_ENOTSUP;
  }
  if (!(prm->rtol >= 0.0) || !(prm->atol >= 0.0) || prm->maxit < 1) {
    h->err = "rtol, atol must be >= 0 and maxit >= 1";
    return HC_EINVAL;
  }
  return multi_solve_device(h, prm, nrhs, B, X, info);
}

extern "C" hc_status hc_solve_multi(hcop_t* h, const hc_solve_params* prm, int32_t nrhs, const double* B, double* X,
                                    hc_solve_info* info) {
  if (!h || !prm || !B || !X || !info) return HC_EINVAL;
  if (nrhs != 1 && nrhs != 2 && nrhs != 4 && nrhs != 8 && nrhs != 16 && nrhs != 32) {
    h->err = "hc_solve_multi: nrhs must be 1, 2, 4, 8, 16 or 32";
    return HC_EINVAL;
  }
  const size_t bytes = (size_t)h->ndof * nrhs * sizeof(double);
  double *dB = nullptr, *dX = nullptr;
  if (dmalloc(h, (void**)&dB, bytes) != cudaSuccess || dmalloc(h, (void**)&dX, bytes) != cudaSuccess) {
    dfree(h, dB);
    dfree(h, dX);
    h->err = "hc_solve_multi: device staging allocation failed";
    return HC_ENOMEM;
  }
  hc_status st = HC_OK;
  if (cudaMemcpyAsync(dB, B, bytes, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
      cudaMemcpyAsync(dX, X, bytes, cudaMemcpyHostToDevice, h->stream) != cudaSuccess) {
    h->err = "hc_solve_multi: host-to-device copy failed";
    st = HC_ECUDA;
  }
  if (st == HC_OK) st = hc_solve_multi_device(h, prm, nrhs, dB, dX, info);
  if (st == HC_OK || st == HC_NOT_CONVERGED || st == HC_BREAKDOWN) {
    if (cudaMemcpyAsync(X, dX, bytes, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
        cudaStreamSynchronize(h->stream) != cudaSuccess) {
      h->err = "hc_solve_multi: device-to-host copy failed";
      st = HC_ECUDA;
    }
  }
  dfree(h, dB);
  dfree(h, dX);
  cudaStreamSynchronize(h->stream);
  return st;
}

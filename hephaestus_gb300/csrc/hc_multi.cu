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

// Segmented (per right-hand side) sum of NV values per thread; thread t owns
// rhs t % R.  Returns, on thread 0 of the last block, the grid totals in
// shared memory (total of value k for rhs r at [k * kMaxRhs + r]); nullptr
// elsewhere.
template <int NV>
__device__ const double* mgrid_sum(double (&v)[NV], int R, double* partials, unsigned int* counter) {
  __shared__ double sh[NV][kMThreads / 32][kMaxRhs];
  __shared__ double tot[NV * kMaxRhs];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k)
    for (int o = 16; o >= R; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
  if (lane < R)
#pragma unroll
    for (int k = 0; k < NV; ++k) sh[k][w][lane] = v[k];
  __syncthreads();
  // block partial per rhs, written by thread r < R
  if (threadIdx.x < R) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0.0;
      for (int i = 0; i < kMThreads / 32; ++i) s += sh[k][i][threadIdx.x];
      partials[((size_t)k * R + threadIdx.x) * gridDim.x + blockIdx.x] = s;
    }
  }
  __threadfence();
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

// Loop over the entries i = dof * R + rhs of this thread.  The grid stride is a
// multiple of R, so every thread keeps one right-hand side, K_COL = tid % R,
// and the dof is i >> lgR (R a power of two).
#define M_THREAD(R)                                                          \
  const int64_t m_t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;       \
  const int64_t m_stride = (int64_t)gridDim.x * blockDim.x;                  \
  const int K_COL = (int)(m_t0 & ((R) - 1));                                 \
  const int m_lg = __ffs(R) - 1;                                             \
  (void)K_COL;                                                               \
  (void)m_lg
#define M_LOOP(i, n, R) _Pragma("unroll 4") for (int64_t i = m_t0; i < (n) * (R); i += m_stride)

// Per-thread partial sums.  FP32 vectors accumulate runs of 32 terms in FP32
// and flush them into FP64 (GB300's FP64 rate is a small fraction of its FP32
// rate); FP64 vectors accumulate in FP64.
template <typename T, int NV>
struct MAcc {
  double v[NV];
  T a[NV];
  int cnt;
  __device__ MAcc() : cnt(0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      v[k] = 0.0;
      a[k] = T(0);
    }
  }
  __device__ __forceinline__ void flush() {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      v[k] += (double)a[k];
      a[k] = T(0);
    }
    cnt = 0;
  }
  __device__ __forceinline__ void step() {
    if (sizeof(T) == 4 && ++cnt == 32) flush();
  }
};

// r = b - q; bb, rr, rz per rhs; tolerances and the first stopping test
template <typename T>
__global__ void __launch_bounds__(kMThreads)
    k_m_setup(int64_t n, int R, const T* __restrict__ b, const T* __restrict__ q, T* __restrict__ r,
              const T* __restrict__ dinv, MScalars* S, double* partials) {
  M_THREAD(R);
  MAcc<T, 3> acc;
  M_LOOP(i, n, R) {
    const T bi = b[i], ri = bi - q[i];
    r[i] = ri;
    acc.a[0] += bi * bi;
    acc.a[1] += ri * ri;
    acc.a[2] += ri * ri * dinv[i >> m_lg];
    acc.step();
  }
  acc.flush();
  if (const double* tot = mgrid_sum<3>(acc.v, R, partials, &S->counter[0])) {
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
template <typename T>
__global__ void __launch_bounds__(kMThreads)
    k_m_dir(int64_t n, int R, const T* __restrict__ r, const T* __restrict__ z, const T* __restrict__ dinv,
            T* __restrict__ p, T* __restrict__ q, const uint8_t* __restrict__ ess, const MScalars* S) {
  if (S->all_done) return;
  M_THREAD(R);
  const bool stop = S->done[K_COL] != 0;
  const T beta = (T)S->beta[K_COL];
  M_LOOP(i, n, R) {
    const int64_t d = i >> m_lg;
    const T zi = z ? z[i] : dinv[d] * r[i];
    const T pi = stop ? T(0) : zi + beta * p[i];
    p[i] = pi;
    q[i] = ess[d] ? pi : T(0);
  }
}

// alpha = rz / p.q per rhs (q = J p)
template <typename T>
__global__ void __launch_bounds__(kMThreads)
    k_m_alpha(int64_t n, int R, const T* __restrict__ p, const T* __restrict__ q, MScalars* S, double* partials) {
  if (S->all_done) return;
  M_THREAD(R);
  MAcc<T, 1> acc;
  M_LOOP(i, n, R) {
    acc.a[0] += p[i] * q[i];
    acc.step();
  }
  acc.flush();
  if (const double* tot = mgrid_sum<1>(acc.v, R, partials, &S->counter[1])) {
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
template <typename T>
__global__ void __launch_bounds__(kMThreads)
    k_m_update(int64_t n, int R, T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
               const T* __restrict__ q, const T* __restrict__ dinv, int jac, MScalars* S, double* partials) {
  if (S->all_done) return;
  M_THREAD(R);
  const T a = (T)S->alpha[K_COL];
  MAcc<T, 2> acc;
  M_LOOP(i, n, R) {
    x[i] += a * p[i];
    const T ri = r[i] - a * q[i];
    r[i] = ri;
    acc.a[0] += ri * ri;
    if (jac) acc.a[1] += ri * ri * dinv[i >> m_lg];
    acc.step();
  }
  acc.flush();
  if (const double* tot = mgrid_sum<2>(acc.v, R, partials, &S->counter[2])) {
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
template <typename T>
__global__ void __launch_bounds__(kMThreads)
    k_m_rz(int64_t n, int R, const T* __restrict__ r, const T* __restrict__ z, int first, MScalars* S,
           double* partials) {
  if (S->all_done) return;
  M_THREAD(R);
  MAcc<T, 1> acc;
  M_LOOP(i, n, R) {
    acc.a[0] += r[i] * z[i];
    acc.step();
  }
  acc.flush();
  if (const double* tot = mgrid_sum<1>(acc.v, R, partials, &S->counter[1])) {
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
  M_THREAD(R);
  double v[2] = {0, 0};
  M_LOOP(i, n, R) {
    const double bi = b[i], ri = bi - r[i];
    r[i] = ri;
    v[0] += ri * ri;
    v[1] += bi * bi;
  }
  if (const double* tot = mgrid_sum<2>(v, R, partials, &S->counter[3]))
    for (int k = 0; k < R; ++k) {
      S->rr[k] = tot[k];
      S->bb[k] = tot[kMaxRhs + k];
    }
}
// rf = r / |r_k| per column (FP32); c = 0
__global__ void __launch_bounds__(kMThreads)
    k_m_d2f(int64_t n, int R, const double* __restrict__ r, const double* __restrict__ inv, float* __restrict__ rf,
            float* __restrict__ c) {
  M_THREAD(R);
  const double s = inv[K_COL];
  M_LOOP(i, n, R) {
    rf[i] = (float)(r[i] * s);
    c[i] = 0.0f;
  }
}
// x += |r_k| c per column
__global__ void __launch_bounds__(kMThreads)
    k_m_axpy(int64_t n, int R, const float* __restrict__ c, const double* __restrict__ scale, double* __restrict__ x) {
  M_THREAD(R);
  const double s = scale[K_COL];
  M_LOOP(i, n, R) x[i] += s * (double)c[i];
}

static inline unsigned mgrid(int64_t n, int R) {
  // the grid stride (blocks x threads) is a multiple of 32 >= R: one rhs per thread
  const int64_t b = (n * R + kMThreads - 1) / kMThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, kMBlocks));
}

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
template <typename T>
static hc_status mpcg_run(hcop* h, int R, double rtol, double atol, int maxit, const T* B, T* X, T* wk,
                          const T* dinv, bool aux) {
  MultiWork* w = mwork(h);
  cudaStream_t s = h->stream;
  const int64_t n = h->ndof;
  T *r = wk, *p = wk + n * R, *q = wk + 2 * n * R;
  T* z = aux ? wk + 3 * n * R : nullptr;
  const int* all_done = &w->S->all_done;
  auto precond = [&](int first) -> hc_status {
    if (!aux) return HC_OK;
    HC_CUDA_TRY(h, tetaux_apply<T>(h, R, r, z, dinv, all_done, s));
    k_m_rz<T><<<mgrid(n, R), kMThreads, 0, s>>>(n, R, r, z, first, w->S, w->partials);
    return HC_OK;
  };
  MScalars* hs = w->hS;
  std::memset(hs, 0, sizeof(MScalars));
  hs->rtol2 = rtol * rtol;
  hs->atol2 = atol * atol;
  hs->maxit = maxit;
  HC_CUDA_TRY(h, cudaMemcpyAsync(w->S, hs, sizeof(MScalars), cudaMemcpyHostToDevice, s));
  const unsigned g = mgrid(n, R);
  HC_CUDA_TRY(h, multi_apply<T>(h, R, X, q, s));
  k_m_setup<T><<<g, kMThreads, 0, s>>>(n, R, B, q, r, dinv, w->S, w->partials);
  HC_CUDA_TRY(h, cudaMemsetAsync(p, 0, n * R * sizeof(T), s));
  hc_status pst = precond(1);
  if (pst != HC_OK) return pst;
  k_m_dir<T><<<g, kMThreads, 0, s>>>(n, R, r, z, dinv, p, q, h->ess, w->S);
  HC_CUDA_TRY(h, cudaGetLastError());
  const int chunk = 25;
  for (int launched = 0;;) {
    for (int k = 0; k < chunk && launched < maxit; ++k, ++launched) {
      // q holds (I-P) p; the apply adds P K P p
      HC_CUDA_TRY(h, tet_apply_launch<T>(h, sizeof(T) == 8 ? (const T*)h->tetK64 : (const T*)h->tetK32, p, q, R,
                                         true, 1.0, &w->S->all_done, s));
      k_m_alpha<T><<<g, kMThreads, 0, s>>>(n, R, p, q, w->S, w->partials);
      k_m_update<T><<<g, kMThreads, 0, s>>>(n, R, X, r, p, q, dinv, aux ? 0 : 1, w->S, w->partials);
      pst = precond(0);
      if (pst != HC_OK) return pst;
      k_m_dir<T><<<g, kMThreads, 0, s>>>(n, R, r, z, dinv, p, q, h->ess, w->S);
    }
    HC_CUDA_TRY(h, cudaGetLastError());
    HC_CUDA_TRY(h, cudaMemcpyAsync(hs, w->S, sizeof(MScalars), cudaMemcpyDeviceToHost, s));
    HC_CUDA_TRY(h, cudaStreamSynchronize(s));
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
    st = mpcg_run<double>(h, R, prm->rtol, prm->atol, prm->maxit, B, X, (double*)w->vec, h->dinv, aux);
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
  for (int step = 0;; ++step) {
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
                         h->dinvf, aux);
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
    int used = 0;
    for (int k = 0; k < R; ++k) used = std::max(used, total[k]);
    st = mpcg_run<double>(h, R, prm->rtol, prm->atol, std::max(1, prm->maxit - used), B, X, wk64, h->dinv, aux);
    if (st != HC_OK) return st;
    for (int k = 0; k < R; ++k) {
      total[k] += w->hS->it[k];
      ++outer[k];
    }
    st = residual();
    if (st != HC_OK) return st;
  }
  hc_status worst = HC_OK;
  for (int k = 0; k < R; ++k) {
    const bool ok = std::isfinite(rn[k]) && rn[k] <= tol[k] * (stalled ? 1.01 : 1.0);
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
  if (prm->precision != HC_FP64 && prm->precision != HC_MIXED) {
    h->err = "precision must be HC_FP64 or HC_MIXED";
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

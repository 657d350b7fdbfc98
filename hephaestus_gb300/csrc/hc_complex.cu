// hc_complex.cu -- frequency-domain operator A = C_nu + i omega M_sigma and its
// complex-symmetric solve.
//
// Reference: ComplexMaxwellOperator::Solve assembles a ParSesquilinearForm with
// CurlCurlIntegrator(nu) in the real part and VectorFEMassIntegrator(omega
// sigma) in the imaginary part (src/formulations/ComplexMaxwell/complex_maxwell_formulation.cpp:171-222)
// and solves the 2N x 2N real system (Hermitian convention) with SuperLU.  The
// same system is the complex-symmetric A u = b, solved here matrix-free by
// COCG (conjugate orthogonal CG, van der Vorst & Melissen 1990) with a complex
// Jacobi preconditioner, in FP64 or as FP32 inner COCG inside FP64 iterative
// refinement.  Vectors are planar (separate real and imaginary arrays).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "hc_graph.h"
#include "hc_internal.h"
#include "hc_reduce.cuh"

namespace hc {

#define GS_LOOP(i, n) \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

static inline unsigned cgrid(int64_t n) {
  int64_t b = (n + kRedThreads - 1) / kRedThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, kRedBlocks));
}

struct CScalars {
  double rho_r, rho_i;    // r^T z
  double alpha_r, alpha_i;
  double beta_r, beta_i;
  double rr, bb, tol2;  // tol2 = max(rtol2 |b|^2, atol2), set by k_c_setup
  double rtol2, atol2;
  int it, done, status, maxit;
  int trips;  // WHILE-loop trips of a graph-driven solve
  unsigned int counter[6];
};

// ---- complex operator -------------------------------------------------------------
// y = (I-P) x + P (C + i w M) P x, planar.  The curl factor of the handle
// carries dt, so C_nu = (dt C_nu) / dt.
#define HC_EXTERN_CPLX(T, P)                                                                              \
  extern template cudaError_t hex_launch_cplx_p<T, P>(const HexDev&, const T*, const T*, const T*, T*, T*, T, T, \
                                                      bool, const int*, cudaStream_t);
HC_EXTERN_CPLX(double, 1)
HC_EXTERN_CPLX(double, 2)
HC_EXTERN_CPLX(float, 1)
HC_EXTERN_CPLX(float, 2)
#undef HC_EXTERN_CPLX

// y = (I-P) x for both parts in one launch; skipped when *done != 0.
template <typename T>
__global__ void k_c_init_masked(int64_t n, const uint8_t* __restrict__ ess, const T* __restrict__ xr,
                                const T* __restrict__ xi, T* __restrict__ yr, T* __restrict__ yi,
                                const int* __restrict__ done) {
  if (done && *done) return;
  GS_LOOP(k, n) {
    const bool e = ess[k] != 0;
    yr[k] = e ? xr[k] : T(0);
    yi[k] = e ? xi[k] : T(0);
  }
}

// One init for both parts ((I-P) x) and one fused kernel (orders 1-2); `done`
// (may be null) skips both once a COCG batch has stopped.
template <typename T>
cudaError_t complex_apply_done(hcop* h, double omega, const T* xr, const T* xi, T* yr, T* yi, const int* done,
                               cudaStream_t s) {
  const T* fac = sizeof(T) == 8 ? (const T*)h->fac : (const T*)h->facf;
  const HexDev d = h->hexdev();
  const T cs = (T)(1.0 / h->dt);
  const T om = h->has_mass ? (T)omega : T(0);
  k_c_init_masked<T><<<cgrid(h->ndof), kRedThreads, 0, s>>>(h->ndof, h->ess, xr, xi, yr, yi, done);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  switch (h->p) {
    case 1: return hex_launch_cplx_p<T, 1>(d, fac, xr, xi, yr, yi, om, cs, true, done, s);
    case 2: return hex_launch_cplx_p<T, 2>(d, fac, xr, xi, yr, yi, om, cs, true, done, s);
    case 3: {
      (void)done;
      if (!d.full) {  // one two-input launch per output
        e = hex_launch_pair<T, 3>(d, fac, xr, xi, yr, -om, cs, s);
        if (e == cudaSuccess) e = hex_launch_pair<T, 3>(d, fac, xi, xr, yi, om, cs, s);
        return e;
      }
      // general parallelepipeds: four launches of the real kernel
      e = hex_apply<T>(d, fac, xr, yr, 0.0, (double)cs, true, nullptr, nullptr, s, false);
      if (e == cudaSuccess && om != T(0)) e = hex_apply<T>(d, fac, xi, yr, -omega, 0.0, true, nullptr, nullptr, s, false);
      if (e == cudaSuccess) e = hex_apply<T>(d, fac, xi, yi, 0.0, (double)cs, true, nullptr, nullptr, s, false);
      if (e == cudaSuccess && om != T(0)) e = hex_apply<T>(d, fac, xr, yi, omega, 0.0, true, nullptr, nullptr, s, false);
      return e;
    }
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
cudaError_t complex_apply(hcop* h, double omega, const T* xr, const T* xi, T* yr, T* yi, cudaStream_t s) {
  return complex_apply_done<T>(h, omega, xr, xi, yr, yi, nullptr, s);
}

// Complex inverse diagonal: 1 / (dC + i w dM) at free dofs, 1 at essential rows.
__global__ void k_cinv_diag(int64_t n, const uint8_t* __restrict__ ess, const double* __restrict__ dC,
                            const double* __restrict__ dM, double omega, double* __restrict__ ir,
                            double* __restrict__ ii, float* __restrict__ irf, float* __restrict__ iif) {
  GS_LOOP(k, n) {
    double a = 1.0, b = 0.0;
    if (!ess[k]) {
      a = dC[k];
      b = omega * dM[k];
    }
    double den = a * a + b * b;
    if (!(den > 0.0) || !isfinite(den)) {
      a = 1.0;
      b = 0.0;
      den = 1.0;
    }
    const double r = a / den, im = -b / den;
    ir[k] = r;
    ii[k] = im;
    irf[k] = (float)r;
    iif[k] = (float)im;
  }
}

// ---- COCG kernels ---------------------------------------------------------------------
// The bilinear dots r^T z of COCG are not positive and can cancel, so their
// products and sums stay in FP64 even for FP32 vectors (the real PCG kernels,
// whose dots are positive, sum in the vectors' precision per thread).
// r = b - Ax (q holds Ax); z = D^-1 r; p = z; rho = r^T z; rr = |r|^2; bb = |b|^2
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_c_setup(int64_t n, const T* br, const T* bi, const T* qr, const T* qi, T* rr_, T* ri_, T* pr, T* pi,
              const T* dr, const T* di, CScalars* S, double* partials, const int* active) {
  // active (may be null): 0 skips the launch (a stopped refinement loop);
  // qr == nullptr: x = 0, r = b
  if (active && !*active) return;
  double v[4] = {0, 0, 0, 0}, tot[4];
  GS_LOOP(k, n) {
    const double a = qr ? (double)br[k] - (double)qr[k] : (double)br[k];
    const double b = qr ? (double)bi[k] - (double)qi[k] : (double)bi[k];
    rr_[k] = (T)a;
    ri_[k] = (T)b;
    const double zr = a * (double)dr[k] - b * (double)di[k], zi = a * (double)di[k] + b * (double)dr[k];
    pr[k] = (T)zr;
    pi[k] = (T)zi;
    v[0] += a * zr - b * zi;
    v[1] += a * zi + b * zr;
    v[2] += a * a + b * b;
    v[3] += (double)br[k] * (double)br[k] + (double)bi[k] * (double)bi[k];
  }
  block_sum_n<4>(v);
  if (grid_sum_n<4>(v, partials, &S->counter[0], tot)) {
    S->rho_r = tot[0];
    S->rho_i = tot[1];
    S->rr = tot[2];
    S->bb = tot[3];
    S->it = 0;
    S->done = 0;
    S->status = HC_NOT_CONVERGED;
    S->tol2 = fmax(S->rtol2 * tot[3], S->atol2);
    if (!isfinite(tot[2]) || !isfinite(tot[3])) {
      S->done = 1;
      S->status = HC_BREAKDOWN;
    } else if (tot[2] <= S->tol2) {
      S->done = 1;
      S->status = HC_OK;
    }
  }
}

// alpha = rho / (p^T q)
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_c_alpha(int64_t n, const T* pr, const T* pi, const T* qr, const T* qi, CScalars* S, double* partials) {
  if (S->done) return;
  double v[2] = {0, 0}, tot[2];
  GS_LOOP(k, n) {
    const double a = pr[k], b = pi[k], c = qr[k], d = qi[k];
    v[0] += a * c - b * d;
    v[1] += a * d + b * c;
  }
  block_sum_n<2>(v);
  if (grid_sum_n<2>(v, partials, &S->counter[1], tot)) {
    const double den = tot[0] * tot[0] + tot[1] * tot[1];
    if (!(den > 0.0) || !isfinite(den)) {
      S->done = 1;
      S->status = HC_BREAKDOWN;
      S->alpha_r = S->alpha_i = 0.0;
    } else {
      // (rho_r + i rho_i) / (t_r + i t_i)
      S->alpha_r = (S->rho_r * tot[0] + S->rho_i * tot[1]) / den;
      S->alpha_i = (S->rho_i * tot[0] - S->rho_r * tot[1]) / den;
    }
  }
}

// x += alpha p; r -= alpha q; z = D^-1 r; rho' = r^T z; rr = |r|^2; beta = rho'/rho
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_c_update(int64_t n, T* xr, T* xi, T* rr_, T* ri_, const T* pr, const T* pi, const T* qr, const T* qi,
               const T* dr, const T* di, CScalars* S, double* partials) {
  if (S->done) return;
  const T ar = (T)S->alpha_r, ai = (T)S->alpha_i;
  double v[3] = {0, 0, 0}, tot[3];
  GS_LOOP(k, n) {
    const T p_r = pr[k], p_i = pi[k];
    xr[k] += ar * p_r - ai * p_i;
    xi[k] += ar * p_i + ai * p_r;
    const T q_r = qr[k], q_i = qi[k];
    const T a = rr_[k] - (ar * q_r - ai * q_i), b = ri_[k] - (ar * q_i + ai * q_r);
    rr_[k] = a;
    ri_[k] = b;
    const double da = a, db = b, zr = da * (double)dr[k] - db * (double)di[k],
                 zi = da * (double)di[k] + db * (double)dr[k];
    v[0] += da * zr - db * zi;
    v[1] += da * zi + db * zr;
    v[2] += da * da + db * db;
  }
  block_sum_n<3>(v);
  if (grid_sum_n<3>(v, partials, &S->counter[2], tot)) {
    S->it += 1;
    S->rr = tot[2];
    const double den = S->rho_r * S->rho_r + S->rho_i * S->rho_i;
    if (!isfinite(tot[2]) || !(den > 0.0)) {
      S->done = 1;
      S->status = HC_BREAKDOWN;
    } else if (tot[2] <= S->tol2) {
      S->done = 1;
      S->status = HC_OK;
    } else if (S->it >= S->maxit) {
      S->done = 1;
      S->status = HC_NOT_CONVERGED;
    }
    if (den > 0.0) {
      S->beta_r = (tot[0] * S->rho_r + tot[1] * S->rho_i) / den;
      S->beta_i = (tot[1] * S->rho_r - tot[0] * S->rho_i) / den;
    }
    S->rho_r = tot[0];
    S->rho_i = tot[1];
  }
}

// p = D^-1 r + beta p
template <typename T>
__global__ void k_c_dir(int64_t n, const T* rr_, const T* ri_, const T* dr, const T* di, T* pr, T* pi,
                        const CScalars* S) {
  if (S->done) return;
  const T br = (T)S->beta_r, bi = (T)S->beta_i;
  GS_LOOP(k, n) {
    const T a = rr_[k], b = ri_[k];
    const T zr = a * dr[k] - b * di[k], zi = a * di[k] + b * dr[k];
    const T p_r = pr[k], p_i = pi[k];
    pr[k] = zr + br * p_r - bi * p_i;
    pi[k] = zi + br * p_i + bi * p_r;
  }
}

// ---- COCG with a materialised preconditioned residual z = B r (HC_PRECOND_AUX) ------------
// r = b - q (q == nullptr: x = 0); |b|^2, |r|^2; scalars reset
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_ca_setup(int64_t n, const T* br, const T* bi, const T* qr, const T* qi, T* rr_, T* ri_, CScalars* S,
               double* partials, const int* active) {
  if (active && !*active) return;
  double v[2] = {0, 0}, tot[2];
  GS_LOOP(k, n) {
    const double a = qr ? (double)br[k] - (double)qr[k] : (double)br[k];
    const double b = qr ? (double)bi[k] - (double)qi[k] : (double)bi[k];
    rr_[k] = (T)a;
    ri_[k] = (T)b;
    v[0] += a * a + b * b;
    v[1] += (double)br[k] * (double)br[k] + (double)bi[k] * (double)bi[k];
  }
  block_sum_n<2>(v);
  if (grid_sum_n<2>(v, partials, &S->counter[0], tot)) {
    S->rr = tot[0];
    S->bb = tot[1];
    S->it = 0;
    S->done = 0;
    S->status = HC_NOT_CONVERGED;
    S->tol2 = fmax(S->rtol2 * tot[1], S->atol2);
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
      S->done = 1;
      S->status = HC_BREAKDOWN;
    } else if (tot[0] <= S->tol2) {
      S->done = 1;
      S->status = HC_OK;
    }
  }
}

// x += alpha p; r -= alpha q; |r|^2; stopping tests
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_ca_update(int64_t n, T* xr, T* xi, T* rr_, T* ri_, const T* pr, const T* pi, const T* qr, const T* qi,
                CScalars* S, double* partials) {
  if (S->done) return;
  const T ar = (T)S->alpha_r, ai = (T)S->alpha_i;
  double v[1] = {0}, tot[1];
  GS_LOOP(k, n) {
    const T p_r = pr[k], p_i = pi[k];
    xr[k] += ar * p_r - ai * p_i;
    xi[k] += ar * p_i + ai * p_r;
    const T q_r = qr[k], q_i = qi[k];
    const T a = rr_[k] - (ar * q_r - ai * q_i), b = ri_[k] - (ar * q_i + ai * q_r);
    rr_[k] = a;
    ri_[k] = b;
    v[0] += (double)a * (double)a + (double)b * (double)b;
  }
  block_sum_n<1>(v);
  if (grid_sum_n<1>(v, partials, &S->counter[2], tot)) {
    S->it += 1;
    S->rr = tot[0];
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
  }
}

// z = D^-1 r (complex Jacobi part)
template <typename T>
__global__ void k_ca_jz(int64_t n, const T* rr_, const T* ri_, const T* dr, const T* di, T* zr, T* zi,
                        const CScalars* S) {
  if (S->done) return;
  GS_LOOP(k, n) {
    const T a = rr_[k], b = ri_[k];
    zr[k] = a * dr[k] - b * di[k];
    zi[k] = a * di[k] + b * dr[k];
  }
}

// rho' = r^T z; beta = rho'/rho (0 on the first call); rho = rho'
template <typename T>
__global__ void __launch_bounds__(kRedThreads)
    k_ca_rho(int64_t n, const T* rr_, const T* ri_, const T* zr, const T* zi, int first, CScalars* S,
             double* partials) {
  if (S->done) return;
  double v[2] = {0, 0}, tot[2];
  GS_LOOP(k, n) {
    const double a = rr_[k], b = ri_[k], c = zr[k], d = zi[k];
    v[0] += a * c - b * d;
    v[1] += a * d + b * c;
  }
  block_sum_n<2>(v);
  if (grid_sum_n<2>(v, partials, &S->counter[4], tot)) {
    if (first) {
      S->beta_r = S->beta_i = 0.0;
    } else {
      const double den = S->rho_r * S->rho_r + S->rho_i * S->rho_i;
      if (!(den > 0.0) || !isfinite(den) || !isfinite(tot[0]) || !isfinite(tot[1])) {
        S->done = 1;
        S->status = HC_BREAKDOWN;
        S->beta_r = S->beta_i = 0.0;
      } else {
        S->beta_r = (tot[0] * S->rho_r + tot[1] * S->rho_i) / den;
        S->beta_i = (tot[1] * S->rho_r - tot[0] * S->rho_i) / den;
      }
    }
    S->rho_r = tot[0];
    S->rho_i = tot[1];
  }
}

// p = z + beta p (first: p = z)
template <typename T>
__global__ void k_ca_dir(int64_t n, const T* zr, const T* zi, T* pr, T* pi, int first, const CScalars* S) {
  if (S->done) return;
  const T br = (T)S->beta_r, bi = (T)S->beta_i;
  GS_LOOP(k, n) {
    if (first) {
      pr[k] = zr[k];
      pi[k] = zi[k];
    } else {
      const T p_r = pr[k], p_i = pi[k];
      pr[k] = zr[k] + br * p_r - bi * p_i;
      pi[k] = zi[k] + br * p_i + bi * p_r;
    }
  }
}

// ---- host drivers -----------------------------------------------------------------------
struct ComplexWork {
  double *dC = nullptr, *dM = nullptr, *ir = nullptr, *ii = nullptr;
  float *irf = nullptr, *iif = nullptr;
  double omega = -1.0;
  CScalars* S = nullptr;
  CScalars* hS = nullptr;
  void* vec = nullptr;
  size_t vec_bytes = 0;
  void* graph = nullptr;  // ComplexGraph of the graph-driven solve
};

static void cgraph_free(hcop* h, ComplexWork* w);

static ComplexWork* cwork(hcop* h) {
  if (!h->cwork) h->cwork = new ComplexWork();
  return static_cast<ComplexWork*>(h->cwork);
}

void complex_free(hcop* h) {
  if (!h->cwork) return;
  ComplexWork* w = static_cast<ComplexWork*>(h->cwork);
  cgraph_free(h, w);
  for (void* p : {(void*)w->dC, (void*)w->dM, (void*)w->ir, (void*)w->ii, (void*)w->irf, (void*)w->iif,
                  (void*)w->S, w->vec})
    dfree(h, p);
  pinned_put(w->hS);
  delete w;
  h->cwork = nullptr;
}

static hc_status complex_prepare(hcop* h, double omega) {
  ComplexWork* w = cwork(h);
  const int64_t n = h->ndof;
  if (!w->dC) {
    if (dmalloc(h, (void**)&w->dC, n * 8) != cudaSuccess || dmalloc(h, (void**)&w->dM, n * 8) != cudaSuccess ||
        dmalloc(h, (void**)&w->ir, n * 8) != cudaSuccess || dmalloc(h, (void**)&w->ii, n * 8) != cudaSuccess ||
        dmalloc(h, (void**)&w->irf, n * 4) != cudaSuccess || dmalloc(h, (void**)&w->iif, n * 4) != cudaSuccess ||
        dmalloc(h, (void**)&w->S, sizeof(CScalars)) != cudaSuccess ||
        !(w->hS = static_cast<CScalars*>(pinned_get(sizeof(CScalars))))) {
      h->err = "complex work space allocation failed";
      return HC_ENOMEM;
    }
    cudaMemsetAsync(w->S, 0, sizeof(CScalars), h->stream);
    HexDev d = h->hexdev();
    HC_CUDA_TRY(h, cudaMemsetAsync(w->dC, 0, n * 8, h->stream));
    HC_CUDA_TRY(h, cudaMemsetAsync(w->dM, 0, n * 8, h->stream));
    HC_CUDA_TRY(h, hex_diag_scaled(d, w->dC, 0.0, 1.0 / h->dt, h->stream));
    HC_CUDA_TRY(h, hex_diag_scaled(d, w->dM, 1.0, 0.0, h->stream));
  }
  if (w->omega != omega) {
    k_cinv_diag<<<cgrid(n), kRedThreads, 0, h->stream>>>(n, h->ess, w->dC, w->dM, omega, w->ir, w->ii, w->irf,
                                                         w->iif);
    HC_CUDA_TRY(h, cudaGetLastError());
    w->omega = omega;
  }
  return HC_OK;
}

// work vectors: FP64 path 8n doubles; mixed: 2n doubles (residual) + 2n
// floats (rhs) + 2n floats (correction) + 8n floats (COCG: r, p, q, z),
// then 8n doubles for the FP64 polish that follows a stalled refinement
static size_t polish_offset(int64_t n) { return (size_t)2 * n * sizeof(double) + (size_t)12 * n * 4; }
static hc_status complex_vectors(hcop* h) {
  ComplexWork* w = cwork(h);
  const int64_t n = h->ndof;
  const size_t need = polish_offset(n) + (size_t)8 * n * sizeof(double);
  if (w->vec_bytes >= need) return HC_OK;
  if (w->graph) cgraph_free(h, w);  // built on the old vectors
  dfree(h, w->vec);
  w->vec = nullptr;
  w->vec_bytes = 0;
  if (dmalloc(h, &w->vec, need) != cudaSuccess) {
    h->err = "complex work vectors allocation failed";
    return HC_ENOMEM;
  }
  w->vec_bytes = need;
  return HC_OK;
}

template <typename T>
static const T* cdr(ComplexWork* w);
template <>
const double* cdr<double>(ComplexWork* w) {
  return w->ir;
}
template <>
const float* cdr<float>(ComplexWork* w) {
  return w->irf;
}
template <typename T>
static const T* cdi(ComplexWork* w);
template <>
const double* cdi<double>(ComplexWork* w) {
  return w->ii;
}
template <>
const float* cdi<float>(ComplexWork* w) {
  return w->iif;
}

// One COCG solve's kernels: setup and one iteration, Jacobi (z formed on the
// fly) or auxiliary-space (z = D^-1 r + G V G^T r / (i omega), materialised).
// wk: 8 n-vectors of T: r, p, q, z (each re, im).
template <typename T>
struct CocgPlan {
  hcop* h;
  double omega;
  bool aux;
  T* wk;
  CScalars* S;
  int64_t n() const { return h->ndof; }
  T* r(int c) const { return wk + (0 + c) * n(); }
  T* p(int c) const { return wk + (2 + c) * n(); }
  T* q(int c) const { return wk + (4 + c) * n(); }
  T* z(int c) const { return wk + (6 + c) * n(); }
  const T* dr() const { return cdr<T>(cwork(h)); }
  const T* di() const { return cdi<T>(cwork(h)); }

  cudaError_t precond(cudaStream_t s) const {
    const int64_t nn = n();
    k_ca_jz<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, r(0), r(1), dr(), di(), z(0), z(1), S);
    const float io = (float)(1.0 / omega);
    const float coef[4] = {0.0f, io, -io, 0.0f};  // (0 - i/omega) (v0 + i v1)
    return auxmg_apply<T, 2>(h, r(0), r(1), z(0), z(1), coef, &S->done, s);
  }
  // r = b - A x (x_zero: r = b), first direction; skipped when active reads 0
  cudaError_t setup(const T* br, const T* bi, const T* xr, const T* xi, bool x_zero, const int* active,
                    cudaStream_t s, const int* apply_done = nullptr) const {
    const int64_t nn = n();
    if (!x_zero) {
      cudaError_t e = complex_apply_done<T>(h, omega, xr, xi, q(0), q(1), apply_done, s);
      if (e != cudaSuccess) return e;
    }
    const T* q0 = x_zero ? nullptr : q(0);
    const T* q1 = x_zero ? nullptr : q(1);
    if (!aux) {
      k_c_setup<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, br, bi, q0, q1, r(0), r(1), p(0), p(1), dr(), di(), S,
                                                      h->partials, active);
      return cudaGetLastError();
    }
    k_ca_setup<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, br, bi, q0, q1, r(0), r(1), S, h->partials, active);
    cudaError_t e = precond(s);
    if (e != cudaSuccess) return e;
    k_ca_rho<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, r(0), r(1), z(0), z(1), 1, S, h->partials);
    k_ca_dir<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, z(0), z(1), p(0), p(1), 1, S);
    return cudaGetLastError();
  }
  cudaError_t iterate(T* xr, T* xi, cudaStream_t s) const {
    const int64_t nn = n();
    cudaError_t e = complex_apply_done<T>(h, omega, p(0), p(1), q(0), q(1), &S->done, s);
    if (e != cudaSuccess) return e;
    k_c_alpha<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, p(0), p(1), q(0), q(1), S, h->partials);
    if (!aux) {
      k_c_update<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, xr, xi, r(0), r(1), p(0), p(1), q(0), q(1), dr(), di(), S,
                                                      h->partials);
      k_c_dir<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, r(0), r(1), dr(), di(), p(0), p(1), S);
      return cudaGetLastError();
    }
    k_ca_update<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, xr, xi, r(0), r(1), p(0), p(1), q(0), q(1), S,
                                                     h->partials);
    e = precond(s);
    if (e != cudaSuccess) return e;
    k_ca_rho<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, r(0), r(1), z(0), z(1), 0, S, h->partials);
    k_ca_dir<T><<<cgrid(nn), kRedThreads, 0, s>>>(nn, z(0), z(1), p(0), p(1), 0, S);
    return cudaGetLastError();
  }
};

// Host-driven COCG on A x = b (planar); wk: 8 n-vectors of T.
template <typename T>
static hc_status cocg_run(hcop* h, double omega, bool aux, double rtol, double atol, int maxit, const T* br,
                          const T* bi, T* xr, T* xi, bool x_zero, T* wk, int* iters) {
  ComplexWork* w = cwork(h);
  cudaStream_t s = h->stream;
  CScalars* S = w->S;
  CScalars* hs = w->hS;
  const CocgPlan<T> plan{h, omega, aux, wk, S};
  std::memset(hs, 0, sizeof(CScalars));
  hs->rtol2 = rtol * rtol;
  hs->atol2 = atol * atol;
  hs->maxit = maxit;
  HC_CUDA_TRY(h, cudaMemcpyAsync(S, hs, sizeof(CScalars), cudaMemcpyHostToDevice, s));
  HC_CUDA_TRY(h, plan.setup(br, bi, xr, xi, x_zero, nullptr, s));
  const int chunk = 20;
  int launched = 0;
  for (;;) {
    for (int k = 0; k < chunk && launched < maxit; ++k, ++launched) HC_CUDA_TRY(h, plan.iterate(xr, xi, s));
    HC_CUDA_TRY(h, cudaMemcpyAsync(hs, S, sizeof(CScalars), cudaMemcpyDeviceToHost, s));
    HC_CUDA_TRY(h, cudaStreamSynchronize(s));
    if (hs->done || launched >= maxit) break;
  }
  *iters = hs->it;
  return hs->done ? (hc_status)hs->status : HC_NOT_CONVERGED;
}

__global__ void k_c_resid64(int64_t n, const double* br, const double* bi, double* rr_, double* ri_, CScalars* S,
                            double* partials) {
  double v[2] = {0, 0}, tot[2];
  GS_LOOP(k, n) {
    const double a = br[k] - rr_[k], b = bi[k] - ri_[k];
    rr_[k] = a;
    ri_[k] = b;
    v[0] += a * a + b * b;
    v[1] += br[k] * br[k] + bi[k] * bi[k];
  }
  block_sum_n<2>(v);
  if (grid_sum_n<2>(v, partials, &S->counter[3], tot)) {
    S->rr = tot[0];
    S->bb = tot[1];
  }
}
__global__ void k_c_d2f(int64_t n, const double* a, const double* b, float* af, float* bf, double s) {
  GS_LOOP(k, n) {
    af[k] = (float)(a[k] * s);
    bf[k] = (float)(b[k] * s);
  }
}
__global__ void k_c_axpy(int64_t n, const float* cr, const float* ci, double* xr, double* xi, double s) {
  GS_LOOP(k, n) {
    xr[k] += s * (double)cr[k];
    xi[k] += s * (double)ci[k];
  }
}

hc_status complex_solve_device(hcop* h, const hc_solve_params* prm, double omega, const double* br,
                               const double* bi, double* xr, double* xi, hc_solve_info* info) {
  if (h->type != HC_HEX) {
    h->err = "complex solves: structured hex grids only in this build";
    return HC_ENOTSUP;
  }
  hc_status st = complex_prepare(h, omega);
  if (st != HC_OK) return st;
  st = complex_vectors(h);
  if (st != HC_OK) return st;
  const bool aux = prm->precond == HC_PRECOND_AUX;
  if (aux) {
    st = auxmg_setup(h);
    if (st != HC_OK) return st;
  }
  ComplexWork* w = cwork(h);
  const int64_t n = h->ndof;
  std::memset(info, 0, sizeof(*info));
  cudaStream_t s = h->stream;
  if (prm->precision == HC_FP64) {
    int it = 0;
    st = cocg_run<double>(h, omega, aux, prm->rtol, prm->atol, prm->maxit, br, bi, xr, xi, false, (double*)w->vec,
                          &it);
    info->status = st;
    info->iterations = it;
    info->outer_iterations = 1;
    info->rel_residual = w->hS->bb > 0 ? std::sqrt(w->hS->rr / w->hS->bb) : std::sqrt(w->hS->rr);
    return st;
  }
  // FP32 inner COCG inside FP64 refinement
  double* r64 = (double*)w->vec;
  double* i64 = r64 + n;
  float* rf = (float*)(i64 + n);
  float* if_ = rf + n;
  float* cr = if_ + n;
  float* ci = cr + n;
  float* wk = ci + n;
  const unsigned g = cgrid(n);
  int total = 0, outer = 0;
  auto residual = [&](double* rn2, double* bn2) -> hc_status {
    HC_CUDA_TRY(h, complex_apply<double>(h, omega, xr, xi, r64, i64, s));
    k_c_resid64<<<g, kRedThreads, 0, s>>>(n, br, bi, r64, i64, w->S, h->partials);
    HC_CUDA_TRY(h, cudaMemcpyAsync(w->hS, w->S, sizeof(CScalars), cudaMemcpyDeviceToHost, s));
    HC_CUDA_TRY(h, cudaStreamSynchronize(s));
    *rn2 = w->hS->rr;
    *bn2 = w->hS->bb;
    return HC_OK;
  };
  double rn2 = 0, bn2 = 0;
  st = residual(&rn2, &bn2);
  if (st != HC_OK) return st;
  const double bn = std::sqrt(bn2), tol = std::max(prm->rtol * bn, prm->atol);
  const double inner = prm->inner_rtol > 0 ? prm->inner_rtol : 1e-4;
  const int max_outer = prm->max_outer > 0 ? prm->max_outer : 50;
  hc_status result = HC_NOT_CONVERGED;
  // stalled refinement (a step that does not cut the residual by 4x): finish in FP64
  bool stalled = false;
  double rn_prev = 0.0;
  const int inner_cap = std::max(100, prm->maxit / 4);
  for (;;) {
    const double rn = std::sqrt(rn2);
    if (!std::isfinite(rn)) {
      result = HC_BREAKDOWN;
      break;
    }
    if (rn <= tol) {
      result = HC_OK;
      break;
    }
    if (outer >= max_outer || total >= prm->maxit) break;
    if (outer >= 2 && rn > 0.25 * rn_prev) {
      stalled = true;
      break;
    }
    rn_prev = rn;
    ++outer;
    k_c_d2f<<<g, kRedThreads, 0, s>>>(n, r64, i64, rf, if_, 1.0 / rn);
    HC_CUDA_TRY(h, cudaMemsetAsync(cr, 0, 2 * n * sizeof(float), s));  // x = 0 start
    int it = 0;
    hc_status ist = cocg_run<float>(h, omega, aux, inner, 0.0, std::min(prm->maxit - total, inner_cap), rf, if_, cr,
                                    ci, true, wk, &it);
    total += it;
    if (ist == HC_ECUDA || ist == HC_ENOMEM) return ist;
    k_c_axpy<<<g, kRedThreads, 0, s>>>(n, cr, ci, xr, xi, rn);
    HC_CUDA_TRY(h, cudaGetLastError());
    st = residual(&rn2, &bn2);
    if (st != HC_OK) return st;
    if (ist == HC_BREAKDOWN && it == 0) {
      result = HC_BREAKDOWN;
      break;
    }
  }
  if (stalled && total < prm->maxit) {
    int it = 0;
    double* wk64 = (double*)((char*)w->vec + polish_offset(n));
    const hc_status pst = cocg_run<double>(h, omega, aux, prm->rtol, prm->atol, prm->maxit - total, br, bi, xr, xi,
                                           false, wk64, &it);
    total += it;
    ++outer;
    if (pst == HC_ECUDA || pst == HC_ENOMEM) return pst;
    st = residual(&rn2, &bn2);
    if (st != HC_OK) return st;
    // the FP64 Krylov's own verdict (recursive residual), as for a plain FP64 solve
    result = std::isfinite(std::sqrt(rn2)) ? pst : HC_BREAKDOWN;
  }
  info->status = result;
  info->iterations = total;
  info->outer_iterations = outer;
  info->rel_residual = bn > 0 ? std::sqrt(rn2) / bn : std::sqrt(rn2);
  return result;
}

}  // namespace hc

namespace hc {
hc_status complex_graph_launch(hcop* h, const hc_solve_params* prm, double omega, const double* br,
                               const double* bi, double* xr, double* xi, int chunk);
hc_status complex_graph_result(hcop* h, hc_solve_info* info);
}  // namespace hc

using namespace hc;

// ---- C entry points -------------------------------------------------------------------
static hc_status complex_check(hcop* h, double omega) {
  if (h->type != HC_HEX) {
    h->err = "complex operator: structured hex grids only in this build";
    return HC_ENOTSUP;
  }
  if (!std::isfinite(omega) || omega < 0.0) {
    h->err = "complex operator: omega must be finite and >= 0";
    return HC_EINVAL;
  }
  return HC_OK;
}

extern "C" {

hc_status hc_mult_complex_device(hcop_t* h, double omega, const double* xr, const double* xi, double* yr,
                                 double* yi) {
  if (!h || !xr || !xi || !yr || !yi) return HC_EINVAL;
  hc_status st = complex_check(h, omega);
  if (st != HC_OK) return st;
  HC_CUDA_TRY(h, complex_apply<double>(h, omega, xr, xi, yr, yi, h->stream));
  return HC_OK;
}

hc_status hc_mult_complex_device_f32(hcop_t* h, double omega, const float* xr, const float* xi, float* yr,
                                     float* yi) {
  if (!h || !xr || !xi || !yr || !yi) return HC_EINVAL;
  hc_status st = complex_check(h, omega);
  if (st != HC_OK) return st;
  HC_CUDA_TRY(h, complex_apply<float>(h, omega, xr, xi, yr, yi, h->stream));
  return HC_OK;
}

// Host vectors: x = [xr | xi] and y = [yr | yi], each 2 n_dof doubles (the
// real-then-imaginary block layout of MFEM's ComplexOperator).
hc_status hc_mult_complex(hcop_t* h, double omega, const double* x, double* y) {
  if (!h || !x || !y) return HC_EINVAL;
  hc_status st = complex_check(h, omega);
  if (st != HC_OK) return st;
  const int64_t n = h->ndof;
  double* d = nullptr;
  HC_CUDA_TRY(h, cudaMallocAsync((void**)&d, 4 * n * sizeof(double), h->stream));
  cudaError_t e = cudaMemcpyAsync(d, x, 2 * n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = complex_apply<double>(h, omega, d, d + n, d + 2 * n, d + 3 * n, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(y, d + 2 * n, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  cudaFreeAsync(d, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    h->err = std::string("hc_mult_complex: ") + cudaGetErrorString(e);
    return HC_ECUDA;
  }
  return HC_OK;
}

static hc_status complex_params(hcop* h, const hc_solve_params* p) {
  if (!p) {
    h->err = "null solve parameters";
    return HC_EINVAL;
  }
  if (p->precision != HC_FP64 && p->precision != HC_MIXED && p->precision != HC_MIXED_RR) {
    h->err = "precision must be HC_FP64, HC_MIXED or HC_MIXED_RR";
    return HC_EINVAL;
  }
  if (p->precond != HC_PRECOND_JACOBI && p->precond != HC_PRECOND_AUX) {
    h->err = "complex solves take the complex Jacobi or the auxiliary-space (Jacobi + gradient) preconditioner";
    return HC_ENOTSUP;
  }
  if (!(p->rtol >= 0.0) || !(p->atol >= 0.0) || p->maxit < 1) {
    h->err = "rtol, atol must be >= 0 and maxit >= 1";
    return HC_EINVAL;
  }
  return HC_OK;
}

hc_status hc_solve_complex_device(hcop_t* h, const hc_solve_params* prm, double omega, const double* br,
                                  const double* bi, double* xr, double* xi, hc_solve_info* info) {
  if (!h || !br || !bi || !xr || !xi) return HC_EINVAL;
  hc_status st = complex_check(h, omega);
  if (st == HC_OK) st = complex_params(h, prm);
  if (st != HC_OK) return st;
  hc_solve_info loc{};
  if (prm->precision == HC_MIXED_RR) {  // residual replacement is built in the graph-driven solve
    st = complex_graph_launch(h, prm, omega, br, bi, xr, xi, 0);
    if (st != HC_OK) return st;
    return complex_graph_result(h, info ? info : &loc);
  }
  return complex_solve_device(h, prm, omega, br, bi, xr, xi, info ? info : &loc);
}

hc_status hc_solve_complex(hcop_t* h, const hc_solve_params* prm, double omega, const double* b, double* x,
                           hc_solve_info* info) {
  if (!h || !b || !x) return HC_EINVAL;
  hc_status st = complex_check(h, omega);
  if (st == HC_OK) st = complex_params(h, prm);
  if (st != HC_OK) return st;
  const int64_t n = h->ndof;
  double* d = nullptr;
  HC_CUDA_TRY(h, cudaMallocAsync((void**)&d, 4 * n * sizeof(double), h->stream));
  cudaError_t e = cudaMemcpyAsync(d, b, 2 * n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d + 2 * n, x, 2 * n * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  hc_status sst = HC_ECUDA;
  if (e == cudaSuccess) {
    hc_solve_info loc{};
    if (prm->precision == HC_MIXED_RR) {
      sst = complex_graph_launch(h, prm, omega, d, d + n, d + 2 * n, d + 3 * n, 0);
      if (sst == HC_OK) sst = complex_graph_result(h, info ? info : &loc);
    } else {
      sst = complex_solve_device(h, prm, omega, d, d + n, d + 2 * n, d + 3 * n, info ? info : &loc);
    }
  }
  if (e == cudaSuccess && sst != HC_ECUDA && sst != HC_ENOMEM)
    e = cudaMemcpyAsync(x, d + 2 * n, 2 * n * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
  cudaFreeAsync(d, h->stream);
  cudaError_t e2 = cudaStreamSynchronize(h->stream);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) {
    h->err = std::string("hc_solve_complex: ") + cudaGetErrorString(e);
    return HC_ECUDA;
  }
  return sst;
}

hc_status hc_solve_complex_graph(hcop_t* h, const hc_solve_params* prm, double omega, const double* br,
                                 const double* bi, double* xr, double* xi) {
  if (!h || !br || !bi || !xr || !xi) return HC_EINVAL;
  hc_status st = complex_check(h, omega);
  if (st == HC_OK) st = complex_params(h, prm);
  if (st != HC_OK) return st;
  return complex_graph_launch(h, prm, omega, br, bi, xr, xi, 0);
}

hc_status hc_graph_solve_info(hcop_t* h, hc_solve_info* info) {
  if (!h || !info) return HC_EINVAL;
  return complex_graph_result(h, info);
}

hc_status hc_solve_complex_batch(int32_t n, hcop_t* const* hs, const hc_solve_params* prm, const double* omega,
                                 const double* const* br, const double* const* bi, double* const* xr,
                                 double* const* xi, hc_solve_info* info) {
  if (n < 0 || (n > 0 && (!hs || !prm || !omega || !br || !bi || !xr || !xi || !info))) return HC_EINVAL;
  hc_status first = HC_OK;
  for (int32_t i = 0; i < n; ++i) {
    std::memset(&info[i], 0, sizeof(hc_solve_info));
    const hc_status st = hc_solve_complex_graph(hs[i], prm, omega[i], br[i], bi[i], xr[i], xi[i]);
    if (st != HC_OK) {
      info[i].status = st;
      if (first == HC_OK) first = st;
    }
  }
  for (int32_t i = 0; i < n; ++i) {
    if (info[i].status != HC_OK) continue;  // not launched
    const hc_status st = hc_graph_solve_info(hs[i], &info[i]);
    info[i].status = st;
    if (st != HC_OK && first == HC_OK) first = st;
  }
  return first;
}

}  // extern "C"

namespace hc {
// ---- graph-driven solves ----------------------------------------------------------------
// The same COCG (and refinement) as above, built once per argument set into
// one CUDA graph whose loops are conditional WHILE nodes.  Stopping decisions
// are taken on the device; every loop has a hard trip bound.
struct CRefine {
  double rn, bn, tol, rtol, atol, rn_prev;
  int outer, total, max_outer, maxit, status, active, trips, polish;
  // residual replacement (HC_MIXED_RR): FP32 units of the initial residual,
  // recursive |r|^2 at the last replacement, replacement threshold
  double scale, rr_last, delta2, rr_rec;
  int since, slow, stop, flat;
};

__global__ void k_g_init(CScalars* S, double rtol2, double atol2, int maxit) {
  S->rtol2 = rtol2;
  S->atol2 = atol2;
  S->maxit = maxit;
  S->trips = 0;
}

// end of a COCG WHILE body: continue while not done and under the trip bound
__global__ void k_c_cond(CScalars* S, cudaGraphConditionalHandle hnd, int max_trips) {
  const int t = ++S->trips;
  const int go = (!S->done && t < max_trips) ? 1 : 0;
  if (!go && !S->done) {
    S->done = 1;
    S->status = HC_NOT_CONVERGED;
  }
  cudaGraphSetConditional(hnd, (unsigned)go);
}

__global__ void k_r_init(CRefine* R, double rtol, double atol, int maxit, int max_outer) {
  R->rtol = rtol;
  R->atol = atol;
  R->tol = -1.0;
  R->rn = R->bn = 0.0;
  R->maxit = maxit;
  R->max_outer = max_outer;
  R->outer = R->total = R->trips = R->active = R->polish = 0;
  R->rn_prev = 0.0;
  R->status = HC_NOT_CONVERGED;
}

// refinement step decision from the FP64 residual in S->rr (and |b|^2 in S->bb)
__global__ void k_r_check(CRefine* R, const CScalars* S, cudaGraphConditionalHandle hnd, int max_trips) {
  const double rn = sqrt(S->rr);
  if (R->tol < 0.0) {
    R->bn = sqrt(S->bb);
    R->tol = fmax(R->rtol * R->bn, R->atol);
  }
  const int t = ++R->trips;
  int stop = 1;
  if (R->status == HC_BREAKDOWN) {
  } else if (!isfinite(rn)) {
    R->status = HC_BREAKDOWN;
  } else if (rn <= R->tol) {
    R->status = HC_OK;
  } else if (R->outer >= R->max_outer || R->total >= R->maxit || t >= max_trips) {
    R->status = HC_NOT_CONVERGED;
  } else if (R->outer >= 2 && rn > 0.25 * R->rn_prev) {
    // the FP32 inner solves stopped paying: finish in FP64
    R->status = HC_NOT_CONVERGED;
    R->polish = 1;
  } else {
    stop = 0;
  }
  R->rn_prev = rn;
  R->rn = rn;
  R->active = !stop;
  if (!stop) R->outer += 1;
  cudaGraphSetConditional(hnd, stop ? 0u : 1u);
}

// rf = r / |r| in FP32, correction = 0
__global__ void k_r_d2f(int64_t n, const CRefine* R, const double* a, const double* b, float* af, float* bf,
                        float* cr, float* ci) {
  if (!R->active) return;
  const double s = 1.0 / R->rn;
  GS_LOOP(k, n) {
    af[k] = (float)(a[k] * s);
    bf[k] = (float)(b[k] * s);
    cr[k] = 0.0f;
    ci[k] = 0.0f;
  }
}

__global__ void k_r_inner_init(CScalars* S, const CRefine* R, double rtol2, cudaGraphConditionalHandle hnd) {
  S->rtol2 = rtol2;
  S->atol2 = 0.0;
  S->maxit = R->maxit - R->total;
  S->trips = 0;
  if (!R->active) S->done = 1;
  cudaGraphSetConditional(hnd, R->active ? 1u : 0u);
}

// FP64 polish after a stalled refinement: scalars for a COCG from the current x
__global__ void k_polish_init(CScalars* S, CRefine* R, double rtol2, double atol2, cudaGraphConditionalHandle hnd) {
  const int go = (R->polish && R->total < R->maxit) ? 1 : 0;
  R->polish = go;
  S->rtol2 = rtol2;
  S->atol2 = atol2;
  S->maxit = R->maxit - R->total;
  S->trips = 0;
  S->done = go ? 0 : 1;
  cudaGraphSetConditional(hnd, (unsigned)go);
}
__global__ void k_polish_finish(CRefine* R, const CScalars* S) {
  if (!R->polish) return;
  R->total += S->it;
  R->outer += 1;
  R->status = S->status;
  R->rn = sqrt(S->rr);
}

// x += |r| c
__global__ void k_r_accum(int64_t n, CRefine* R, const CScalars* S, const float* cr, const float* ci, double* xr,
                          double* xi) {
  if (!R->active) return;
  const double s = R->rn;
  GS_LOOP(k, n) {
    xr[k] += s * (double)cr[k];
    xi[k] += s * (double)ci[k];
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    R->total += S->it;
    if (S->status == HC_BREAKDOWN && S->it == 0) R->status = HC_BREAKDOWN;
  }
}

// ---- residual replacement in the graph-driven COCG (HC_MIXED_RR) ----------------------
// One FP32 COCG runs through; at the end of a batch of iterations where its
// recursive residual fell by delta since the last replacement, met its
// tolerance, or 8 batches passed, an IF node adds the FP32 correction to the
// FP64 x, computes b - J x in FP64 and puts it (in units of the initial
// residual) in place of the FP32 recursive residual; direction and r^T z are
// kept (van der Vorst & Ye residual replacement, as in the real solver).
__global__ void k_rr_start(CRefine* R, CScalars* S, double delta2, cudaGraphConditionalHandle hl) {
  const double rn = sqrt(S->rr);
  R->bn = sqrt(S->bb);
  R->tol = fmax(R->rtol * R->bn, R->atol);
  R->rn = rn;
  R->rn_prev = rn;
  R->scale = rn > 0.0 ? rn : 1.0;
  R->rr_last = 1.0;
  R->delta2 = delta2;
  R->since = R->slow = R->stop = R->flat = 0;
  R->rr_rec = 1.0;
  int go = 1;
  if (!isfinite(rn)) {
    R->status = HC_BREAKDOWN;
    go = 0;
  } else if (rn <= R->tol) {
    R->status = HC_OK;
    go = 0;
  }
  R->active = go;
  R->stop = !go;
  // the FP32 COCG's stopping test, relative to |r0 / scale| = 1
  const double t = 0.5 * R->tol / R->scale;
  S->rtol2 = t * t;
  S->atol2 = 0.0;
  S->maxit = R->maxit;
  S->trips = 0;
  S->done = go ? 0 : 1;
  cudaGraphSetConditional(hl, (unsigned)go);
}

// end of a batch: is a replacement due?
__global__ void k_rr_due(CRefine* R, const CScalars* S, cudaGraphConditionalHandle hif) {
  int due = 0;
  if (!(S->done && S->status == HC_BREAKDOWN)) {
    ++R->since;
    due = S->done || S->rr <= R->delta2 * R->rr_last || R->since >= 8;
  }
  if (due) {
    R->since = 0;
    R->rr_rec = S->rr;  // the recursive residual the replacement is about to overwrite
  }
  cudaGraphSetConditional(hif, (unsigned)due);
}

// x += scale c, c = 0
__global__ void k_rr_fold(int64_t n, const CRefine* R, float* cr, float* ci, double* xr, double* xi) {
  const double s = R->scale;
  GS_LOOP(k, n) {
    xr[k] += s * (double)cr[k];
    xi[k] += s * (double)ci[k];
    cr[k] = 0.0f;
    ci[k] = 0.0f;
  }
}

// decision from the FP64 residual (S->rr = |b - J x|^2 from k_c_resid64)
__global__ void k_rr_after(CRefine* R, CScalars* S) {
  const double rn = sqrt(S->rr);
  R->rn = rn;
  R->total = S->it;
  R->outer += 1;
  if (!isfinite(rn)) {
    R->status = HC_BREAKDOWN;
    R->stop = 1;
  } else if (rn <= R->tol) {
    R->status = HC_OK;
    R->stop = 1;
  } else if (S->it >= S->maxit) {
    R->status = HC_NOT_CONVERGED;
    R->stop = 1;
  } else {
    // FP32 floor: the true residual no longer halves while the recursive one
    // runs ahead of it (10x in norm).  COCG's residual also has plateaus
    // where both stall together: those are not a floor, but six of them in a
    // row end the FP32 iteration too.
    const double tr = rn / R->scale;
    const bool drift = tr * tr > 100.0 * R->rr_rec;
    const bool flat = rn > 0.5 * R->rn_prev;
    R->slow = (flat && drift) ? R->slow + 1 : 0;
    R->flat = flat ? R->flat + 1 : 0;
    R->rn_prev = rn;
    if (R->slow >= 2 || R->flat >= 6) {  // the FP32 iteration stopped paying: finish in FP64
      R->status = HC_NOT_CONVERGED;
      R->polish = 1;
      R->stop = 1;
    }
  }
  if (R->stop) {
    S->done = 1;
    return;
  }
  const double rr = S->rr / (R->scale * R->scale);
  S->rr = rr;
  S->done = 0;
  S->status = HC_NOT_CONVERGED;
  R->rr_last = rr;
}

// the FP32 recursive residual := (b - J x) / scale
__global__ void k_rr_d2f(int64_t n, const CRefine* R, const double* a, const double* b, float* af, float* bf) {
  if (R->stop) return;
  const double s = 1.0 / R->scale;
  GS_LOOP(k, n) {
    af[k] = (float)(a[k] * s);
    bf[k] = (float)(b[k] * s);
  }
}

// after the loop: a batch that ended on the iteration cap or a breakdown
// without a replacement leaves its correction in c; its true residual decides
__global__ void k_rr_final(CRefine* R, const CScalars* S) {
  const double rn = sqrt(S->rr);
  if (!R->stop) {
    R->rn = rn;
    R->total = S->it;
    R->status = !isfinite(rn) ? HC_BREAKDOWN : (rn <= R->tol ? HC_OK : (S->status == HC_BREAKDOWN ? HC_BREAKDOWN
                                                                                                 : HC_NOT_CONVERGED));
    R->stop = 1;
  }
}

struct ComplexGraph {
  cudaGraphExec_t exec = nullptr;
  cudaStream_t cap = nullptr;
  CRefine* R = nullptr;
  CRefine* hR = nullptr;
  // arguments the graph was built for
  int precision = -1, precond = -1, maxit = 0, max_outer = 0, chunk = 0;
  double omega = 0, rtol = 0, atol = 0, inner = 0;
  const void* ptr[4] = {nullptr, nullptr, nullptr, nullptr};
};

static ComplexGraph* cgraph(hcop* h) {
  ComplexWork* w = cwork(h);
  if (!w->graph) w->graph = new ComplexGraph();
  return static_cast<ComplexGraph*>(w->graph);
}

static void cgraph_free(hcop* h, ComplexWork* w) {
  ComplexGraph* g = static_cast<ComplexGraph*>(w->graph);
  if (!g) return;
  cudaStreamSynchronize(h->stream);  // no launch of this graph may still be pending
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->cap) cudaStreamDestroy(g->cap);
  dfree(h, g->R);
  pinned_put(g->hR);
  delete g;
  w->graph = nullptr;
}

static hc_status complex_graph_build(hcop* h, const hc_solve_params* prm, double omega, const double* br,
                                     const double* bi, double* xr, double* xi, int chunk) {
  ComplexWork* w = cwork(h);
  ComplexGraph* G = cgraph(h);
  const int64_t n = h->ndof;
  if (!G->cap) HC_CUDA_TRY(h, cudaStreamCreateWithFlags(&G->cap, cudaStreamNonBlocking));
  if (!G->R) {
    HC_CUDA_TRY(h, dmalloc(h, (void**)&G->R, sizeof(CRefine)));
    G->hR = static_cast<CRefine*>(pinned_get(sizeof(CRefine)));
    if (!G->hR) {
      h->err = "pinned scalar allocation failed";
      return HC_ENOMEM;
    }
  }
  if (G->exec) {
    cudaGraphExecDestroy(G->exec);
    G->exec = nullptr;
  }
  CScalars* S = w->S;
  const int unit = prm->maxit / chunk + 3;  // trip bound of one COCG loop
  cudaGraph_t top = nullptr;
  HC_CUDA_TRY(h, cudaGraphCreate(&top, 0));
  GraphChain c{top, nullptr};
  cudaError_t e = cudaSuccess;
  const bool aux = prm->precond == HC_PRECOND_AUX;
  if (prm->precision == HC_FP64) {
    const CocgPlan<double> plan{h, omega, aux, (double*)w->vec, S};
    e = chain_segment(c, G->cap, [&](cudaStream_t s) {
      k_g_init<<<1, 1, 0, s>>>(S, prm->rtol * prm->rtol, prm->atol * prm->atol, prm->maxit);
      return plan.setup(br, bi, xr, xi, false, nullptr, s);
    });
    cudaGraphConditionalHandle hl = 0;
    GraphChain body;
    if (e == cudaSuccess) e = chain_handle(c, &hl);
    if (e == cudaSuccess) e = chain_while(c, hl, &body);
    if (e == cudaSuccess)
      e = chain_segment(body, G->cap, [&](cudaStream_t s) {
        for (int k = 0; k < chunk; ++k) {
          cudaError_t ee = plan.iterate(xr, xi, s);
          if (ee != cudaSuccess) return ee;
        }
        k_c_cond<<<1, 1, 0, s>>>(S, hl, unit);
        return cudaGetLastError();
      });
  } else if (prm->precision == HC_MIXED_RR) {
    double* r64 = (double*)w->vec;
    double* i64 = r64 + n;
    float* rf = (float*)(i64 + n);
    float* if_ = rf + n;
    float* cr = if_ + n;
    float* ci = cr + n;
    const CocgPlan<float> plan{h, omega, aux, ci + n, S};
    CRefine* R = G->R;
    const double delta = prm->inner_rtol > 0 ? std::min(prm->inner_rtol, 0.5) : 0.1;
    const int max_outer = prm->max_outer > 0 ? prm->max_outer : 50;
    cudaGraphConditionalHandle hl = 0, hif = 0;
    GraphChain body, rep;
    if (e == cudaSuccess) e = chain_handle(c, &hl);
    if (e == cudaSuccess)
      e = chain_segment(c, G->cap, [&](cudaStream_t s) {
        k_r_init<<<1, 1, 0, s>>>(R, prm->rtol, prm->atol, prm->maxit, max_outer);
        cudaError_t ee = complex_apply_done<double>(h, omega, xr, xi, r64, i64, nullptr, s);
        if (ee != cudaSuccess) return ee;
        k_c_resid64<<<cgrid(n), kRedThreads, 0, s>>>(n, br, bi, r64, i64, S, h->partials);
        k_rr_start<<<1, 1, 0, s>>>(R, S, delta * delta, hl);
        // rf = r / |r|, c = 0 (scale = |r| = R->rn at the start)
        k_r_d2f<<<cgrid(n), kRedThreads, 0, s>>>(n, R, r64, i64, rf, if_, cr, ci);
        return plan.setup(rf, if_, nullptr, nullptr, true, &R->active, s);
      });
    if (e == cudaSuccess) e = chain_while(c, hl, &body);
    if (e == cudaSuccess) e = chain_handle(body, &hif);
    if (e == cudaSuccess)
      e = chain_segment(body, G->cap, [&](cudaStream_t s) {
        for (int k = 0; k < chunk; ++k) {
          cudaError_t ee = plan.iterate(cr, ci, s);
          if (ee != cudaSuccess) return ee;
        }
        k_rr_due<<<1, 1, 0, s>>>(R, S, hif);
        return cudaGetLastError();
      });
    if (e == cudaSuccess) e = chain_if(body, hif, &rep);
    if (e == cudaSuccess)
      e = chain_segment(rep, G->cap, [&](cudaStream_t s) {
        k_rr_fold<<<cgrid(n), kRedThreads, 0, s>>>(n, R, cr, ci, xr, xi);
        cudaError_t ee = complex_apply_done<double>(h, omega, xr, xi, r64, i64, nullptr, s);
        if (ee != cudaSuccess) return ee;
        k_c_resid64<<<cgrid(n), kRedThreads, 0, s>>>(n, br, bi, r64, i64, S, h->partials);
        k_rr_after<<<1, 1, 0, s>>>(R, S);
        k_rr_d2f<<<cgrid(n), kRedThreads, 0, s>>>(n, R, r64, i64, plan.r(0), plan.r(1));
        return cudaGetLastError();
      });
    if (e == cudaSuccess)
      e = chain_segment(body, G->cap, [&](cudaStream_t s) {
        k_c_cond<<<1, 1, 0, s>>>(S, hl, unit);
        return cudaGetLastError();
      });
    // the correction of a loop that ended without a replacement, and the true residual
    if (e == cudaSuccess)
      e = chain_segment(c, G->cap, [&](cudaStream_t s) {
        k_rr_fold<<<cgrid(n), kRedThreads, 0, s>>>(n, R, cr, ci, xr, xi);
        cudaError_t ee = complex_apply_done<double>(h, omega, xr, xi, r64, i64, nullptr, s);
        if (ee != cudaSuccess) return ee;
        k_c_resid64<<<cgrid(n), kRedThreads, 0, s>>>(n, br, bi, r64, i64, S, h->partials);
        k_rr_final<<<1, 1, 0, s>>>(R, S);
        return cudaGetLastError();
      });
    // FP64 polish (runs only when the FP32 iteration stalled)
    const CocgPlan<double> p64{h, omega, aux, (double*)((char*)w->vec + polish_offset(n)), S};
    cudaGraphConditionalHandle hp = 0;
    GraphChain pb;
    if (e == cudaSuccess) e = chain_handle(c, &hp);
    if (e == cudaSuccess)
      e = chain_segment(c, G->cap, [&](cudaStream_t s) {
        k_polish_init<<<1, 1, 0, s>>>(S, R, prm->rtol * prm->rtol, prm->atol * prm->atol, hp);
        return p64.setup(br, bi, xr, xi, false, &R->polish, s, &S->done);
      });
    if (e == cudaSuccess) e = chain_while(c, hp, &pb);
    if (e == cudaSuccess)
      e = chain_segment(pb, G->cap, [&](cudaStream_t s) {
        for (int k = 0; k < chunk; ++k) {
          cudaError_t ee = p64.iterate(xr, xi, s);
          if (ee != cudaSuccess) return ee;
        }
        k_c_cond<<<1, 1, 0, s>>>(S, hp, unit);
        return cudaGetLastError();
      });
    if (e == cudaSuccess)
      e = chain_segment(c, G->cap, [&](cudaStream_t s) {
        k_polish_finish<<<1, 1, 0, s>>>(R, S);
        return cudaMemcpyAsync(G->hR, R, sizeof(CRefine), cudaMemcpyDeviceToHost, s);
      });
  } else {
    double* r64 = (double*)w->vec;
    double* i64 = r64 + n;
    float* rf = (float*)(i64 + n);
    float* if_ = rf + n;
    float* cr = if_ + n;
    float* ci = cr + n;
    const CocgPlan<float> plan{h, omega, aux, ci + n, S};
    CRefine* R = G->R;
    const double inner = prm->inner_rtol > 0 ? prm->inner_rtol : 1e-4;
    const int max_outer = prm->max_outer > 0 ? prm->max_outer : 50;
    e = chain_segment(c, G->cap, [&](cudaStream_t s) {
      k_r_init<<<1, 1, 0, s>>>(R, prm->rtol, prm->atol, prm->maxit, max_outer);
      return cudaGetLastError();
    });
    cudaGraphConditionalHandle ho = 0, hi = 0;
    GraphChain ob, ib;
    if (e == cudaSuccess) e = chain_handle(c, &ho);
    if (e == cudaSuccess) e = chain_while(c, ho, &ob);
    if (e == cudaSuccess) e = chain_handle(ob, &hi);
    if (e == cudaSuccess)
      e = chain_segment(ob, G->cap, [&](cudaStream_t s) {
        cudaError_t ee = complex_apply_done<double>(h, omega, xr, xi, r64, i64, nullptr, s);
        if (ee != cudaSuccess) return ee;
        k_c_resid64<<<cgrid(n), kRedThreads, 0, s>>>(n, br, bi, r64, i64, S, h->partials);
        k_r_check<<<1, 1, 0, s>>>(R, S, ho, max_outer + 2);
        k_r_d2f<<<cgrid(n), kRedThreads, 0, s>>>(n, R, r64, i64, rf, if_, cr, ci);
        k_r_inner_init<<<1, 1, 0, s>>>(S, R, inner * inner, hi);
        return plan.setup(rf, if_, nullptr, nullptr, true, &R->active, s);
      });
    if (e == cudaSuccess) e = chain_while(ob, hi, &ib);
    if (e == cudaSuccess)
      e = chain_segment(ib, G->cap, [&](cudaStream_t s) {
        for (int k = 0; k < chunk; ++k) {
          cudaError_t ee = plan.iterate(cr, ci, s);
          if (ee != cudaSuccess) return ee;
        }
        k_c_cond<<<1, 1, 0, s>>>(S, hi, unit);
        return cudaGetLastError();
      });
    if (e == cudaSuccess)
      e = chain_segment(ob, G->cap, [&](cudaStream_t s) {
        k_r_accum<<<cgrid(n), kRedThreads, 0, s>>>(n, R, S, cr, ci, xr, xi);
        return cudaGetLastError();
      });
    // FP64 polish (runs only when the refinement stalled)
    const CocgPlan<double> p64{h, omega, aux, (double*)((char*)w->vec + polish_offset(n)), S};
    cudaGraphConditionalHandle hp = 0;
    GraphChain pb;
    if (e == cudaSuccess) e = chain_handle(c, &hp);
    if (e == cudaSuccess)
      e = chain_segment(c, G->cap, [&](cudaStream_t s) {
        k_polish_init<<<1, 1, 0, s>>>(S, R, prm->rtol * prm->rtol, prm->atol * prm->atol, hp);
        return p64.setup(br, bi, xr, xi, false, &R->polish, s, &S->done);
      });
    if (e == cudaSuccess) e = chain_while(c, hp, &pb);
    if (e == cudaSuccess)
      e = chain_segment(pb, G->cap, [&](cudaStream_t s) {
        for (int k = 0; k < chunk; ++k) {
          cudaError_t ee = p64.iterate(xr, xi, s);
          if (ee != cudaSuccess) return ee;
        }
        k_c_cond<<<1, 1, 0, s>>>(S, hp, unit);
        return cudaGetLastError();
      });
    if (e == cudaSuccess)
      e = chain_segment(c, G->cap, [&](cudaStream_t s) {
        k_polish_finish<<<1, 1, 0, s>>>(R, S);
        return cudaMemcpyAsync(G->hR, R, sizeof(CRefine), cudaMemcpyDeviceToHost, s);
      });
  }
  if (e == cudaSuccess)
    e = chain_segment(c, G->cap, [&](cudaStream_t s) {
      return cudaMemcpyAsync(w->hS, S, sizeof(CScalars), cudaMemcpyDeviceToHost, s);
    });
  if (e == cudaSuccess) e = cudaGraphInstantiate(&G->exec, top, 0);
  cudaGraphDestroy(top);
  if (e != cudaSuccess) {
    G->exec = nullptr;
    h->err = std::string("solve graph construction failed: ") + cudaGetErrorString(e);
    return HC_ECUDA;
  }
  G->precision = prm->precision;
  G->precond = prm->precond;
  G->maxit = prm->maxit;
  G->max_outer = prm->max_outer;
  G->chunk = chunk;
  G->omega = omega;
  G->rtol = prm->rtol;
  G->atol = prm->atol;
  G->inner = prm->inner_rtol;
  G->ptr[0] = br;
  G->ptr[1] = bi;
  G->ptr[2] = xr;
  G->ptr[3] = xi;
  return HC_OK;
}

static int default_chunk(int64_t n) { return n < 200000 ? 16 : 8; }

hc_status complex_graph_launch(hcop* h, const hc_solve_params* prm, double omega, const double* br,
                               const double* bi, double* xr, double* xi, int chunk) {
  if (h->type != HC_HEX) {
    h->err = "complex solves: structured hex grids only in this build";
    return HC_ENOTSUP;
  }
  hc_status st = complex_prepare(h, omega);
  if (st != HC_OK) return st;
  st = complex_vectors(h);
  if (st != HC_OK) return st;
  if (prm->precond == HC_PRECOND_AUX) {
    st = auxmg_setup(h);
    if (st != HC_OK) return st;
  }
  if (chunk <= 0) chunk = default_chunk(h->ndof);
  ComplexGraph* G = cgraph(h);
  const bool same = G->exec && G->precision == prm->precision && G->precond == prm->precond &&
                    G->maxit == prm->maxit &&
                    G->max_outer == prm->max_outer && G->chunk == chunk && G->omega == omega && G->rtol == prm->rtol &&
                    G->atol == prm->atol && G->inner == prm->inner_rtol && G->ptr[0] == br && G->ptr[1] == bi &&
                    G->ptr[2] == xr && G->ptr[3] == xi;
  if (!same) {
    // warm the launch-shape caches outside of capture
    HC_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    st = complex_graph_build(h, prm, omega, br, bi, xr, xi, chunk);
    if (st != HC_OK) return st;
  }
  HC_CUDA_TRY(h, cudaGraphLaunch(G->exec, h->stream));
  return HC_OK;
}

hc_status complex_graph_result(hcop* h, hc_solve_info* info) {
  ComplexWork* w = static_cast<ComplexWork*>(h->cwork);
  ComplexGraph* G = w ? static_cast<ComplexGraph*>(w->graph) : nullptr;
  if (!G || !G->exec) {
    h->err = "no graph-driven solve has been launched on this handle";
    return HC_EINVAL;
  }
  HC_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  std::memset(info, 0, sizeof(*info));
  const CScalars* hs = w->hS;
  if (G->precision == HC_FP64) {
    info->status = hs->status;
    info->iterations = hs->it;
    info->outer_iterations = 1;
    info->rel_residual = hs->bb > 0 ? std::sqrt(hs->rr / hs->bb) : std::sqrt(hs->rr);
  } else {
    const CRefine* R = G->hR;
    info->status = R->status;
    info->iterations = R->total;
    info->outer_iterations = R->outer;
    info->rel_residual = R->bn > 0 ? R->rn / R->bn : R->rn;
  }
  return (hc_status)info->status;
}

template cudaError_t complex_apply<double>(hcop*, double, const double*, const double*, double*, double*,
                                           cudaStream_t);
template cudaError_t complex_apply<float>(hcop*, double, const float*, const float*, float*, float*, cudaStream_t);

}  // namespace hc

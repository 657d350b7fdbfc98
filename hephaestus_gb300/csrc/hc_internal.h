// hc_internal.h -- shared declarations of the GB300 H(curl) operator library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "hcurl_op.h"

namespace hc {

constexpr int kMaxP = 3;             // hex orders 1..3
constexpr int kRedBlocks = 304;      // 2 x 152 SMs: blocks of every grid-stride vector kernel
constexpr int kRedThreads = 512;
constexpr int kMaxLanczos = 64;

// 1-D operators of the hex element on [0,1]: closed (Gauss-Lobatto nodal, p+1
// functions) and open (Gauss-Legendre nodal, p functions) bases.
//   Mcc[i][j] = int phi^c_i phi^c_j,  Mco[i][j] = int phi^c_i phi^o_j,
//   Moo[i][j] = int phi^o_i phi^o_j,  D[a][j] = (phi^c_j)'(x^o_a)
// D expands the derivative of a closed function in the open basis exactly.
template <typename T>
struct Tab1D {
  T Mcc[kMaxP + 1][kMaxP + 1];
  T Mco[kMaxP + 1][kMaxP];
  T Moo[kMaxP][kMaxP];
  T D[kMaxP][kMaxP + 1];
};
void build_tab1d(int p, Tab1D<double>* t);  // host, FP64

// Device-resident scalars of one Krylov solve: the host reads them once per
// batch of iterations, never per iteration.
struct KrylovScalars {
  double rz;       // r.z of the current iterate
  double pq;       // p.Jp (starts as the essential-dof part, then the apply adds)
  double rr;       // r.r
  double bb;       // b.b
  double tol2;     // squared absolute stopping threshold
  double rtol2, atol2;
  double alpha, beta;
  double lz[2 * kMaxLanczos + 2];  // Lanczos alphas, betas
  int it;          // completed iterations
  int done;        // 1 = stop (converged or failed)
  int status;      // hc_status when done
  int maxit;
  unsigned int counter[8];  // tickets of the grid reductions
};

// Structured hex problem as the kernels see it.  Factors are SoA:
// fac[k*ne + e], k = 0..5 the mass tensor sigma |det J| J^-1 J^-T, k = 6..11 the
// curl tensor dt nu / |det J| J^T J, each packed symmetric (00,01,02,11,12,22).
struct HexDev {
  int p, nx, ny, nz;
  int64_t ne, ndof;
  int64_t off[3];
  int full;           // 1 = general parallelepipeds (9 tensor blocks), 0 = axis aligned
  int ess_bits;       // face attribute bits (implicit mask)
  const uint8_t* ess; // explicit device mask or nullptr
  const double* fac;  // FP64 factors (diagonal, FP64 apply)
  const int* tab;     // brick tile table of the active brick shape (relative dof
                      // offsets, bit 31 = brick face)
  int shape;          // brick shape of the tiled kernels (orders 1-2): 0 = 16x4x2, 1 = 8x8x2
  int per_sm;         // CTAs per SM of the tiled kernels, 0 = the launcher's choice
};

}  // namespace hc

struct hcop {
  int type = HC_HEX;
  int p = 1;
  int nx = 0, ny = 0, nz = 0;
  int64_t ndof = 0, ne = 0;
  int64_t off[3] = {0, 0, 0};
  double dt = 1.0;
  bool has_mass = false;
  bool full = false;
  int ess_bits = 0;
  bool explicit_mask = false;
  cudaStream_t stream = nullptr;
  std::string err;
  std::vector<uint8_t> ess_host;

  // device memory owned by the handle
  double* fac = nullptr;      // 12*ne FP64 factors
  float* facf = nullptr;      // 12*ne FP32 copy (FP32 apply)
  uint8_t* ess = nullptr;     // ndof essential flags
  double* diag = nullptr;     // ndof diagonal of J
  double* dinv = nullptr;     // ndof 1/diag
  float* dinvf = nullptr;     // FP32 copy
  double* sdinv = nullptr;    // 1/sqrt(diag)
  float* sdinvf = nullptr;
  hc::KrylovScalars* scal = nullptr;   // device scalars
  hc::KrylovScalars* hscal = nullptr;  // pinned host mirror
  double* partials = nullptr;          // device, reduction partials
  void* work = nullptr;                // Krylov vectors
  size_t work_bytes = 0;
  double* xbuf = nullptr;              // device staging for host-pointer calls
  double* ybuf = nullptr;
  double lmax64 = 0.0, lmax32 = 0.0;   // cached Chebyshev bounds
  double* verts = nullptr;             // device vertex coordinates (hex grid)
  // tetrahedral meshes
  int64_t n_edges = 0, n_faces = 0;
  int32_t* tet_edofs = nullptr;        // ne * L element dofs
  int32_t* tet_sv = nullptr;           // ne * 4 element vertices, sorted by global index
  double* tetK64 = nullptr;            // ne * L * L element matrices (FP64)
  float* tetK32 = nullptr;             // FP32 copy
  void* tetK16 = nullptr;              // BF16 copy (made on first use)
  int* tab = nullptr;                  // brick tile table of the apply kernel (shape 0)
  int* tab1 = nullptr;                 // the same for brick shape 1 (orders 1-2)
  int shape = 0, per_sm = 0;           // launch configuration of the tiled kernels (hc_autotune)
  void* cwork = nullptr;               // complex (frequency-domain) work space, hc_complex.cu
  void* aux = nullptr;                 // auxiliary-space preconditioner, hc_auxmg.cu
  void* mwork = nullptr;               // multi-RHS block PCG work space, hc_multi.cu
  void* taux = nullptr;                // tet auxiliary-space preconditioner, hc_tetaux.cu
  int64_t n_vert = 0;                  // tet meshes: vertices
  double* nu = nullptr;                // per-element nu (FP64), for nu-weighted post-processing
  hcop* mass_child = nullptr;          // unit-coefficient Nedelec mass on the same space (hc_fields.cu)

  hc::HexDev hexdev() const {
    hc::HexDev d;
    d.p = p;
    d.nx = nx;
    d.ny = ny;
    d.nz = nz;
    d.ne = ne;
    d.ndof = ndof;
    d.off[0] = off[0];
    d.off[1] = off[1];
    d.off[2] = off[2];
    d.full = full ? 1 : 0;
    d.ess_bits = ess_bits;
    d.ess = explicit_mask ? ess : nullptr;
    d.fac = fac;
    d.shape = (shape == 1 && tab1) ? 1 : 0;
    d.tab = d.shape ? tab1 : tab;
    d.per_sm = per_sm;
    return d;
  }
};

namespace hc {
// ---- memory (hc_api.cu) ----
// Device memory of a handle is stream-ordered on the handle's stream
// (cudaMallocAsync / cudaFreeAsync from the device's default pool): creating,
// growing or destroying a handle never synchronises the device, so requests
// come and go while others compute.
cudaError_t dmalloc(const hcop* h, void** p, size_t bytes);
void dfree(const hcop* h, void* p);
// Pinned host blocks (at most 4 KB) from a process-wide pool that is never
// returned to the driver (cudaFreeHost would synchronise the device).
void* pinned_get(size_t bytes);
void pinned_put(void* p);

// ---- hc_hex.cu ----
cudaError_t upload_tables();
int hex_apply_blocks(const HexDev& d);
// y += op(x).  masked: skip essential rows and zero essential entries of x
// (y must already hold (I-P)x for J).  mscale/cscale multiply the mass/curl
// factors.  S != nullptr: PCG mode (energy p.Jp accumulated onto S->pq,
// alpha formed, skipped when S->done).
// y_zero_free: the caller guarantees y == 0 at every non-essential dof, so
// brick-interior results may be stored instead of added.
template <typename T>
cudaError_t hex_apply(const HexDev& d, const T* fac, const T* x, T* y, double mscale, double cscale,
                      bool masked, KrylovScalars* S, double* partials, cudaStream_t s, bool y_zero_free);
cudaError_t hex_diag(const HexDev& d, double* diag, cudaStream_t s);
// diag += mscale * diag(M) + cscale * diag(dt C) (the two parts of hex_diag, scaled)
cudaError_t hex_diag_scaled(const HexDev& d, double* diag, double mscale, double cscale, cudaStream_t s);
// a launch configuration stored by hc_autotune for this handle's problem, if any (hc_tune.cu)
void tune_lookup(hcop* h);
// tile table of the brick kernel for order p and brick shape `shape` on an nx x ny grid (host)
void hex_tile_table(int p, int shape, int nx, int ny, std::vector<int>& tab);

// ---- hc_post.cu ----
void hex_rt_layout(const HexDev& d, int64_t* off1, int64_t* off2, int64_t* n);
cudaError_t hex_curl(const HexDev& d, const double* A, double* B, cudaStream_t s);
cudaError_t hex_load_coil(const HexDev& d, const double* V, const double coil[7], int q, const double* xq,
                          const double* wq, const double* bc, const double* bo, double* b, cudaStream_t s);
// points of the q^3 Gauss-Legendre rule per element (ne * q^3 * 3)
cudaError_t hex_quad_points(const HexDev& d, const double* V, int q, const double* xq, const double* wq,
                            const double* bc, const double* bo, double* xyz, cudaStream_t s);
// b = (J, w_i) for a source given per element (per_point = 0) or at the rule's points (1)
cudaError_t hex_load_field(const HexDev& d, const double* V, int per_point, const double* src, int q,
                           const double* xq, const double* wq, const double* bc, const double* bo, double* b,
                           cudaStream_t s);
// b_i = (nu curl A, w_i) with per-element nu
cudaError_t hex_curl_load(const HexDev& d, const double* nu, const double* A, double* b, cudaStream_t s);

// ---- hc_tet.cu ----
hc_status tet_topology(hcop* h, const hc_problem_desc* d, std::vector<int32_t>& edofs,
                       std::vector<int32_t>& sorted_verts);
cudaError_t tet_setup_device(hcop* h, const hc_problem_desc* desc, const std::vector<int32_t>& edofs,
                             const std::vector<int32_t>& sv);
template <typename T>
cudaError_t tet_apply_launch(const hcop* h, const T* K, const T* x, T* y, int nrhs, bool masked, double scale,
                             const int* done, cudaStream_t s);
cudaError_t tet_ensure_bf16(hcop* h);
cudaError_t tet_apply_launch_bf16(const hcop* h, const float* x, float* y, int nrhs, bool masked, cudaStream_t s);
// b = coil load (I0, xc, yc, r0, r1, z0, z1) with a q^3 collapsed Gauss-Legendre rule per tet (1 <= q <= 8)
cudaError_t tet_load_coil(const hcop* h, const double coil[7], int q, const double* xq, const double* wq, double* b,
                          cudaStream_t s);
// points of the collapsed q^3 rule per tet (ne * q^3 * 3)
cudaError_t tet_quad_points(const hcop* h, int q, const double* xq, double* xyz, cudaStream_t s);
// b = (J, w_i) for a source given per element (per_point = 0) or at the rule's points (1)
cudaError_t tet_load_field(const hcop* h, int per_point, const double* src, int q, const double* xq,
                           const double* wq, double* b, cudaStream_t s);
// b_i = (nu curl A, w_i) with per-element nu (collapsed rule, q points per direction)
cudaError_t tet_curl_load(const hcop* h, const double* A, int q, const double* xq, const double* wq, double* b,
                          cudaStream_t s);
// B = curl A at npts reference points (<= 16) of every tet (ne * npts * 3)
cudaError_t tet_curl_points(const hcop* h, const double* A, int npts, const double* xi, double* B, cudaStream_t s);
// pq = p.q over all dofs, then alpha = rz / pq (PCG mode of operators without a fused energy)
template <typename T>
cudaError_t dot_alpha(int64_t n, const T* p, const T* q, KrylovScalars* S, double* partials, cudaStream_t s);

// fused complex apply, orders 1-2 (hc_hex_cplx.cuh, instantiated in hc_hex_p{1,2}.cu):
// y_r += C x_r - omega M x_i, y_i += C x_i + omega M x_r with the curl factor
// scaled by cscale; skipped when *done != 0
template <typename T, int P>
cudaError_t hex_launch_cplx_p(const HexDev& d, const T* fac, const T* xr, const T* xi, T* yr, T* yi, T omega,
                              T cs, bool masked, const int* done, cudaStream_t s);
// y += cs C xc + ms M xm (masked, axis-aligned grids; order 3, hc_hex_p3.cu)
template <typename T, int P>
cudaError_t hex_launch_pair(const HexDev& d, const T* fac, const T* xc, const T* xm, T* y, T ms, T cs,
                            cudaStream_t s);
// ---- hc_auxmg.cu ----
// gradient-space (auxiliary) preconditioner: setup once per handle (FP32)
hc_status auxmg_setup(hcop* h);
void auxmg_free(hcop* h);
// z += C G V G^T r; NV = 1: z0 += coef[0] (G V G^T r0); NV = 2 (planar complex):
// z0 += coef[0] v0 + coef[1] v1, z1 += coef[2] v0 + coef[3] v1
template <typename T, int NV>
cudaError_t auxmg_apply(const hcop* h, const T* r0, const T* r1, T* z0, T* z1, const float coef[4], const int* done,
                        cudaStream_t s);

// ---- hc_complex.cu ----
// y = (I-P) x + P (C_nu + i omega M_sigma) P x on planar (re, im) vectors
template <typename T>
cudaError_t complex_apply(hcop* h, double omega, const T* xr, const T* xi, T* yr, T* yi, cudaStream_t s);
// COCG with complex Jacobi (FP64, or FP32 inner in FP64 refinement)
hc_status complex_solve_device(hcop* h, const hc_solve_params* prm, double omega, const double* br,
                               const double* bi, double* xr, double* xi, hc_solve_info* info);
void complex_free(hcop* h);

// ---- hc_multi.cu ----
// block PCG (Jacobi) for R right-hand sides in [dof][rhs] layout (tet meshes)
hc_status multi_solve_device(hcop* h, const hc_solve_params* prm, int R, const double* B, double* X,
                             hc_solve_info* info);
void multi_free(hcop* h);

// ---- hc_tetaux.cu ----
// gradient-space (auxiliary) preconditioner of tet meshes: AMG setup once per handle
hc_status tetaux_setup(hcop* h);
void tetaux_free(hcop* h);
// work vectors for R right-hand sides (call before applying with R columns)
hc_status tetaux_reserve(hcop* h, int R);
// z = D^-1 r + (PG) V (PG)^T r for R columns in [dof][rhs] layout; skipped when *done
template <typename T>
cudaError_t tetaux_apply(const hcop* h, int R, const T* r, T* z, const T* dinv, const int* done, cudaStream_t s);
// y = G u: discrete gradient of vertex values u (P1) into the Nedelec space
cudaError_t tet_gradient(const hcop* h, const double* u, double* y, cudaStream_t s);

// ---- hc_krylov.cu ----
cudaError_t diag_finish(int64_t n, const uint8_t* ess, double* d, double* dinv, float* dinvf, double* sd,
                        float* sdf, cudaStream_t s);
template <typename T>
cudaError_t init_masked(int64_t n, const uint8_t* ess, const T* x, T* y, cudaStream_t s);
// y[i*nrhs + r] = ess[i] ? x[i*nrhs + r] : 0
template <typename T>
cudaError_t init_masked_multi(int64_t n, int nrhs, const uint8_t* ess, const T* x, T* y, cudaStream_t s);
// operator callback used by the solvers: y = J x with y pre-initialised by the
// callee; S/partials as in hex_apply
template <typename T>
struct OpJ {
  hcop* h;
  const T* fac;
  cudaError_t apply(const T* x, T* y, KrylovScalars* S, double* partials, cudaStream_t s,
                    bool y_zero_free = true) const;
};
// Weight c of the gradient-space correction in HC_PRECOND_AUX_MULT.  The
// correction V only approximates (G^T J G)^-1 (an additive two-level V-cycle
// that can overshoot up to twice); damping it keeps the multiplicative cycle
// a contraction.
constexpr float kAuxMultWeight = 0.5f;
struct SolveCfg {
  int precond;
  int cheb_degree;
  double cheb_ratio;
  double lmax;
  double rtol, atol;
  int maxit;
};
// Preconditioned CG on J x = b, device vectors of type T, x = initial guess.
template <typename T>
hc_status pcg_device(hcop* h, const SolveCfg& cfg, const T* b, T* x, int* iters, int* applies,
                     double* relres_dev_norm);
// Lanczos estimate of lambda_max(D^-1 J) with operator precision T.
template <typename T>
hc_status lanczos_device(hcop* h, int steps, double* lmax);
// Mixed precision: FP32 inner PCG in FP64 iterative refinement.
hc_status mixed_device(hcop* h, const hc_solve_params* prm, const double* b, double* x,
                       hc_solve_info* info);
// FP32 PCG with FP64 residual replacement (HC_MIXED_RR).
hc_status mixed_rr_device(hcop* h, const hc_solve_params* prm, const double* b, double* x,
                          hc_solve_info* info);
hc_status ensure_work(hcop* h, size_t bytes);
// z = D^-1 r (FP64, the handle's Jacobi diagonal)
cudaError_t jacobi_apply(int64_t n, const double* dinv, const double* r, double* z, cudaStream_t s);
cudaError_t ensure_scalars(hcop* h);
double vec_norm2_host(hcop* h, const double* x, int64_t n);  // synchronous helper

}  // namespace hc

#define HC_CUDA_TRY(h, expr)                                                              \
  do {                                                                                    \
    cudaError_t _e = (expr);                                                              \
    if (_e != cudaSuccess) {                                                              \
      (h)->err = std::string(#expr) + ": " + cudaGetErrorString(_e);                      \
      return HC_ECUDA;                                                                    \
    }                                                                                     \
  } while (0)

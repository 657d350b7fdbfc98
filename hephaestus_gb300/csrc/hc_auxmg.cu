// hc_auxmg.cu -- auxiliary-space (gradient) preconditioner for the structured
// hex Nedelec operator: the gradient part of the Hiptmair-Xu / AMS
// preconditioner that the reference configures with HypreAMS
// (src/formulations/HCurl/hcurl_formulation.cpp:69-79):
//
//     B r = D^-1 r + c G V (G^T r)
//
// G is the discrete gradient from the order-p H1 space (closed Gauss-Lobatto
// nodes, the space whose gradients the Nedelec space contains) to the Nedelec
// space: a matrix-free stencil, (G phi)_c(a) = sum_q D[a][q] phi(q) along the
// open direction c.  On free nodes G^T K G = G^T M_sigma G =: L, the
// sigma-weighted H1 stiffness (the curl of a gradient vanishes), so V ~ L^-1:
//   * order p > 1: V = D_L^-1 + P0 V1 P0^T, P0 the trilinear interpolation
//     from the element-vertex (Q1) grid to the Gauss-Lobatto nodes;
//   * V1: one multigrid V-cycle on Q1 grids: the finest level's element
//     matrices are the Q1 stiffness of the handle's mass tensor
//     sigma |det J| J^-1 J^-T, coarser levels halve each direction (ceil) with
//     index-space trilinear interpolation and Galerkin element matrices
//     W^T K W; every level is applied as an assembled 27-point stencil (a
//     gather per node, no atomics); Chebyshev-Jacobi smoothing (degree 3, interval
//     [lmax/30, lmax], lmax a Gershgorin bound), Chebyshev(8) on the coarsest
//     grid (<= 1000 nodes).
// The V-cycle runs in FP32 for one (real) or two (real and imaginary)
// vectors.  c = 1 for K = dt C + M_sigma, c = 1/(i omega) for C + i omega M_sigma.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cooperative_groups.h>

#include "hc_internal.h"

namespace hc {

#define GS_LOOP(i, n) \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

constexpr int kAuxMaxLevels = 10;
constexpr int kAuxCoarseNodes = 1000;
constexpr int kAuxDegree = 2;        // Chebyshev degree of the pre- and post-smoothers
constexpr int kAuxCoarseDegree = 4;  // Chebyshev degree on the coarsest grid
constexpr double kAuxRatio = 30.0;
constexpr int kAuxGraphs = 8;
// coarse-level cluster launch of the V-cycle (k_vcycle_cluster)
constexpr int kClusterCtas = 8;
constexpr int kClusterThreads = 1024;
constexpr int64_t kSmallLevelNodes = 10000;
// forms of the V-cycle (vcycle_mode)
enum { kVKernels = 0, kVCoop = 1, kVHybrid = 2, kVCluster = 3 };

static inline unsigned agrid(int64_t n, int threads = 256) {
  const int64_t b = (n + threads - 1) / threads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 4 * 152));
}

// 1-D data of the order-p H1 / Nedelec pair
struct AuxTab {
  int p;
  float D[kMaxP][kMaxP + 1];  // D[a][q] = phi_q'(open node a)
  float gll[kMaxP + 1];       // Gauss-Lobatto nodes on [0,1]
  float Kd[kMaxP + 1];        // int (phi_q')^2
  float Md[kMaxP + 1];        // int phi_q^2
};

struct Dims {
  int nx, ny, nz;
  __host__ __device__ int64_t nodes() const { return (int64_t)(nx + 1) * (ny + 1) * (nz + 1); }
  __host__ __device__ int64_t elems() const { return (int64_t)nx * ny * nz; }
};

struct AuxLevel {
  Dims d{0, 0, 0};
  float* Ke = nullptr;    // 64 per element (setup only; freed once the next level is built)
  float* St = nullptr;    // 27-point stencil, 27 * nodes
  float* dinv = nullptr;  // 0 at fixed nodes
  float *x = nullptr, *b = nullptr, *r = nullptr, *dv = nullptr, *t = nullptr;  // 2 * nodes each
  // t doubles as the second Chebyshev direction buffer (the fused steps
  // read one direction at stencil neighbours and write the other)
  double lmax = 2.0;
};

// A replayable capture of one preconditioner application (fixed buffers).
struct AuxGraph {
  cudaGraphExec_t exec = nullptr;
  const void* key[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  int nv = 0, tsize = 0, coop = 0;
  float coef[4] = {0, 0, 0, 0};
};

// Grid barrier of the cooperative V-cycle (device memory, zeroed at setup).
struct CoopBar {
  unsigned count;  // arrivals at the current barrier
  unsigned gen;    // barriers completed
  int err;         // 1: a wait gave up (sticky; the V-cycle then returns NaN)
};

struct AuxMG {
  int p = 1, nlev = 0;
  CoopBar* bar = nullptr;  // cooperative V-cycle state, nullptr: per-step kernels
  bool cluster_ok = false;  // the coarse-level cluster launch fits on this device
  int coop_blocks = 0;     // co-resident blocks of the cooperative V-cycle (per NV: [NV - 1])
  int coop_blocks2 = 0;
  std::vector<AuxGraph> graphs;   // at most kAuxGraphs, oldest replaced first
  int next_graph = 0;
  cudaStream_t cap = nullptr;     // private stream the captures are made on
  AuxLevel lev[kAuxMaxLevels];
  Dims q{0, 0, 0};         // Gauss-Lobatto node grid as "elements" (nodes = (n p + 1)^3), p > 1
  int64_t nq = 0;
  float* qdinv = nullptr;  // 1/diag(L) on the Gauss-Lobatto grid, 0 at fixed nodes
  float* g = nullptr;      // 2 * nq
  float* phi = nullptr;    // 2 * nq
  AuxTab tab{};
};

// ---- element matrices of Q1 ---------------------------------------------------
// K[a][b] = sum_cd F_cd int d_c N_a d_d N_b on the reference cube; F packed
// symmetric (00,01,02,11,12,22).  1-D factors: k = int N_a' N_b', g = int N_a' N_b,
// m = int N_a N_b for the linear functions N_0 = 1 - x, N_1 = x.
__device__ __forceinline__ float q1_1d(int dir, int c, int d, int a, int b) {
  if (dir == c && dir == d) return a == b ? 1.0f : -1.0f;
  if (dir == c) return a == 0 ? -0.5f : 0.5f;
  if (dir == d) return b == 0 ? -0.5f : 0.5f;
  return a == b ? (1.0f / 3.0f) : (1.0f / 6.0f);
}
__device__ __forceinline__ void q1_matrix(const float F[6], float K[64]) {
  const int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  for (int a = 0; a < 8; ++a)
    for (int b = a; b < 8; ++b) {
      float s = 0.0f;
      for (int c = 0; c < 3; ++c)
        for (int d = 0; d < 3; ++d) {
          const float f = F[sym[c][d]];
          if (f == 0.0f) continue;
          s += f * q1_1d(0, c, d, a & 1, b & 1) * q1_1d(1, c, d, (a >> 1) & 1, (b >> 1) & 1) *
               q1_1d(2, c, d, (a >> 2) & 1, (b >> 2) & 1);
        }
      K[a * 8 + b] = s;
      K[b * 8 + a] = s;
    }
}
__device__ __forceinline__ void load_F(const float* facf, int64_t ne, int64_t e, float F[6]) {
  for (int k = 0; k < 6; ++k) F[k] = facf[(int64_t)k * ne + e];
}
__device__ __forceinline__ int64_t vnode(const Dims& d, int i, int j, int k) {
  return i + (int64_t)(d.nx + 1) * (j + (int64_t)(d.ny + 1) * k);
}
__device__ __forceinline__ void elem_ijk(const Dims& d, int64_t e, int& i, int& j, int& k) {
  i = (int)(e % d.nx);
  j = (int)((e / d.nx) % d.ny);
  k = (int)(e / ((int64_t)d.nx * d.ny));
}

// finest-level element matrices from the mass factors
__global__ void k_q1_build(Dims d, const float* __restrict__ facf, float* __restrict__ Ke) {
  const int64_t ne = d.elems();
  GS_LOOP(e, ne) {
    float F[6], K[64];
    load_F(facf, ne, e, F);
    q1_matrix(F, K);
    for (int q = 0; q < 64; ++q) Ke[e * 64 + q] = K[q];
  }
}

// assembled 27-point stencil St[q * nn + node], q = (dx+1) + 3 (dy+1) + 9 (dz+1),
// gathered from the (up to) 8 elements around each node; diag and |row| sums
__global__ void k_stencil(Dims d, const float* __restrict__ Ke, float* __restrict__ St, float* __restrict__ diag,
                          float* __restrict__ absrow) {
  const int64_t nn = d.nodes();
  GS_LOOP(n, nn) {
    const int i = (int)(n % (d.nx + 1)), j = (int)((n / (d.nx + 1)) % (d.ny + 1)),
              k = (int)(n / ((int64_t)(d.nx + 1) * (d.ny + 1)));
    float st[27];
    for (int q = 0; q < 27; ++q) st[q] = 0.0f;
    for (int ek = k - 1; ek <= k; ++ek)
      for (int ej = j - 1; ej <= j; ++ej)
        for (int ei = i - 1; ei <= i; ++ei) {
          if (ei < 0 || ej < 0 || ek < 0 || ei >= d.nx || ej >= d.ny || ek >= d.nz) continue;
          const int64_t e = ei + (int64_t)d.nx * (ej + (int64_t)d.ny * ek);
          const int a = (i - ei) + 2 * (j - ej) + 4 * (k - ek);
          for (int b = 0; b < 8; ++b) {
            const int dx = ei + (b & 1) - i, dy = ej + ((b >> 1) & 1) - j, dz = ek + ((b >> 2) & 1) - k;
            st[(dx + 1) + 3 * (dy + 1) + 9 * (dz + 1)] += Ke[e * 64 + a * 8 + b];
          }
        }
    float sa = 0.0f;
    for (int q = 0; q < 27; ++q) {
      St[q * nn + n] = st[q];
      sa += fabsf(st[q]);
    }
    diag[n] = st[13];
    absrow[n] = sa;
  }
}

// Node-grid kernels: a block of 256 threads covers 256 consecutive nodes of
// one z-plane (the plane's rows flattened, i fastest), grid.y = the planes.
// (One block per grid row left a third of the lanes idle on 65-node rows:
// 66 nodes in 96 threads, the third warp with two active lanes.)
struct NodeGrid {
  dim3 grid, block;
};
constexpr int kNodeThreads = 256;
static inline NodeGrid node_grid(int nx, int ny, int nz) {
  const int64_t plane = (int64_t)(nx + 1) * (ny + 1);
  return NodeGrid{dim3((unsigned)((plane + kNodeThreads - 1) / kNodeThreads), (unsigned)(nz + 1), 1u),
                  dim3((unsigned)kNodeThreads)};
}
// Transfer kernels on the large grids: KT consecutive z-planes per thread,
// every load issued before the node's mask is applied, so that a thread keeps
// several independent gathers in flight (one node per thread and a mask test
// ahead of the gathers left these kernels bound by two memory latencies per
// node).
constexpr int kKT = 4;
static inline NodeGrid node_grid_kt(int nx, int ny, int nz) {
  NodeGrid g = node_grid(nx, ny, nz);
  g.grid.y = (unsigned)((nz + 1 + kKT - 1) / kKT);
  return g;
}
// (i, j) of this thread's node in a plane of (nx + 1) x (ny + 1) nodes; threads
// past the plane's end return
#define PLANE_IJ(nx, ny, i, j)                                  \
  const int t_ = blockIdx.x * blockDim.x + threadIdx.x;         \
  if (t_ >= ((nx) + 1) * ((ny) + 1)) return;                    \
  const int i = t_ % ((nx) + 1), j = t_ / ((nx) + 1)
#define NODE_IJK(d, i, j, k, n)                                 \
  PLANE_IJ((d).nx, (d).ny, i, j);                               \
  const int k = blockIdx.y;                                     \
  const int n = t_ + ((d).nx + 1) * ((d).ny + 1) * k

// Loads of level vectors.  COH (the cooperative V-cycle, where one launch
// writes a vector in one step and other blocks read it in a later one): L2
// loads (ld.global.cg), never the per-SM read-only or L1 copies, which are
// not kept coherent with other SMs' writes within a launch.
template <bool COH>
__device__ __forceinline__ float vld(const float* p) {
  if constexpr (COH) return __ldcg(p);
  else return *p;
}

// (L v)_n: all 27 coefficient and value loads issued together; the stencil of
// a boundary node has zero coefficients outside the grid, whose loads are
// redirected to the node itself
template <int NV, bool COH = false>
__device__ __forceinline__ void st_row(const Dims& d, const float* __restrict__ St, const float* __restrict__ v,
                                       int nn, int n, int i, int j, int k, float (&acc)[NV]) {
  const int sx = d.nx + 1, sxy = (d.nx + 1) * (d.ny + 1);
  for (int q = 0; q < NV; ++q) acc[q] = 0.0f;
#pragma unroll
  for (int q = 0; q < 27; ++q) {
    const int dx = q % 3 - 1, dy = (q / 3) % 3 - 1, dz = q / 9 - 1;
    const bool in = (unsigned)(i + dx) <= (unsigned)d.nx && (unsigned)(j + dy) <= (unsigned)d.ny &&
                    (unsigned)(k + dz) <= (unsigned)d.nz;
    const int m = in ? n + dx + sx * dy + sxy * dz : n;
    const float c = St[q * nn + n];
#pragma unroll
    for (int w = 0; w < NV; ++w) acc[w] = __fmaf_rn(c, vld<COH>(v + w * nn + m), acc[w]);
  }
}

// One fused Chebyshev step (Saad Alg. 12.1): t = L d_in, r -= t,
// d_out = c1 d_in + c2 D^-1 r, x += (add_in ? d_in : 0) + d_out.
// d_in is read at stencil neighbours and never written here.
template <int NV, bool COH = false>
__device__ __forceinline__ void cheb_fused_at(const Dims& d, const float* __restrict__ St,
                                              const float* __restrict__ dinv, const float* __restrict__ din,
                                              float* __restrict__ dout, float* __restrict__ r,
                                              float* __restrict__ x, float c1, float c2, int add_in, int n, int i,
                                              int j, int k) {
  const int nn = (int)d.nodes();
  float t[NV];
  st_row<NV, COH>(d, St, din, nn, n, i, j, k, t);
  const float dv = dinv[n];
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int id = q * nn + n;
    const float ri = __fsub_rn(vld<COH>(r + id), t[q]);
    const float di = vld<COH>(din + id);
    const float dn = __fmaf_rn(c1, di, __fmul_rn(__fmul_rn(c2, dv), ri));
    r[id] = ri;
    dout[id] = dn;
    x[id] = __fadd_rn(vld<COH>(x + id), __fadd_rn(add_in ? di : 0.0f, dn));
  }
}
template <int NV>
__global__ void k_cheb_fused(Dims d, const float* __restrict__ St, const float* __restrict__ dinv,
                             const float* __restrict__ din, float* __restrict__ dout, float* __restrict__ r,
                             float* __restrict__ x, float c1, float c2, int add_in, const int* __restrict__ done) {
  if (done && *done) return;
  NODE_IJK(d, i, j, k, n);
  cheb_fused_at<NV>(d, St, dinv, din, dout, r, x, c1, c2, add_in, n, i, j, k);
}
// r = b - L x (zero at fixed nodes), d = D^-1 r / theta; x untouched
template <int NV, bool COH = false>
__device__ __forceinline__ void cheb_resid_at(const Dims& d, const float* __restrict__ St,
                                              const float* __restrict__ dinv, const float* __restrict__ b,
                                              const float* __restrict__ x, float* __restrict__ r,
                                              float* __restrict__ dv, float inv_theta, int n, int i, int j, int k) {
  const int nn = (int)d.nodes();
  float t[NV];
  st_row<NV, COH>(d, St, x, nn, n, i, j, k, t);
  const float di = dinv[n];
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const int id = q * nn + n;
    const float ri = di != 0.0f ? __fsub_rn(vld<COH>(b + id), t[q]) : 0.0f;
    r[id] = ri;
    dv[id] = __fmul_rn(__fmul_rn(di, ri), inv_theta);
  }
}
template <int NV>
__global__ void k_cheb_resid(Dims d, const float* __restrict__ St, const float* __restrict__ dinv,
                             const float* __restrict__ b, const float* __restrict__ x, float* __restrict__ r,
                             float* __restrict__ dv, float inv_theta, const int* __restrict__ done) {
  if (done && *done) return;
  NODE_IJK(d, i, j, k, n);
  cheb_resid_at<NV>(d, St, dinv, b, x, r, dv, inv_theta, n, i, j, k);
}
// x += d (a one-step smoother from a nonzero start)
template <int NV>
__global__ void k_add(int nn, const float* __restrict__ d, float* __restrict__ x, const int* __restrict__ done) {
  if (done && *done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < NV * nn; i += gridDim.x * blockDim.x)
    x[i] = __fadd_rn(x[i], d[i]);
}

// coarse element matrices: K_C = sum over children W^T K_child W (index-space trilinear W)
__device__ __forceinline__ void child_weights(int f, int lo, int nf, float& wlo, float& whi) {
  // coarse element spans fine [2 lo, min(2 lo + 2, nf)]
  const int a = 2 * lo, b = min(2 * lo + 2, nf);
  whi = (float)(f - a) / (float)(b - a);
  wlo = 1.0f - whi;
}
__global__ void k_coarsen(Dims fd, Dims cd, const float* __restrict__ Kf, float* __restrict__ Kc) {
  const int64_t nec = cd.elems();
  GS_LOOP(E, nec) {
    int I, J, Kk;
    elem_ijk(cd, E, I, J, Kk);
    float KC[64];
    for (int q = 0; q < 64; ++q) KC[q] = 0.0f;
    for (int ck = 2 * Kk; ck < min(2 * Kk + 2, fd.nz); ++ck)
      for (int cj = 2 * J; cj < min(2 * J + 2, fd.ny); ++cj)
        for (int ci = 2 * I; ci < min(2 * I + 2, fd.nx); ++ci) {
          const int64_t e = ci + (int64_t)fd.nx * (cj + (int64_t)fd.ny * ck);
          float K[64];
          for (int q = 0; q < 64; ++q) K[q] = Kf[e * 64 + q];
          // W[a][A]: fine local vertex a -> coarse local vertex A
          float W[8][8];
          for (int a = 0; a < 8; ++a) {
            float wl[3], wh[3];
            child_weights(ci + (a & 1), I, fd.nx, wl[0], wh[0]);
            child_weights(cj + ((a >> 1) & 1), J, fd.ny, wl[1], wh[1]);
            child_weights(ck + ((a >> 2) & 1), Kk, fd.nz, wl[2], wh[2]);
            for (int A = 0; A < 8; ++A)
              W[a][A] = ((A & 1) ? wh[0] : wl[0]) * (((A >> 1) & 1) ? wh[1] : wl[1]) * (((A >> 2) & 1) ? wh[2] : wl[2]);
          }
          float KW[8][8];  // K W
          for (int a = 0; a < 8; ++a)
            for (int B = 0; B < 8; ++B) {
              float s = 0.0f;
              for (int b = 0; b < 8; ++b) s += K[a * 8 + b] * W[b][B];
              KW[a][B] = s;
            }
          for (int A = 0; A < 8; ++A)
            for (int B = 0; B < 8; ++B) {
              float s = 0.0f;
              for (int a = 0; a < 8; ++a) s += W[a][A] * KW[a][B];
              KC[A * 8 + B] += s;
            }
        }
    for (int q = 0; q < 64; ++q) Kc[E * 64 + q] = KC[q];
  }
}

__global__ void k_finish_dinv(int64_t n, const float* __restrict__ diag, const uint8_t* __restrict__ fixed,
                              float* __restrict__ dinv) {
  GS_LOOP(i, n) dinv[i] = (fixed[i] || !(diag[i] > 0.0f)) ? 0.0f : 1.0f / diag[i];
}

// ---- grid transfers between Q1 levels ------------------------------------------------
// 1-D transfer weights between a fine grid of nf cells and its 2:1 coarsening
// (coarse node I sits at fine node min(2 I, nf)).
// weight of fine node f for coarse node I
__device__ __forceinline__ float w1d(int f, int I, int nf) {
  if (f < 0 || f > nf) return 0.0f;
  if ((f & 1) == 0) return (f >> 1) == I ? 1.0f : 0.0f;
  if (f == nf) return I == (nf + 1) / 2 ? 1.0f : 0.0f;
  return (I == (f - 1) / 2 || I == (f + 1) / 2) ? 0.5f : 0.0f;
}
// b_c = R r_f (r_f is zero at fixed fine nodes), zero at fixed coarse nodes
// The producer of a level's right-hand side also starts its Chebyshev
// smoother from x = 0: r = b, d = D^-1 b / theta, x = d.
struct ChebStart {
  float* r;
  float* d;
  float* x;
  float inv_theta;
};
template <int NV>
__device__ __forceinline__ void cheb_start_at(const ChebStart& cs, int nn, int n, float dinv, const float (&b)[NV]) {
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const float dv = __fmul_rn(__fmul_rn(dinv, b[v]), cs.inv_theta);
    cs.r[v * nn + n] = b[v];
    cs.d[v * nn + n] = dv;
    cs.x[v * nn + n] = dv;
  }
}

template <int NV, bool COH = false>
__device__ __forceinline__ void restrict_at(const Dims& fd, const Dims& cd, const float* __restrict__ rf,
                                            const float* __restrict__ dinvc, float* __restrict__ bc,
                                            const ChebStart& cs, int n, int I, int J, int K) {
  const int nc = (int)cd.nodes(), nf = (int)fd.nodes();
  const int sx = fd.nx + 1, sxy = (fd.nx + 1) * (fd.ny + 1);
  float acc[NV];
  for (int v = 0; v < NV; ++v) acc[v] = 0.0f;
  if (dinvc[n] != 0.0f) {
#pragma unroll
    for (int q = 0; q < 27; ++q) {
      const int fi = 2 * I - 1 + q % 3, fj = 2 * J - 1 + (q / 3) % 3, fk = 2 * K - 1 + q / 9;
      const float w = __fmul_rn(__fmul_rn(w1d(fi, I, fd.nx), w1d(fj, J, fd.ny)), w1d(fk, K, fd.nz));
      const int g = w != 0.0f ? fi + sx * fj + sxy * fk : 0;
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v] = __fmaf_rn(w, vld<COH>(rf + v * nf + g), acc[v]);
    }
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) bc[v * nc + n] = acc[v];
  cheb_start_at<NV>(cs, nc, n, dinvc[n], acc);
}
template <int NV>
__global__ void k_restrict(Dims fd, Dims cd, const float* __restrict__ rf, const float* __restrict__ dinvc,
                           float* __restrict__ bc, ChebStart cs, const int* __restrict__ done) {
  if (done && *done) return;
  NODE_IJK(cd, I, J, K, n);
  restrict_at<NV>(fd, cd, rf, dinvc, bc, cs, n, I, J, K);
}
// x_f += P x_c at free fine nodes
__device__ __forceinline__ void coarse_pair(int f, int nf, int& c0, int& c1, float& w0, float& w1) {
  if ((f & 1) == 0) {
    c0 = c1 = f >> 1;
    w0 = 1.0f;
    w1 = 0.0f;
  } else if (f == nf) {
    c0 = c1 = (nf + 1) / 2;
    w0 = 1.0f;
    w1 = 0.0f;
  } else {
    c0 = (f - 1) / 2;
    c1 = (f + 1) / 2;
    w0 = w1 = 0.5f;
  }
}
template <int NV, bool COH = false>
__device__ __forceinline__ void prolong_add_at(const Dims& fd, const Dims& cd, const float* __restrict__ xc,
                                               const float* __restrict__ dinvf, float* __restrict__ xf, int n,
                                               int i, int j, int k) {
  if (dinvf[n] == 0.0f) return;
  const int nc = (int)cd.nodes(), nf = (int)fd.nodes();
  int ci[2], cj[2], ck[2];
  float wi[2], wj[2], wk[2];
  coarse_pair(i, fd.nx, ci[0], ci[1], wi[0], wi[1]);
  coarse_pair(j, fd.ny, cj[0], cj[1], wj[0], wj[1]);
  coarse_pair(k, fd.nz, ck[0], ck[1], wk[0], wk[1]);
  const int sx = cd.nx + 1, sxy = (cd.nx + 1) * (cd.ny + 1);
  float acc[NV];
  for (int v = 0; v < NV; ++v) acc[v] = 0.0f;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    const int a = q & 1, b = (q >> 1) & 1, c = q >> 2;
    const float w = __fmul_rn(__fmul_rn(wi[a], wj[b]), wk[c]);
    const int g = ci[a] + sx * cj[b] + sxy * ck[c];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = __fmaf_rn(w, vld<COH>(xc + v * nc + g), acc[v]);
  }
#pragma unroll
  for (int v = 0; v < NV; ++v) xf[v * nf + n] = __fadd_rn(vld<COH>(xf + v * nf + n), acc[v]);
}
template <int NV>
__global__ void k_prolong_add(Dims fd, Dims cd, const float* __restrict__ xc, const float* __restrict__ dinvf,
                              float* __restrict__ xf, const int* __restrict__ done) {
  if (done && *done) return;
  NODE_IJK(fd, i, j, k, n);
  prolong_add_at<NV>(fd, cd, xc, dinvf, xf, n, i, j, k);
}

// ---- Nedelec <-> Gauss-Lobatto nodes ----------------------------------------------------
// (dof counts are below 2^31: checked when the handle is created; the order P
// is a template parameter so that element/local splits are shifts and
// multiplications)

// g = G^T r on the Gauss-Lobatto grid (mx+1, my+1, mz+1), zero where qdinv = 0.
// Per component c, node index I_c = e P + q lies in one element (0 < q < P) or
// on the boundary between two (q = 0 of e, q = P of e - 1); both cases are
// written as two visits with 0/1 weights, so that the gathers carry no branch.
template <typename T, int NV, int P>
__device__ __forceinline__ void gt_at(const HexDev& h, const AuxTab& tab, const T* __restrict__ r0,
                                      const T* __restrict__ r1, int mx, int my, int I, int J, int K,
                                      float (&acc)[NV]) {
  const T* rr[2] = {r0, r1};
  for (int v = 0; v < NV; ++v) acc[v] = 0.0f;
  const int idx[3] = {I, J, K};
  const int ne[3] = {h.nx, h.ny, h.nz};
  const int base[3] = {(int)h.off[0], (int)h.off[1], (int)h.off[2]};
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const int ic = idx[c];
    // strides of component c's dof array
    const int n0 = mx + (c != 0), n1 = my + (c != 1);
    const int s_c = c == 0 ? 1 : (c == 1 ? n0 : n0 * n1);
    int tt[3] = {I, J, K};
    tt[c] = 0;
    const int b0 = base[c] + tt[0] + n0 * (tt[1] + n1 * tt[2]);
    const int e0 = ic / P, q0 = ic - e0 * P;
    // visit 1: (e0, q0) inside, else (e0 - 1, P); visit 2: (e0, 0) on a boundary
    const int ea = q0 != 0 ? e0 : max(e0 - 1, 0), qa = q0 != 0 ? q0 : P;
    const float ma = (q0 != 0 || ic > 0) ? 1.0f : 0.0f;
#pragma unroll
    for (int a2 = 0; a2 < P; ++a2) {
      const float wa = ma * tab.D[a2][qa];
      const int ga = b0 + (ea * P + a2) * s_c;
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[v] += wa * (float)rr[v][ga];
    }
    // the second visit only on element boundaries: along z the same for the
    // whole warp, along y for all but the warps that straddle two rows
    if (c == 0 || q0 == 0) {
      const int eb = min(e0, ne[c] - 1);
      const float mb = (q0 == 0 && e0 < ne[c]) ? 1.0f : 0.0f;
#pragma unroll
      for (int a2 = 0; a2 < P; ++a2) {
        const float wb = mb * tab.D[a2][0];
        const int gb = b0 + (eb * P + a2) * s_c;
#pragma unroll
        for (int v = 0; v < NV; ++v) acc[v] += wb * (float)rr[v][gb];
      }
    }
  }
}
template <typename T, int NV, int P>
__global__ void k_gt(HexDev h, AuxTab tab, const T* __restrict__ r0, const T* __restrict__ r1,
                     const float* __restrict__ qdinv, float* __restrict__ g, ChebStart cs,
                     const int* __restrict__ done) {
  if (done && *done) return;
  const Dims qd{h.nx * P, h.ny * P, h.nz * P};
  PLANE_IJ(qd.nx, qd.ny, I, J);
  const int nq = (int)qd.nodes();
  float acc[kKT][NV], dq[kKT];
#pragma unroll
  for (int t = 0; t < kKT; ++t) {  // gathers of all planes first
    const int K = min((int)blockIdx.y * kKT + t, qd.nz);
    gt_at<T, NV, P>(h, tab, r0, r1, qd.nx, qd.ny, I, J, K, acc[t]);
    dq[t] = qdinv[I + (qd.nx + 1) * (J + (qd.ny + 1) * K)];
  }
#pragma unroll
  for (int t = 0; t < kKT; ++t) {
    const int K = blockIdx.y * kKT + t;
    if (K > qd.nz) break;
    const int n = I + (qd.nx + 1) * (J + (qd.ny + 1) * K);
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      acc[t][v] = dq[t] != 0.0f ? acc[t][v] : 0.0f;
      g[v * nq + n] = acc[t][v];
    }
    if (cs.r) cheb_start_at<NV>(cs, nq, n, dq[t], acc[t]);
  }
}

// z += C G phi for the dofs of component c (grid n0 x n1 x n2, open along c);
// C a 2x2 real matrix acting on (phi_0, phi_1); NV = 1 uses C[0]
template <typename T, int NV, int P, int c>
__global__ void k_g(HexDev h, AuxTab tab, const float* __restrict__ phi, const uint8_t* __restrict__ ess,
                    T* __restrict__ z0, T* __restrict__ z1, float c00, float c01, float c10, float c11,
                    const int* __restrict__ done) {
  if (done && *done) return;
  const int mx = h.nx * P, my = h.ny * P, mz = h.nz * P;
  const int n0 = mx + (c != 0), n1 = my + (c != 1), n2 = mz + (c != 2);
  PLANE_IJ(n0 - 1, n1 - 1, i, j);
  const int nq = (mx + 1) * (my + 1) * (mz + 1);
  const int stride = c == 0 ? 1 : (c == 1 ? (mx + 1) : (mx + 1) * (my + 1));
  // loads of all kKT dofs first (phi gathers, masks, the z values), then the updates
  float v[kKT][NV];
  T za[kKT], zb[kKT];
  bool on[kKT];
#pragma unroll
  for (int t = 0; t < kKT; ++t) {
    const int k = blockIdx.y * kKT + t;
    on[t] = k < n2;
    const int kk = on[t] ? k : n2 - 1;
    const int gd = (int)h.off[c] + i + n0 * (j + n1 * kk);
    const int o = c == 0 ? i : (c == 1 ? j : kk);
    const int e = o / P, a = o - e * P;
    int tq[3] = {i, j, kk};
    tq[c] = e * P;
    const int n_base = tq[0] + (mx + 1) * (tq[1] + (my + 1) * tq[2]);
    for (int s2 = 0; s2 < NV; ++s2) v[t][s2] = 0.0f;
#pragma unroll
    for (int q = 0; q <= P; ++q) {
      const float w = tab.D[a][q];
#pragma unroll
      for (int s2 = 0; s2 < NV; ++s2) v[t][s2] += w * phi[s2 * nq + n_base + q * stride];
    }
    on[t] = on[t] && !ess[gd];
    za[t] = z0[gd];
    if (NV > 1) zb[t] = z1[gd];
  }
#pragma unroll
  for (int t = 0; t < kKT; ++t) {
    if (!on[t]) continue;
    const int k = blockIdx.y * kKT + t;
    const int gd = (int)h.off[c] + i + n0 * (j + n1 * k);
    if (NV == 1) {
      z0[gd] = za[t] + (T)(c00 * v[t][0]);
    } else {
      z0[gd] = za[t] + (T)(c00 * v[t][0] + c01 * v[t][NV - 1]);
      z1[gd] = zb[t] + (T)(c10 * v[t][0] + c11 * v[t][NV - 1]);
    }
  }
}

// weight of Gauss-Lobatto index I for element vertex i in one direction: the
// trilinear function of vertex i evaluated at that node (I in [(i-1)p, (i+1)p])
__device__ __forceinline__ float wq1d(int I, int i, int p, const AuxTab& tab) {
  if (I < i * p) return tab.gll[I - (i - 1) * p];
  if (I == i * p) return 1.0f;
  return 1.0f - tab.gll[I - i * p];
}
// Gauss-Lobatto grid -> element vertices: b1 = P0^T g (zero at fixed vertices)
template <int NV, int P>
__global__ void k_rq(Dims vd, AuxTab tab, const float* __restrict__ g, const float* __restrict__ dinv1,
                     float* __restrict__ b1, ChebStart cs, const int* __restrict__ done) {
  if (done && *done) return;
  PLANE_IJ(vd.nx, vd.ny, i, j);
  const int mx = vd.nx * P, my = vd.ny * P, mz = vd.nz * P;
  const int nq = (mx + 1) * (my + 1) * (mz + 1), n1 = (int)vd.nodes();
  // 1-D taps with out-of-grid entries clamped and weighted 0 (no branches)
  int ix[2 * P + 1];
  float wx[2 * P + 1];
#pragma unroll
  for (int d = -P; d <= P; ++d) {
    const int Iq = i * P + d;
    const bool in = Iq >= 0 && Iq <= mx;
    ix[d + P] = min(max(Iq, 0), mx);
    wx[d + P] = in ? wq1d(Iq, i, P, tab) : 0.0f;
  }
#pragma unroll
  for (int t = 0; t < kKT; ++t) {
    const int k = blockIdx.y * kKT + t;
    if (k > vd.nz) break;
    const int n = i + (vd.nx + 1) * (j + (vd.ny + 1) * k);
    float acc[NV];
    for (int v = 0; v < NV; ++v) acc[v] = 0.0f;
#pragma unroll
    for (int dz = -P; dz <= P; ++dz) {
      const int Kq = k * P + dz;
      const float wz = (Kq >= 0 && Kq <= mz) ? wq1d(Kq, k, P, tab) : 0.0f;
      const int Kc = min(max(Kq, 0), mz);
#pragma unroll
      for (int dy = -P; dy <= P; ++dy) {
        const int Jq = j * P + dy;
        const float wy = (Jq >= 0 && Jq <= my) ? wq1d(Jq, j, P, tab) * wz : 0.0f;
        const int row = (mx + 1) * (min(max(Jq, 0), my) + (my + 1) * Kc);
#pragma unroll
        for (int dx = 0; dx <= 2 * P; ++dx) {
          const float w = wx[dx] * wy;
#pragma unroll
          for (int v = 0; v < NV; ++v) acc[v] += w * g[v * nq + row + ix[dx]];
        }
      }
    }
    const float d1 = dinv1[n];
#pragma unroll
    for (int v = 0; v < NV; ++v) {
      acc[v] = d1 != 0.0f ? acc[v] : 0.0f;
      b1[v * n1 + n] = acc[v];
    }
    cheb_start_at<NV>(cs, n1, n, d1, acc);
  }
}

// phi = D_L^-1 g + P0 x1 on the Gauss-Lobatto grid (zero at fixed nodes)
template <int NV, int P>
__global__ void k_pq(Dims vd, AuxTab tab, const float* __restrict__ g, const float* __restrict__ qdinv,
                     const float* __restrict__ x1, float* __restrict__ phi, const int* __restrict__ done) {
  if (done && *done) return;
  const Dims qd{vd.nx * P, vd.ny * P, vd.nz * P};
  PLANE_IJ(qd.nx, qd.ny, I, J);
  const int nq = (int)qd.nodes(), n1 = (int)vd.nodes();
  const int sx = vd.nx + 1, sxy = (vd.nx + 1) * (vd.ny + 1);
  const int ex = min(I / P, vd.nx - 1), ey = min(J / P, vd.ny - 1);
  const float xi = tab.gll[I - ex * P], yi = tab.gll[J - ey * P];
  float acc[kKT][NV], dq[kKT];
#pragma unroll
  for (int t = 0; t < kKT; ++t) {  // loads of all planes first
    const int K = min((int)blockIdx.y * kKT + t, qd.nz);
    const int n = I + (qd.nx + 1) * (J + (qd.ny + 1) * K);
    const int ez = min(K / P, vd.nz - 1);
    const float zi = tab.gll[K - ez * P];
    dq[t] = qdinv[n];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[t][v] = dq[t] * g[v * nq + n];
    const int v0 = ex + sx * ey + sxy * ez;
#pragma unroll
    for (int a = 0; a < 8; ++a) {
      const float w = ((a & 1) ? xi : 1.0f - xi) * (((a >> 1) & 1) ? yi : 1.0f - yi) *
                      (((a >> 2) & 1) ? zi : 1.0f - zi);
      const int vn = v0 + (a & 1) + sx * ((a >> 1) & 1) + sxy * ((a >> 2) & 1);
#pragma unroll
      for (int v = 0; v < NV; ++v) acc[t][v] += w * x1[v * n1 + vn];
    }
  }
#pragma unroll
  for (int t = 0; t < kKT; ++t) {
    const int K = blockIdx.y * kKT + t;
    if (K > qd.nz) break;
    const int n = I + (qd.nx + 1) * (J + (qd.ny + 1) * K);
#pragma unroll
    for (int v = 0; v < NV; ++v) phi[v * nq + n] = dq[t] != 0.0f ? acc[t][v] : 0.0f;
  }
}

// diag of L = G^T M_sigma G on the Gauss-Lobatto grid (order p > 1)
__global__ void k_qp_diag(HexDev h, AuxTab tab, const float* __restrict__ facf, float* __restrict__ diag) {
  const int p = tab.p;
  const int mx = h.nx * p, my = h.ny * p;
  const int sym[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};
  GS_LOOP(e, h.ne) {
    const int ex = (int)(e % h.nx), ey = (int)((e / h.nx) % h.ny), ez = (int)(e / ((int64_t)h.nx * h.ny));
    float F[6];
    for (int q = 0; q < 6; ++q) F[q] = facf[(int64_t)q * h.ne + e];
    for (int k = 0; k <= p; ++k)
      for (int j = 0; j <= p; ++j)
        for (int i = 0; i <= p; ++i) {
          const int idx[3] = {i, j, k};
          float s = 0.0f;
          for (int c = 0; c < 3; ++c)
            for (int d = 0; d < 3; ++d) {
              const float f = F[sym[c][d]];
              if (f == 0.0f) continue;
              float prod = f;
              for (int dir = 0; dir < 3; ++dir) {
                const int q = idx[dir];
                float t;
                if (dir == c && dir == d) t = tab.Kd[q];
                else if (dir == c || dir == d) t = 0.5f * ((q == p ? 1.0f : 0.0f) - (q == 0 ? 1.0f : 0.0f));
                else t = tab.Md[q];
                prod *= t;
              }
              s += prod;
            }
          const int64_t n = (ex * p + i) + (int64_t)(mx + 1) * ((ey * p + j) + (int64_t)(my + 1) * (ez * p + k));
          atomicAdd(diag + n, s);
        }
  }
}

// ---- host side ---------------------------------------------------------------------------
static double gll_host(int n, int i) {
  // Gauss-Lobatto nodes on [0, 1] for n = 2..4 points
  if (n == 2) return i == 0 ? 0.0 : 1.0;
  if (n == 3) return 0.5 * i;
  const double s = 0.5 - 0.5 / std::sqrt(5.0);
  const double x[4] = {0.0, s, 1.0 - s, 1.0};
  return x[i];
}

static AuxTab make_tab(int p) {
  AuxTab t{};
  t.p = p;
  Tab1D<double> T1;
  build_tab1d(p, &T1);
  for (int a = 0; a < p; ++a)
    for (int q = 0; q <= p; ++q) t.D[a][q] = (float)T1.D[a][q];
  for (int q = 0; q <= p; ++q) {
    t.gll[q] = (float)gll_host(p + 1, q);
    double k = 0.0;
    for (int a = 0; a < p; ++a)
      for (int b = 0; b < p; ++b) k += T1.D[a][q] * T1.Moo[a][b] * T1.D[b][q];
    t.Kd[q] = (float)k;
    t.Md[q] = (float)T1.Mcc[q][q];
  }
  return t;
}

void auxmg_free(hcop* h) {
  AuxMG* M = static_cast<AuxMG*>(h->aux);
  if (!M) return;
  for (int l = 0; l < M->nlev; ++l) {
    AuxLevel& L = M->lev[l];
    dfree(h, L.Ke);
    dfree(h, L.St);
    dfree(h, L.dinv);
    dfree(h, L.x);
    dfree(h, L.b);
    dfree(h, L.r);
    dfree(h, L.dv);
    dfree(h, L.t);
  }
  for (AuxGraph& g : M->graphs)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (M->cap) cudaStreamDestroy(M->cap);
  dfree(h, M->qdinv);
  dfree(h, M->g);
  dfree(h, M->phi);
  dfree(h, M->bar);
  delete M;
  h->aux = nullptr;
}

// fixed (Dirichlet) node flags of a grid with nx x ny x nz cells
static void face_fixed(int nx, int ny, int nz, int bits, std::vector<uint8_t>& f) {
  f.assign((size_t)(nx + 1) * (ny + 1) * (nz + 1), 0);
  for (int k = 0; k <= nz; ++k)
    for (int j = 0; j <= ny; ++j)
      for (int i = 0; i <= nx; ++i) {
        const bool e = (i == 0 && (bits & 1)) || (i == nx && (bits & 2)) || (j == 0 && (bits & 4)) ||
                       (j == ny && (bits & 8)) || (k == 0 && (bits & 16)) || (k == nz && (bits & 32));
        f[i + (size_t)(nx + 1) * (j + (size_t)(ny + 1) * k)] = e;
      }
}

static void coop_setup(hcop* h, AuxMG* M);

hc_status auxmg_setup(hcop* h) {
  if (h->aux) return HC_OK;
  if (h->type != HC_HEX) {
    h->err = "the auxiliary-space preconditioner needs a structured hex grid";
    return HC_ENOTSUP;
  }
  if (!h->has_mass) {
    h->err = "the auxiliary-space preconditioner needs a mass term (sigma)";
    return HC_ENOTSUP;
  }
  AuxMG* M = new AuxMG();
  h->aux = M;
  const int p = h->p;
  M->p = p;
  M->tab = make_tab(p);
  const HexDev hd = h->hexdev();
  // Gauss-Lobatto grid fixed nodes
  const int mx = h->nx * p, my = h->ny * p, mz = h->nz * p;
  std::vector<uint8_t> qfix;
  if (!h->explicit_mask) {
    face_fixed(mx, my, mz, h->ess_bits, qfix);
  } else {
    qfix.assign((size_t)(mx + 1) * (my + 1) * (mz + 1), 0);
    // a node is fixed when its gradient touches an essential Nedelec dof
    for (int c = 0; c < 3; ++c) {
      const int n0 = mx + (c != 0), n1 = my + (c != 1), n2 = mz + (c != 2);
      for (int k = 0; k < n2; ++k)
        for (int j = 0; j < n1; ++j)
          for (int i = 0; i < n0; ++i) {
            const int64_t gd = h->off[c] + i + (int64_t)n0 * (j + (int64_t)n1 * k);
            if (!h->ess_host[gd]) continue;
            int t[3] = {i, j, k};
            const int e = t[c] / p;
            for (int q = 0; q <= p; ++q) {
              t[c] = e * p + q;
              qfix[t[0] + (size_t)(mx + 1) * (t[1] + (size_t)(my + 1) * t[2])] = 1;
            }
          }
    }
  }
  bool any = false;
  for (uint8_t v : qfix) any |= v != 0;
  if (!any) qfix[0] = 1;  // no Dirichlet node at all: pin one (L is singular on constants)
  // level dimensions
  std::vector<std::vector<uint8_t>> fixed;
  Dims d{h->nx, h->ny, h->nz};
  M->nlev = 0;
  while (true) {
    AuxLevel& L = M->lev[M->nlev];
    L.d = d;
    std::vector<uint8_t> f((size_t)d.nodes());
    if (M->nlev == 0) {
      for (int k = 0; k <= d.nz; ++k)
        for (int j = 0; j <= d.ny; ++j)
          for (int i = 0; i <= d.nx; ++i)
            f[i + (size_t)(d.nx + 1) * (j + (size_t)(d.ny + 1) * k)] =
                qfix[(size_t)i * p + (size_t)(mx + 1) * ((size_t)j * p + (size_t)(my + 1) * ((size_t)k * p))];
    } else {
      const Dims fd = M->lev[M->nlev - 1].d;
      const std::vector<uint8_t>& ff = fixed.back();
      for (int k = 0; k <= d.nz; ++k)
        for (int j = 0; j <= d.ny; ++j)
          for (int i = 0; i <= d.nx; ++i) {
            const int fi = std::min(2 * i, fd.nx), fj = std::min(2 * j, fd.ny), fk = std::min(2 * k, fd.nz);
            f[i + (size_t)(d.nx + 1) * (j + (size_t)(d.ny + 1) * k)] =
                ff[fi + (size_t)(fd.nx + 1) * (fj + (size_t)(fd.ny + 1) * fk)];
          }
    }
    fixed.push_back(f);
    ++M->nlev;
    const Dims c{(d.nx + 1) / 2, (d.ny + 1) / 2, (d.nz + 1) / 2};
    if (d.nodes() <= kAuxCoarseNodes || M->nlev == kAuxMaxLevels || (c.nx == d.nx && c.ny == d.ny && c.nz == d.nz))
      break;
    d = c;
  }
  cudaStream_t s = h->stream;
  auto fail = [&](cudaError_t e) {
    h->err = std::string("auxiliary-space setup: ") + cudaGetErrorString(e);
    auxmg_free(h);
    return HC_ECUDA;
  };
  cudaError_t e = cudaSuccess;
  std::vector<float> hd_diag, hd_abs;
  for (int l = 0; l < M->nlev && e == cudaSuccess; ++l) {
    AuxLevel& L = M->lev[l];
    const int64_t nn = L.d.nodes(), ne = L.d.elems();
    float *diag = nullptr, *absr = nullptr;
    uint8_t* fx = nullptr;
    e = dmalloc(h, (void**)&L.Ke, (size_t)ne * 64 * sizeof(float));
    if (e == cudaSuccess) e = dmalloc(h, (void**)&L.St, (size_t)27 * nn * sizeof(float));
    for (float** v : {&L.dinv, &L.x, &L.b, &L.r, &L.dv, &L.t})
      if (e == cudaSuccess) e = dmalloc(h, (void**)v, (size_t)(v == &L.dinv ? 1 : 2) * nn * sizeof(float));
    if (e == cudaSuccess) e = dmalloc(h, (void**)&diag, 2 * nn * sizeof(float));
    if (e == cudaSuccess) e = dmalloc(h, (void**)&fx, nn);
    if (e != cudaSuccess) {
      dfree(h, diag);
      dfree(h, fx);
      break;
    }
    absr = diag + nn;
    cudaMemsetAsync(diag, 0, 2 * nn * sizeof(float), s);
    cudaMemsetAsync(L.x, 0, 2 * nn * sizeof(float), s);
    cudaMemsetAsync(L.t, 0, 2 * nn * sizeof(float), s);
    cudaMemcpyAsync(fx, fixed[l].data(), nn, cudaMemcpyHostToDevice, s);
    if (l == 0) {
      k_q1_build<<<agrid(ne), 256, 0, s>>>(L.d, h->facf, L.Ke);
    } else {
      AuxLevel& F = M->lev[l - 1];
      k_coarsen<<<agrid(ne), 256, 0, s>>>(F.d, L.d, F.Ke, L.Ke);
    }
    k_stencil<<<agrid(nn), 256, 0, s>>>(L.d, L.Ke, L.St, diag, absr);
    k_finish_dinv<<<agrid(nn), 256, 0, s>>>(nn, diag, fx, L.dinv);
    hd_diag.resize(nn);
    hd_abs.resize(nn);
    std::vector<uint8_t> fxh = fixed[l];
    e = cudaMemcpyAsync(hd_diag.data(), diag, nn * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hd_abs.data(), absr, nn * sizeof(float), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    dfree(h, diag);
    dfree(h, fx);
    if (l > 0) {  // the finer level's element matrices were only needed for this level
      dfree(h, M->lev[l - 1].Ke);
      M->lev[l - 1].Ke = nullptr;
    }
    double lm = 0.0;
    for (int64_t i = 0; i < nn; ++i)
      if (!fxh[i] && hd_diag[i] > 0.0f) lm = std::max(lm, (double)hd_abs[i] / (double)hd_diag[i]);
    L.lmax = lm > 0.0 ? lm : 1.0;
  }
  if (M->nlev > 0 && M->lev[M->nlev - 1].Ke) {
    dfree(h, M->lev[M->nlev - 1].Ke);
    M->lev[M->nlev - 1].Ke = nullptr;
  }
  if (e == cudaSuccess && p > 1) {
    M->q = Dims{mx, my, mz};
    M->nq = M->q.nodes();
    float* diag = nullptr;
    uint8_t* fx = nullptr;
    e = dmalloc(h, (void**)&M->qdinv, M->nq * sizeof(float));
    if (e == cudaSuccess) e = dmalloc(h, (void**)&M->g, 2 * M->nq * sizeof(float));
    if (e == cudaSuccess) e = dmalloc(h, (void**)&M->phi, 2 * M->nq * sizeof(float));
    if (e == cudaSuccess) e = dmalloc(h, (void**)&diag, M->nq * sizeof(float));
    if (e == cudaSuccess) e = dmalloc(h, (void**)&fx, M->nq);
    if (e == cudaSuccess) {
      cudaMemsetAsync(diag, 0, M->nq * sizeof(float), s);
      cudaMemcpyAsync(fx, qfix.data(), M->nq, cudaMemcpyHostToDevice, s);
      k_qp_diag<<<agrid(h->ne), 256, 0, s>>>(hd, M->tab, h->facf, diag);
      k_finish_dinv<<<agrid(M->nq), 256, 0, s>>>(M->nq, diag, fx, M->qdinv);
      e = cudaStreamSynchronize(s);
    }
    dfree(h, diag);
    dfree(h, fx);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return fail(e);
  coop_setup(h, M);
  return HC_OK;
}

// ---- V-cycle ----------------------------------------------------------------------------
struct ChebCoef {
  float inv_theta;
  float c1[kAuxCoarseDegree], c2[kAuxCoarseDegree];
};
static ChebCoef cheb_coef(double lmax, int degree) {
  ChebCoef c{};
  const double lmin = lmax / kAuxRatio;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin), s1 = theta / delta;
  c.inv_theta = (float)(1.0 / theta);
  double rho = 1.0 / s1;
  for (int k = 1; k < degree; ++k) {
    const double rn = 1.0 / (2.0 * s1 - rho);
    c.c1[k - 1] = (float)(rn * rho);
    c.c2[k - 1] = (float)(2.0 * rn / delta);
    rho = rn;
  }
  return c;
}

// Chebyshev smoothing of L x = b on a level: from zero (x = d0, then fused
// steps) or from the current x (residual kernel, then fused steps that also
// add d0).  The two direction buffers are dv and t.
template <int NV>
static void smooth(const hcop* h, AuxLevel& L, int degree, bool from_zero, const int* done, cudaStream_t s) {
  (void)h;
  const int64_t nn = L.d.nodes();
  const ChebCoef c = cheb_coef(L.lmax, degree);
  const unsigned gv = agrid(NV * nn);
  const NodeGrid gn = node_grid(L.d.nx, L.d.ny, L.d.nz);
  // from zero: the kernel that produced L.b already set r, d and x (ChebStart)
  if (!from_zero)
    k_cheb_resid<NV><<<gn.grid, gn.block, 0, s>>>(L.d, L.St, L.dinv, L.b, L.x, L.r, L.dv, c.inv_theta, done);
  float* din = L.dv;
  float* dout = L.t;
  for (int k = 1; k < degree; ++k) {
    k_cheb_fused<NV><<<gn.grid, gn.block, 0, s>>>(L.d, L.St, L.dinv, din, dout, L.r, L.x, c.c1[k - 1],
                                                  c.c2[k - 1], (!from_zero && k == 1) ? 1 : 0, done);
    std::swap(din, dout);
  }
  if (!from_zero && degree == 1) k_add<NV><<<gv, 256, 0, s>>>((int)nn, L.dv, L.x, done);
}

static ChebStart start_of(AuxLevel& L) {
  return ChebStart{L.r, L.dv, L.x, cheb_coef(L.lmax, 1).inv_theta};
}

template <int NV>
static bool vcycle_coop(const hcop* h, AuxMG* M, int l0, const int* done, cudaStream_t s);
template <int NV>
static bool vcycle_cluster(const hcop* h, AuxMG* M, int lr, int l0, const int* done, cudaStream_t s);
static int coop_from_level();
static int vcycle_mode();

template <int NV>
static void vcycle(const hcop* h, AuxMG* M, int l, const int* done, cudaStream_t s) {
  AuxLevel& L = M->lev[l];
  // from the configured level down, the rest of the cycle as one cooperative launch
  if (l == coop_from_level() && vcycle_coop<NV>(h, M, l, done, s)) return;
  const bool cl = vcycle_mode() == kVCluster;
  // a V-cycle whose finest level is small: all of it in one cluster launch
  if (cl && l == 0 && L.d.nodes() <= kSmallLevelNodes && vcycle_cluster<NV>(h, M, -1, 0, done, s)) return;
  if (l == M->nlev - 1) {
    smooth<NV>(h, L, kAuxCoarseDegree, true, done, s);
    return;
  }
  AuxLevel& C = M->lev[l + 1];
  smooth<NV>(h, L, kAuxDegree, true, done, s);
  // r = b - L x (masked), restricted
  const NodeGrid gl = node_grid(L.d.nx, L.d.ny, L.d.nz), gc = node_grid(C.d.nx, C.d.ny, C.d.nz);
  k_cheb_resid<NV><<<gl.grid, gl.block, 0, s>>>(L.d, L.St, L.dinv, L.b, L.x, L.r, L.dv, 1.0f, done);
  // the coarse levels below a large one: restriction and their cycle in one cluster launch
  if (!(cl && C.d.nodes() <= kSmallLevelNodes && vcycle_cluster<NV>(h, M, l, l + 1, done, s))) {
    k_restrict<NV><<<gc.grid, gc.block, 0, s>>>(L.d, C.d, L.r, C.dinv, C.b, start_of(C), done);
    vcycle<NV>(h, M, l + 1, done, s);
  }
  k_prolong_add<NV><<<gl.grid, gl.block, 0, s>>>(L.d, C.d, C.x, L.dinv, L.x, done);
  smooth<NV>(h, L, kAuxDegree, false, done, s);
}

// ---- the V-cycle as one cooperative launch ------------------------------------------------
// (The per-node functions above spell their roundings out with __fmaf_rn /
// __fmul_rn / __fadd_rn, so that the compiler's FMA contraction cannot differ
// between the kernels that inline them.)
// The per-step kernels above run one launch per smoothing step, residual,
// restriction and prolongation (21 launches for four levels), most of them on
// grids of a few thousand nodes, where launch latency and the drain between
// dependent kernels cost more than the work.  k_vcycle runs the same steps, in
// the same order and with the same per-node arithmetic (results are
// bit-identical), in one cooperative launch of co-resident blocks that meet
// at a grid barrier between steps.
constexpr int kVThreads = 512;
constexpr int kMaxVSteps = 64;
constexpr unsigned kBarSpins = 1u << 23;  // >= ~1 s of polling (L2 round trips) before a wait gives up
enum : int { kOpFused = 0, kOpResid = 1, kOpRestrict = 2, kOpProlong = 3, kOpAdd = 4 };

struct VStep {
  int op, lev;       // level the step writes (restrict: the fine level it reads)
  int add_in, swap;  // fused step: add d_in to x; swap: d_in = t, d_out = dv (else the reverse)
  float c1, c2;      // fused step coefficients; resid: c1 = 1/theta
};
struct VLevelDev {
  Dims d;
  const float* St;
  const float* dinv;
  float *x, *b, *r, *dv, *t;
  float start_inv_theta;  // 1/theta of the level's first smoothing step (restriction target)
};
struct VCycleArgs {
  int nlev, nsteps;
  CoopBar* bar;
  VLevelDev lev[kAuxMaxLevels];
  VStep step[kMaxVSteps];
};

// All blocks arrive; the last one opens the next generation.  Waits poll with
// a bound: a wait that gives up sets bar->err, and every block leaves.
__device__ __forceinline__ bool coop_sync(CoopBar* bar) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned* vg = &bar->gen;
    volatile int* ve = &bar->err;
    const unsigned g = *vg;
    __threadfence();
    if (atomicAdd(&bar->count, 1u) == gridDim.x - 1) {
      bar->count = 0u;
      __threadfence();
      atomicExch(&bar->gen, g + 1u);
    } else {
      unsigned spins = 0;
      while (*vg == g && *ve == 0) {
        if (++spins > kBarSpins) {
          atomicExch(&bar->err, 1);
          break;
        }
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *(volatile int*)&bar->err == 0;
}

// One step of the V-cycle step list over the level's nodes, thread gt of gs.
template <int NV>
__device__ __forceinline__ void run_step(const VCycleArgs& a, const VStep& st, int64_t gt, int64_t gs) {
  const VLevelDev& L = a.lev[st.lev];
  if (st.op == kOpRestrict) {
    const VLevelDev& C = a.lev[st.lev + 1];
    const ChebStart cs{C.r, C.dv, C.x, C.start_inv_theta};
    const int nx1 = C.d.nx + 1, ny1 = C.d.ny + 1, nn = (int)C.d.nodes();
    for (int64_t q = gt; q < nn; q += gs) {
      const int n = (int)q, i = n % nx1, t = n / nx1, j = t % ny1, k = t / ny1;
      restrict_at<NV, true>(L.d, C.d, L.r, C.dinv, C.b, cs, n, i, j, k);
    }
    return;
  }
  const int nx1 = L.d.nx + 1, ny1 = L.d.ny + 1, nn = (int)L.d.nodes();
  const float* din = st.swap ? L.t : L.dv;
  float* dout = st.swap ? L.dv : L.t;
  for (int64_t q = gt; q < nn; q += gs) {
    const int n = (int)q, i = n % nx1, t = n / nx1, j = t % ny1, k = t / ny1;
    switch (st.op) {
      case kOpFused:
        cheb_fused_at<NV, true>(L.d, L.St, L.dinv, din, dout, L.r, L.x, st.c1, st.c2, st.add_in, n, i, j, k);
        break;
      case kOpResid: cheb_resid_at<NV, true>(L.d, L.St, L.dinv, L.b, L.x, L.r, L.dv, st.c1, n, i, j, k); break;
      case kOpProlong: {
        const VLevelDev& C = a.lev[st.lev + 1];
        prolong_add_at<NV, true>(L.d, C.d, C.x, L.dinv, L.x, n, i, j, k);
        break;
      }
      default:
#pragma unroll
        for (int v = 0; v < NV; ++v)
          L.x[v * nn + n] = __fadd_rn(vld<true>(L.x + v * nn + n), vld<true>(L.dv + v * nn + n));
        break;
    }
  }
}

template <int NV>
__global__ void __launch_bounds__(kVThreads) k_vcycle(const __grid_constant__ VCycleArgs a,
                                                      const int* __restrict__ done) {
  if (done && *done) return;
  const int64_t gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, gs = (int64_t)gridDim.x * blockDim.x;
  bool ok = *(volatile int*)&a.bar->err == 0;
  for (int s = 0; s < a.nsteps && ok; ++s) {
    run_step<NV>(a, a.step[s], gt, gs);
    if (s + 1 < a.nsteps) ok = coop_sync(a.bar);
  }
  if (!ok && blockIdx.x == 0 && threadIdx.x == 0) {
    // a barrier wait gave up: the correction is NaN, which the Krylov
    // reductions turn into HC_BREAKDOWN
    const int nn = (int)a.lev[0].d.nodes();
    for (int v = 0; v < NV; ++v) a.lev[0].x[v * nn] = __int_as_float(0x7fc00000);
  }
}

// The coarse levels (<= kSmallLevelNodes nodes) of the V-cycle in one launch
// of one thread-block cluster: kClusterCtas CTAs of kClusterThreads threads
// walk the step list and meet at the cluster's hardware barrier between steps
// (barrier.cluster arrive/wait: release/acquire at cluster scope; every
// thread reaches every barrier, the loops over nodes sit between them).  On
// grids of a few thousand nodes a step is one or two L2 round trips, far
// below the launch and drain of a separate kernel.

template <int NV>
__global__ void __launch_bounds__(kClusterThreads, 1) k_vcycle_cluster(const __grid_constant__ VCycleArgs a,
                                                                       const int* __restrict__ done) {
  if (done && *done) return;  // the flag is the same for every thread: all leave before any barrier
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int64_t gt = (int64_t)cl.block_rank() * blockDim.x + threadIdx.x;
  const int64_t gs = (int64_t)kClusterCtas * blockDim.x;
  for (int s = 0; s < a.nsteps; ++s) {
    run_step<NV>(a, a.step[s], gt, gs);
    if (s + 1 < a.nsteps) cl.sync();
  }
}

// The step list of vcycle(0) (same order and coefficients as the per-step launches).
static void smooth_steps(const AuxMG* M, int l, int degree, bool from_zero, std::vector<VStep>& out) {
  const ChebCoef c = cheb_coef(M->lev[l].lmax, degree);
  if (!from_zero) out.push_back(VStep{kOpResid, l, 0, 0, c.inv_theta, 0.0f});
  int swap = 0;
  for (int k = 1; k < degree; ++k) {
    out.push_back(VStep{kOpFused, l, (!from_zero && k == 1) ? 1 : 0, swap, c.c1[k - 1], c.c2[k - 1]});
    swap ^= 1;
  }
  if (!from_zero && degree == 1) out.push_back(VStep{kOpAdd, l, 0, 0, 0.0f, 0.0f});
}
static void vcycle_steps(const AuxMG* M, int l, std::vector<VStep>& out) {
  if (l == M->nlev - 1) {
    smooth_steps(M, l, kAuxCoarseDegree, true, out);
    return;
  }
  smooth_steps(M, l, kAuxDegree, true, out);
  out.push_back(VStep{kOpResid, l, 0, 0, 1.0f, 0.0f});
  out.push_back(VStep{kOpRestrict, l, 0, 0, 0.0f, 0.0f});
  vcycle_steps(M, l + 1, out);
  out.push_back(VStep{kOpProlong, l, 0, 0, 0.0f, 0.0f});
  smooth_steps(M, l, kAuxDegree, false, out);
}

// Form of the Q1 V-cycle, from HC_AUX_VCYCLE (read at every application, so one
// handle can run every form; all forms are bit-identical):
//   "kernels" (default): one launch per step, replayed from a CUDA graph;
//   "cluster": per-step kernels on the large levels, the coarse levels
//              (<= kSmallLevelNodes nodes) in one thread-block-cluster launch;
//   "coop":    every level in one cooperative launch (grid barriers);
//   "hybrid":  the levels below the finest in one cooperative launch.
// Measured per preconditioner application at 64^3 / 48^3 p = 2: kernels 258 /
// 158 us, cluster 262 / 163 us, hybrid 275 / 184 us, coop 297 / 204 us.  Inside
// a graph, consecutive small kernels overlap their launch and drain, so a
// coarse-level step costs about as much as a cluster barrier plus the L2
// round trips of the single-launch forms (whose level vectors must bypass L1:
// their blocks read what other blocks wrote in the same launch).
static int vcycle_mode() {
  const char* env = std::getenv("HC_AUX_VCYCLE");
  if (env && std::strcmp(env, "cluster") == 0) return kVCluster;
  if (env && std::strcmp(env, "coop") == 0) return kVCoop;
  if (env && std::strcmp(env, "hybrid") == 0) return kVHybrid;
  return kVKernels;
}
static int coop_from_level() {
  const int m = vcycle_mode();
  return m == kVCoop ? 0 : (m == kVHybrid ? 1 : -1);
}

// false: not available (no cooperative support, too many steps); the caller
// issues the per-step kernels
template <int NV>
static bool vcycle_coop(const hcop* h, AuxMG* M, int l0, const int* done, cudaStream_t s) {
  (void)h;
  const int blocks = NV == 1 ? M->coop_blocks : M->coop_blocks2;
  if (!M->bar || blocks <= 0 || l0 < 0 || l0 >= M->nlev) return false;
  std::vector<VStep> steps;
  vcycle_steps(M, l0, steps);
  if ((int)steps.size() > kMaxVSteps) return false;
  VCycleArgs a{};
  a.nlev = M->nlev;
  a.nsteps = (int)steps.size();
  a.bar = M->bar;
  for (int l = 0; l < M->nlev; ++l) {
    const AuxLevel& L = M->lev[l];
    a.lev[l] = VLevelDev{L.d, L.St, L.dinv, L.x, L.b, L.r, L.dv, L.t, cheb_coef(L.lmax, 1).inv_theta};
  }
  for (int k = 0; k < a.nsteps; ++k) a.step[k] = steps[k];
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(kVThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  // a failed launch is also the thread's last error, which the caller reads
  (void)cudaLaunchKernelEx(&cfg, k_vcycle<NV>, a, done);
  return true;
}

// Restriction lr -> lr + 1 (lr >= 0) and the whole cycle from level l0 down, in
// one cluster launch; false if clusters are unavailable or the list is too long.
template <int NV>
static bool vcycle_cluster(const hcop* h, AuxMG* M, int lr, int l0, const int* done, cudaStream_t s) {
  (void)h;
  if (!M->cluster_ok || l0 < 0 || l0 >= M->nlev) return false;
  std::vector<VStep> steps;
  if (lr >= 0) steps.push_back(VStep{kOpRestrict, lr, 0, 0, 0.0f, 0.0f});
  vcycle_steps(M, l0, steps);
  if ((int)steps.size() > kMaxVSteps) return false;
  VCycleArgs a{};
  a.nlev = M->nlev;
  a.nsteps = (int)steps.size();
  a.bar = M->bar;
  for (int l = 0; l < M->nlev; ++l) {
    const AuxLevel& L = M->lev[l];
    a.lev[l] = VLevelDev{L.d, L.St, L.dinv, L.x, L.b, L.r, L.dv, L.t, cheb_coef(L.lmax, 1).inv_theta};
  }
  for (int k = 0; k < a.nsteps; ++k) a.step[k] = steps[k];
  cudaLaunchConfig_t cfg{};
  cfg.gridDim = dim3(kClusterCtas);
  cfg.blockDim = dim3(kClusterThreads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = kClusterCtas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  // a failed launch is also the thread's last error, which the caller reads
  (void)cudaLaunchKernelEx(&cfg, k_vcycle_cluster<NV>, a, done);
  return true;
}

// Blocks of the cooperative V-cycle: co-resident by construction (occupancy
// x SMs, at most 2 per SM); 0 when the device cannot launch cooperatively.
static void coop_setup(hcop* h, AuxMG* M) {
  M->coop_blocks = M->coop_blocks2 = 0;
  // thread-block clusters of kClusterCtas: at least one must fit for each NV
  {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(kClusterCtas);
    cfg.blockDim = dim3(kClusterThreads);
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = kClusterCtas;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int c1 = 0, c2 = 0;
    const bool ok = cudaOccupancyMaxActiveClusters(&c1, k_vcycle_cluster<1>, &cfg) == cudaSuccess &&
                    cudaOccupancyMaxActiveClusters(&c2, k_vcycle_cluster<2>, &cfg) == cudaSuccess;
    if (!ok) cudaGetLastError();
    M->cluster_ok = ok && c1 > 0 && c2 > 0;
  }
  int dev = 0, coop = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return;
  if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) return;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return;
  int b1 = 0, b2 = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b1, k_vcycle<1>, kVThreads, 0) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, k_vcycle<2>, kVThreads, 0) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  if (b1 < 1 || b2 < 1) return;
  if (dmalloc(h, (void**)&M->bar, sizeof(CoopBar)) != cudaSuccess) {
    M->bar = nullptr;
    cudaGetLastError();
    return;
  }
  if (cudaMemsetAsync(M->bar, 0, sizeof(CoopBar), h->stream) != cudaSuccess) return;
  // one block per SM: the coarse levels have few nodes, and every block is
  // one arrival at each grid barrier
  M->coop_blocks = sms;
  M->coop_blocks2 = sms;
}

// z += C G V G^T r   (NV = 1: real r, coefficient c00; NV = 2: planar complex,
// z_0 += c00 v_0 + c01 v_1, z_1 += c10 v_0 + c11 v_1)
template <typename T, int NV, int P>
static void aux_apply_p(const hcop* h, AuxMG* M, const T* r0, const T* r1, T* z0, T* z1, const float coef[4],
                        const int* done, cudaStream_t s) {
  const HexDev hd = h->hexdev();
  AuxLevel& L0 = M->lev[0];
  const int mx = h->nx * P, my = h->ny * P, mz = h->nz * P;
  float* g = P > 1 ? M->g : L0.b;
  const float* qd = P > 1 ? M->qdinv : L0.dinv;
  const NodeGrid gq = node_grid_kt(mx, my, mz), g1 = node_grid_kt(L0.d.nx, L0.d.ny, L0.d.nz);
  const ChebStart none{nullptr, nullptr, nullptr, 0.0f};
  k_gt<T, NV, P><<<gq.grid, gq.block, 0, s>>>(hd, M->tab, r0, r1, qd, g, P > 1 ? none : start_of(L0), done);
  if (P > 1) k_rq<NV, P><<<g1.grid, g1.block, 0, s>>>(L0.d, M->tab, g, L0.dinv, L0.b, start_of(L0), done);
  vcycle<NV>(h, M, 0, done, s);
  const float* phi = L0.x;  // order 1: phi is the finest Q1 level's x
  if (P > 1) {
    k_pq<NV, P><<<gq.grid, gq.block, 0, s>>>(L0.d, M->tab, g, M->qdinv, L0.x, M->phi, done);
    phi = M->phi;
  }
  // z += C G phi, one launch per Nedelec component (grid open along c)
  const NodeGrid c0 = node_grid_kt(mx - 1, my, mz), c1 = node_grid_kt(mx, my - 1, mz),
                 c2 = node_grid_kt(mx, my, mz - 1);
  k_g<T, NV, P, 0><<<c0.grid, c0.block, 0, s>>>(hd, M->tab, phi, h->ess, z0, z1, coef[0], coef[1], coef[2], coef[3],
                                                done);
  k_g<T, NV, P, 1><<<c1.grid, c1.block, 0, s>>>(hd, M->tab, phi, h->ess, z0, z1, coef[0], coef[1], coef[2], coef[3],
                                                done);
  k_g<T, NV, P, 2><<<c2.grid, c2.block, 0, s>>>(hd, M->tab, phi, h->ess, z0, z1, coef[0], coef[1], coef[2], coef[3],
                                                done);
}

// z += C G V G^T r   (NV = 1: real r, coefficient c00; NV = 2: planar complex,
// z_0 += c00 v_0 + c01 v_1, z_1 += c10 v_0 + c11 v_1)
template <typename T, int NV>
static void aux_apply_any(const hcop* h, AuxMG* M, const T* r0, const T* r1, T* z0, T* z1, const float coef[4],
                          const int* done, cudaStream_t s) {
  switch (M->p) {
    case 1: aux_apply_p<T, NV, 1>(h, M, r0, r1, z0, z1, coef, done, s); break;
    case 2: aux_apply_p<T, NV, 2>(h, M, r0, r1, z0, z1, coef, done, s); break;
    default: aux_apply_p<T, NV, 3>(h, M, r0, r1, z0, z1, coef, done, s); break;
  }
}

// The ~40 small kernels of one application are captured once per argument
// set into a CUDA graph and replayed with one launch (host-driven Krylov
// loops would otherwise be bound by launch overhead).  Inside a stream that
// is itself being captured (a graph-driven solve) the kernels are issued
// directly and become part of that graph.
template <typename T, int NV>
cudaError_t auxmg_apply(const hcop* h, const T* r0, const T* r1, T* z0, T* z1, const float coef[4], const int* done,
                        cudaStream_t s) {
  AuxMG* M = static_cast<AuxMG*>(h->aux);
  if (!M || M->p < 1 || M->p > 3) return cudaErrorInvalidValue;
  cudaStreamCaptureStatus cst = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cst);
  if (e != cudaSuccess) return e;
  if (cst != cudaStreamCaptureStatusNone) {
    aux_apply_any<T, NV>(h, M, r0, r1, z0, z1, coef, done, s);
    return cudaGetLastError();
  }
  const void* key[5] = {r0, r1, z0, z1, done};
  const int coop = vcycle_mode();
  for (AuxGraph& g : M->graphs) {
    if (g.exec && g.nv == NV && g.tsize == (int)sizeof(T) && g.coop == coop &&
        std::memcmp(g.key, key, sizeof(key)) == 0 && std::memcmp(g.coef, coef, sizeof(g.coef)) == 0)
      return cudaGraphLaunch(g.exec, s);
  }
  if (!M->cap) {
    e = cudaStreamCreateWithFlags(&M->cap, cudaStreamNonBlocking);
    if (e != cudaSuccess) return e;
  }
  e = cudaStreamBeginCapture(M->cap, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return e;
  aux_apply_any<T, NV>(h, M, r0, r1, z0, z1, coef, done, M->cap);
  const cudaError_t le = cudaGetLastError();
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(M->cap, &graph);
  if (le != cudaSuccess || e != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return le != cudaSuccess ? le : e;
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return e;
  AuxGraph* slot = nullptr;
  if ((int)M->graphs.size() < kAuxGraphs) {
    M->graphs.emplace_back();
    slot = &M->graphs.back();
  } else {
    // the replaced graph may still have a launch in flight
    cudaDeviceSynchronize();
    slot = &M->graphs[M->next_graph++ % kAuxGraphs];
    cudaGraphExecDestroy(slot->exec);
  }
  slot->exec = exec;
  std::memcpy(slot->key, key, sizeof(key));
  std::memcpy(slot->coef, coef, sizeof(slot->coef));
  slot->nv = NV;
  slot->tsize = (int)sizeof(T);
  slot->coop = coop;
  return cudaGraphLaunch(exec, s);
}

template cudaError_t auxmg_apply<double, 1>(const hcop*, const double*, const double*, double*, double*,
                                            const float*, const int*, cudaStream_t);
template cudaError_t auxmg_apply<float, 1>(const hcop*, const float*, const float*, float*, float*, const float*,
                                           const int*, cudaStream_t);
template cudaError_t auxmg_apply<double, 2>(const hcop*, const double*, const double*, double*, double*,
                                            const float*, const int*, cudaStream_t);
template cudaError_t auxmg_apply<float, 2>(const hcop*, const float*, const float*, float*, float*, const float*,
                                           const int*, cudaStream_t);

}  // namespace hc

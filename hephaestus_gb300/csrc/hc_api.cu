// hc_api.cu -- C ABI of the GB300 H(curl) operator library (include/hcurl_op.h).
//
// Setup computes, in FP64 on the host, the per-element affine factors of the
// structured hex grid and the essential-dof mask, uploads them once, and
// forms the operator diagonal on the device.  Every entry point validates its
// arguments and returns a status; nothing aborts.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "hc_internal.h"

namespace {

thread_local std::string g_create_err;

// ---- 1-D bases (host, FP64) -------------------------------------------------
// Gauss-Legendre nodes/weights on [0,1] by Newton iteration on P_n.
void gl01(int n, double* x, double* w) {
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5)), p0 = 1, p1 = 0, dp = 1;
    for (int it = 0; it < 100; ++it) {
      p0 = 1.0;
      p1 = 0.0;
      for (int k = 1; k <= n; ++k) {
        const double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
      }
      dp = n * (z * p0 - p1) / (z * z - 1.0);
      const double dz = p0 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    p0 = 1.0;
    p1 = 0.0;
    for (int k = 1; k <= n; ++k) {
      const double p2 = p1;
      p1 = p0;
      p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
    }
    dp = n * (z * p0 - p1) / (z * z - 1.0);
    x[n - 1 - i] = 0.5 * (1.0 + z);
    w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}
// Gauss-Lobatto nodes on [0,1]: endpoints plus the roots of
// f(z) = P_{N-1}(z) - z P_N(z) = (1 - z^2) P'_N(z) / N,  N = n - 1, by Newton.
void gll01(int n, double* x) {
  const double pi = 3.14159265358979323846;
  const int N = n - 1;
  x[0] = 0.0;
  x[N] = 1.0;
  for (int i = 1; i < N; ++i) {
    double z = -std::cos(pi * i / N);
    for (int it = 0; it < 100; ++it) {
      double P[16];
      P[0] = 1.0;
      P[1] = z;
      for (int k = 2; k <= N; ++k) P[k] = ((2.0 * k - 1.0) * z * P[k - 1] - (k - 1.0) * P[k - 2]) / k;
      auto dP = [&](int m) { return m == 0 ? 0.0 : m * (P[m - 1] - z * P[m]) / (1.0 - z * z); };
      const double f = P[N - 1] - z * P[N];
      const double fp = dP(N - 1) - P[N] - z * dP(N);
      const double dz = f / fp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    x[i] = 0.5 * (1.0 + z);
  }
  std::sort(x, x + n);
}
void lagrange(const double* nodes, int m, double t, double* v, double* d) {
  for (int j = 0; j < m; ++j) {
    double pv = 1.0, s = 0.0;
    for (int k = 0; k < m; ++k)
      if (k != j) pv *= (t - nodes[k]) / (nodes[j] - nodes[k]);
    for (int l = 0; l < m; ++l) {
      if (l == j) continue;
      double pr = 1.0 / (nodes[j] - nodes[l]);
      for (int k = 0; k < m; ++k)
        if (k != j && k != l) pr *= (t - nodes[k]) / (nodes[j] - nodes[k]);
      s += pr;
    }
    v[j] = pv;
    d[j] = s;
  }
}

bool finite_nonneg(const double* a, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!(a[i] >= 0.0) || !std::isfinite(a[i])) return false;
  return true;
}

}  // namespace

namespace hc {
void build_tab1d(int p, Tab1D<double>* t) {
  std::memset(t, 0, sizeof(*t));
  double xc[kMaxP + 1], xo[kMaxP], wo[kMaxP];
  gll01(p + 1, xc);
  gl01(p, xo, wo);
  const int nq = p + 2;
  std::vector<double> xq(nq), wq(nq);
  gl01(nq, xq.data(), wq.data());
  double cv[kMaxP + 1], cd[kMaxP + 1], ov[kMaxP], od[kMaxP];
  for (int q = 0; q < nq; ++q) {
    lagrange(xc, p + 1, xq[q], cv, cd);
    lagrange(xo, p, xq[q], ov, od);
    for (int i = 0; i <= p; ++i) {
      for (int j = 0; j <= p; ++j) t->Mcc[i][j] += wq[q] * cv[i] * cv[j];
      for (int j = 0; j < p; ++j) t->Mco[i][j] += wq[q] * cv[i] * ov[j];
    }
    for (int i = 0; i < p; ++i)
      for (int j = 0; j < p; ++j) t->Moo[i][j] += wq[q] * ov[i] * ov[j];
  }
  for (int a = 0; a < p; ++a) {
    lagrange(xc, p + 1, xo[a], cv, cd);
    for (int j = 0; j <= p; ++j) t->D[a][j] = cd[j];
  }
}
}  // namespace hc

namespace hc {
cudaError_t dmalloc(const hcop* h, void** p, size_t bytes) {
  static std::once_flag once;
  std::call_once(once, [] {
    // keep freed blocks in the pool instead of returning them to the driver at
    // every synchronisation (a process-local setting of this device's pool)
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  });
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  return cudaMallocAsync(p, bytes, h->stream);
}
void dfree(const hcop* h, void* p) {
  if (p) cudaFreeAsync(p, h->stream);
}
namespace {
std::mutex g_pin_mu;
std::vector<void*> g_pin_free;
}  // namespace
void* pinned_get(size_t bytes) {
  if (bytes > 4096) return nullptr;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  if (!g_pin_free.empty()) {
    void* p = g_pin_free.back();
    g_pin_free.pop_back();
    std::memset(p, 0, 4096);
    return p;
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, 4096) != cudaSuccess) return nullptr;
  std::memset(p, 0, 4096);
  return p;
}
void pinned_put(void* p) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pin_mu);
  g_pin_free.push_back(p);
}
}  // namespace hc

using namespace hc;

// The 1-D tables in constant memory are uploaded once per process (handles
// may be created from several host threads).
static bool tables_ready() {
  static std::mutex mu;
  static bool ok = false;
  std::lock_guard<std::mutex> lk(mu);
  if (!ok) ok = upload_tables() == cudaSuccess;
  return ok;
}

static hc_status fail_create(hcop* h, const std::string& msg, hc_status st) {
  g_create_err = msg;
  if (h) hc_destroy(h);
  return st;
}

static bool alloc_common(hcop* h) {
  const int64_t N = h->ndof;
  auto ok = [](cudaError_t e) { return e == cudaSuccess; };
  return ok(dmalloc(h, (void**)&h->ess, N)) && ok(dmalloc(h, (void**)&h->diag, N * 8)) &&
         ok(dmalloc(h, (void**)&h->dinv, N * 8)) && ok(dmalloc(h, (void**)&h->dinvf, N * 4)) &&
         ok(dmalloc(h, (void**)&h->sdinv, N * 8)) && ok(dmalloc(h, (void**)&h->sdinvf, N * 4)) &&
         ok(dmalloc(h, (void**)&h->xbuf, N * 8)) && ok(dmalloc(h, (void**)&h->ybuf, N * 8));
}

// Tetrahedral mesh: host topology + closed-form FP64 element matrices on the device.
static hc_status create_tet(const hc_problem_desc* desc, hcop_t** out) {
  if (desc->order < 1 || desc->order > 2) return fail_create(nullptr, "hc_create: tet order must be 1 or 2", HC_EINVAL);
  if (desc->n_vert < 4 || desc->n_elem < 1 || !desc->vertices || !desc->elem_verts)
    return fail_create(nullptr, "hc_create: tet mesh needs vertices and elem_verts", HC_EINVAL);
  if (!desc->nu) return fail_create(nullptr, "hc_create: nu is required", HC_EINVAL);
  if (!(desc->dt > 0.0) || !std::isfinite(desc->dt))
    return fail_create(nullptr, "hc_create: dt must be finite and > 0", HC_EINVAL);
  if (!finite_nonneg(desc->nu, desc->n_elem))
    return fail_create(nullptr, "hc_create: nu must be finite and >= 0", HC_EINVAL);
  if (desc->sigma && !finite_nonneg(desc->sigma, desc->n_elem))
    return fail_create(nullptr, "hc_create: sigma must be finite and >= 0", HC_EINVAL);
  hcop* h = new hcop();
  h->type = HC_TET;
  h->p = desc->order;
  h->ne = desc->n_elem;
  h->n_vert = desc->n_vert;
  h->dt = desc->dt;
  h->has_mass = desc->sigma != nullptr;
  std::vector<int32_t> edofs, sv;
  hc_status st = tet_topology(h, desc, edofs, sv);
  if (st != HC_OK) return fail_create(h, h->err, st);
  const int L = h->p == 1 ? 6 : 20;
  const int64_t N = h->ndof;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return fail_create(h, "hc_create: no CUDA device available", HC_ECUDA);
  const size_t need = (size_t)h->ne * L * L * 12 + (size_t)h->ne * L * 4 + (size_t)N * (1 + 8 * 3 + 4 * 2 + 8 * 8);
  if (need > fr) return fail_create(h, "hc_create: problem exceeds free device memory", HC_ENOMEM);
  if (!tables_ready()) return fail_create(h, "hc_create: constant table upload failed", HC_ECUDA);
  if (!alloc_common(h)) return fail_create(h, "hc_create: device allocation failed", HC_ENOMEM);
  if (dmalloc(h, (void**)&h->nu, h->ne * sizeof(double)) != cudaSuccess)
    return fail_create(h, "hc_create: device allocation failed", HC_ENOMEM);
  cudaMemcpyAsync(h->nu, desc->nu, h->ne * sizeof(double), cudaMemcpyHostToDevice, h->stream);
  cudaMemcpyAsync(h->ess, h->ess_host.data(), N, cudaMemcpyHostToDevice, h->stream);
  cudaError_t e = tet_setup_device(h, desc, edofs, sv);
  if (e == cudaErrorInvalidValue && h->err.empty())
    return fail_create(h, "hc_create: degenerate (zero-volume) tet", HC_EINVAL);
  if (e != cudaSuccess) return fail_create(h, "hc_create: " + h->err + " " + cudaGetErrorString(e), HC_ECUDA);
  e = diag_finish(N, h->ess, h->diag, h->dinv, h->dinvf, h->sdinv, h->sdinvf, h->stream);
  if (e == cudaErrorInvalidValue)
    return fail_create(h, "hc_create: operator diagonal is not positive (nu = 0 and sigma = 0 somewhere?)",
                       HC_EINVAL);
  if (e != cudaSuccess) return fail_create(h, std::string("hc_create: ") + cudaGetErrorString(e), HC_ECUDA);
  if (ensure_scalars(h) != cudaSuccess) return fail_create(h, "hc_create: scalar allocation failed", HC_ENOMEM);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess) return fail_create(h, "hc_create: setup failed", HC_ECUDA);
  *out = h;
  return HC_OK;
}

extern "C" {

hc_status hc_last_error(const hcop_t* h, char* buf, size_t n) {
  if (!buf || n == 0) return HC_EINVAL;
  const std::string& s = h ? h->err : g_create_err;
  std::snprintf(buf, n, "%s", s.c_str());
  return HC_OK;
}

int64_t hc_num_dofs(const hcop_t* h) { return h ? h->ndof : -1; }
int64_t hc_num_elems(const hcop_t* h) { return h ? h->ne : -1; }

int64_t hc_hex_dof_index(const hcop_t* h, int c, int64_t i, int64_t j, int64_t k) {
  if (!h || h->type != HC_HEX || c < 0 || c > 2) return -1;
  const int64_t nxo = (int64_t)h->nx * h->p, nyo = (int64_t)h->ny * h->p, nzo = (int64_t)h->nz * h->p;
  const int64_t n0 = nxo + (c != 0), n1 = nyo + (c != 1), n2 = nzo + (c != 2);
  if (i < 0 || j < 0 || k < 0 || i >= n0 || j >= n1 || k >= n2) return -1;
  return h->off[c] + i + n0 * (j + n1 * k);
}

hc_status hc_get_ess_mask(const hcop_t* h, uint8_t* mask) {
  if (!h || !mask) return HC_EINVAL;
  std::memcpy(mask, h->ess_host.data(), h->ess_host.size());
  return HC_OK;
}

hc_status hc_set_stream(hcop_t* h, void* stream) {
  if (!h) return HC_EINVAL;
  // everything queued on the old stream completes before the handle moves
  HC_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  h->stream = (cudaStream_t)stream;
  return HC_OK;
}

void hc_destroy(hcop_t* h) {
  if (!h) return;
  // work still queued on the handle's stream may read these buffers (and copy
  // into the pinned scalars): let it finish, on this stream only
  cudaStreamSynchronize(h->stream);
  complex_free(h);
  auxmg_free(h);
  multi_free(h);
  tetaux_free(h);
  if (h->mass_child) hc_destroy(h->mass_child);
  for (void* p : {(void*)h->nu, (void*)h->fac, (void*)h->facf, (void*)h->ess, (void*)h->diag, (void*)h->dinv, (void*)h->dinvf,
                  (void*)h->sdinv, (void*)h->sdinvf, (void*)h->scal, (void*)h->partials, h->work, (void*)h->xbuf,
                  (void*)h->ybuf, (void*)h->verts, (void*)h->tet_edofs, (void*)h->tet_sv, (void*)h->tetK64, (void*)h->tetK32,
                  h->tetK16, (void*)h->tab, (void*)h->tab1})
    dfree(h, p);
  pinned_put(h->hscal);
  delete h;
}

hc_status hc_create(const hc_problem_desc* desc, hcop_t** out) {
  if (!desc || !out) return fail_create(nullptr, "hc_create: null argument", HC_EINVAL);
  *out = nullptr;
  if (desc->elem_type == HC_TET) return create_tet(desc, out);
  if (desc->elem_type != HC_HEX) return fail_create(nullptr, "hc_create: unknown elem_type", HC_EINVAL);
  if (desc->order < 1 || desc->order > kMaxP)
    return fail_create(nullptr, "hc_create: hex order must be 1..3", HC_EINVAL);
  if (desc->nx < 1 || desc->ny < 1 || desc->nz < 1)
    return fail_create(nullptr, "hc_create: nx, ny, nz must be >= 1", HC_EINVAL);
  if (!desc->nu) return fail_create(nullptr, "hc_create: nu is required", HC_EINVAL);
  if (!(desc->dt > 0.0) || !std::isfinite(desc->dt))
    return fail_create(nullptr, "hc_create: dt must be finite and > 0", HC_EINVAL);
  const int p = desc->order, nx = desc->nx, ny = desc->ny, nz = desc->nz;
  const int64_t ne = (int64_t)nx * ny * nz;
  if (!finite_nonneg(desc->nu, ne)) return fail_create(nullptr, "hc_create: nu must be finite and >= 0", HC_EINVAL);
  if (desc->sigma && !finite_nonneg(desc->sigma, ne))
    return fail_create(nullptr, "hc_create: sigma must be finite and >= 0", HC_EINVAL);

  hcop* h = new hcop();
  h->type = HC_HEX;
  h->p = p;
  h->nx = nx;
  h->ny = ny;
  h->nz = nz;
  h->ne = ne;
  h->dt = desc->dt;
  h->has_mass = desc->sigma != nullptr;
  const int64_t nxo = (int64_t)nx * p, nyo = (int64_t)ny * p, nzo = (int64_t)nz * p;
  h->off[0] = 0;
  h->off[1] = nxo * (nyo + 1) * (nzo + 1);
  h->off[2] = h->off[1] + (nxo + 1) * nyo * (nzo + 1);
  h->ndof = h->off[2] + (nxo + 1) * (nyo + 1) * nzo;
  const int64_t N = h->ndof;
  if (N >= ((int64_t)1 << 31))
    return fail_create(h, "hc_create: more than 2^31 - 1 dofs per problem is not supported", HC_ENOTSUP);

  // HBM budget: resident data + the largest solve work space (6 FP64 vectors)
  size_t need = (size_t)ne * 12 * (8 + 4) + (size_t)N * (1 + 8 * 3 + 4 * 2) + (size_t)N * 8 * 8;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess)
    return fail_create(h, "hc_create: no CUDA device available", HC_ECUDA);
  if (need > fr) return fail_create(h, "hc_create: problem exceeds free device memory", HC_ENOMEM);

  // ---- per-element affine factors (FP64) ----
  std::vector<double> vert;
  const double* V = desc->vertices;
  const int64_t nv = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
  if (!V) {
    vert.resize(nv * 3);
    for (int k = 0; k <= nz; ++k)
      for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
          const int64_t id = i + (int64_t)(nx + 1) * (j + (int64_t)(ny + 1) * k);
          vert[3 * id] = double(i) / nx;
          vert[3 * id + 1] = double(j) / ny;
          vert[3 * id + 2] = double(k) / nz;
        }
    V = vert.data();
  }
  std::vector<double> fac((size_t)12 * ne);
  bool full = false;
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex) {
        const int64_t e = ex + (int64_t)nx * (ey + (int64_t)ny * ez);
        auto P = [&](int a, int b, int c) {
          return V + 3 * ((ex + a) + (int64_t)(nx + 1) * ((ey + b) + (int64_t)(ny + 1) * (ez + c)));
        };
        const double *v0 = P(0, 0, 0), *vx = P(1, 0, 0), *vy = P(0, 1, 0), *vz = P(0, 0, 1);
        double J[9];
        for (int r = 0; r < 3; ++r) {
          J[3 * r] = vx[r] - v0[r];
          J[3 * r + 1] = vy[r] - v0[r];
          J[3 * r + 2] = vz[r] - v0[r];
        }
        // parallelepiped check on the four remaining corners
        double scale = 0.0;
        for (int q = 0; q < 9; ++q) scale = std::max(scale, std::fabs(J[q]));
        const int corners[4][3] = {{1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};
        for (auto& c : corners) {
          const double* vc = P(c[0], c[1], c[2]);
          for (int r = 0; r < 3; ++r) {
            const double pred = v0[r] + c[0] * J[3 * r] + c[1] * J[3 * r + 1] + c[2] * J[3 * r + 2];
            if (std::fabs(vc[r] - pred) > 1e-10 * std::max(scale, 1e-300))
              return fail_create(h, "hc_create: hex element is not a parallelepiped (non-affine map)", HC_EINVAL);
          }
        }
        const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                           J[2] * (J[3] * J[7] - J[4] * J[6]);
        if (!(det > 0.0) || !std::isfinite(det))
          return fail_create(h, "hc_create: hex element with non-positive Jacobian", HC_EINVAL);
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
        const double sg = desc->sigma ? desc->sigma[e] : 0.0;
        const double cu = desc->dt * desc->nu[e];
        const int pr[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
        for (int q = 0; q < 6; ++q) {
          const int r = pr[q][0], c = pr[q][1];
          double m = 0, k = 0;
          for (int s = 0; s < 3; ++s) {
            m += Ji[3 * r + s] * Ji[3 * c + s];
            k += J[3 * s + r] * J[3 * s + c];
          }
          fac[(size_t)q * ne + e] = sg * det * m;
          fac[(size_t)(6 + q) * ne + e] = cu / det * k;
          if (r != c && (m != 0.0 || k != 0.0)) full = true;
        }
      }
  h->full = full;
  std::vector<float> facf(fac.size());
  for (size_t i = 0; i < fac.size(); ++i) facf[i] = (float)fac[i];

  // ---- essential dofs ----
  h->ess_host.assign(N, 0);
  if (desc->ess_mask) {
    std::memcpy(h->ess_host.data(), desc->ess_mask, N);
    for (int64_t i = 0; i < N; ++i) h->ess_host[i] = h->ess_host[i] ? 1 : 0;
    h->explicit_mask = true;
  } else {
    const int bits = desc->ess_attr_bits & 0x3F;
    h->ess_bits = bits;
    for (int c = 0; c < 3; ++c) {
      const int64_t n0 = nxo + (c != 0), n1 = nyo + (c != 1), n2 = nzo + (c != 2);
      for (int64_t k = 0; k < n2; ++k)
        for (int64_t j = 0; j < n1; ++j)
          for (int64_t i = 0; i < n0; ++i) {
            bool e = false;
            if (c != 0) e |= (i == 0 && (bits & 1)) || (i == nxo && (bits & 2));
            if (c != 1) e |= (j == 0 && (bits & 4)) || (j == nyo && (bits & 8));
            if (c != 2) e |= (k == 0 && (bits & 16)) || (k == nzo && (bits & 32));
            h->ess_host[h->off[c] + i + n0 * (j + n1 * k)] = e;
          }
    }
  }

  // ---- upload ----
  if (!tables_ready()) return fail_create(h, "hc_create: constant table upload failed", HC_ECUDA);
  auto alloc = [&](void** p, size_t b) { return dmalloc(h, p, b) == cudaSuccess; };
  if (!alloc((void**)&h->fac, fac.size() * 8) || !alloc((void**)&h->facf, facf.size() * 4) ||
      !alloc((void**)&h->ess, N) || !alloc((void**)&h->diag, N * 8) || !alloc((void**)&h->dinv, N * 8) ||
      !alloc((void**)&h->dinvf, N * 4) || !alloc((void**)&h->sdinv, N * 8) || !alloc((void**)&h->sdinvf, N * 4) ||
      !alloc((void**)&h->xbuf, N * 8) || !alloc((void**)&h->ybuf, N * 8) || !alloc((void**)&h->nu, ne * 8))
    return fail_create(h, "hc_create: device allocation failed", HC_ENOMEM);
  for (int shape = 0; shape < (p <= 2 ? 2 : 1); ++shape) {
    std::vector<int> tab;
    hex_tile_table(p, shape, nx, ny, tab);
    int** dst = shape ? &h->tab1 : &h->tab;
    if (dmalloc(h, (void**)dst, tab.size() * sizeof(int)) != cudaSuccess)
      return fail_create(h, "hc_create: device allocation failed", HC_ENOMEM);
    cudaMemcpyAsync(*dst, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice, h->stream);
    // pageable sources: each copy is staged before the call returns
  }
  tune_lookup(h);  // a stored launch configuration for this problem, if any
  if (dmalloc(h, (void**)&h->verts, nv * 3 * sizeof(double)) != cudaSuccess)
    return fail_create(h, "hc_create: device allocation failed", HC_ENOMEM);
  cudaStream_t cs = h->stream;
  cudaMemcpyAsync(h->verts, V, nv * 3 * sizeof(double), cudaMemcpyHostToDevice, cs);
  cudaMemcpyAsync(h->fac, fac.data(), fac.size() * 8, cudaMemcpyHostToDevice, cs);
  cudaMemcpyAsync(h->facf, facf.data(), facf.size() * 4, cudaMemcpyHostToDevice, cs);
  cudaMemcpyAsync(h->ess, h->ess_host.data(), N, cudaMemcpyHostToDevice, cs);
  cudaMemcpyAsync(h->nu, desc->nu, ne * sizeof(double), cudaMemcpyHostToDevice, cs);
  cudaMemsetAsync(h->diag, 0, N * 8, cs);
  const HexDev d = h->hexdev();
  if (hex_diag(d, h->diag, cs) != cudaSuccess)
    return fail_create(h, "hc_create: diagonal kernel failed", HC_ECUDA);
  cudaError_t e = diag_finish(N, h->ess, h->diag, h->dinv, h->dinvf, h->sdinv, h->sdinvf, cs);
  if (e == cudaErrorInvalidValue)
    return fail_create(h, "hc_create: operator diagonal is not positive (nu = 0 and sigma = 0 somewhere?)",
                       HC_EINVAL);
  if (e != cudaSuccess) return fail_create(h, std::string("hc_create: ") + cudaGetErrorString(e), HC_ECUDA);
  if (ensure_scalars(h) != cudaSuccess) return fail_create(h, "hc_create: scalar allocation failed", HC_ENOMEM);
  if (cudaStreamSynchronize(cs) != cudaSuccess) return fail_create(h, "hc_create: setup failed", HC_ECUDA);
  *out = h;
  return HC_OK;
}

// ---- operator actions --------------------------------------------------------
static hc_status mult_impl(hcop* h, const double* x, double* y) {
  HC_CUDA_TRY(h, init_masked<double>(h->ndof, h->ess, x, y, h->stream));
  const OpJ<double> op{h, h->fac};
  HC_CUDA_TRY(h, op.apply(x, y, nullptr, nullptr, h->stream));
  return HC_OK;
}

hc_status hc_mult_device(hcop_t* h, const double* x, double* y) {
  if (!h || !x || !y) return HC_EINVAL;
  return mult_impl(h, x, y);
}

hc_status hc_mult_device_f32(hcop_t* h, const float* x, float* y) {
  if (!h || !x || !y) return HC_EINVAL;
  HC_CUDA_TRY(h, init_masked<float>(h->ndof, h->ess, x, y, h->stream));
  const OpJ<float> op{h, h->facf};
  HC_CUDA_TRY(h, op.apply(x, y, nullptr, nullptr, h->stream));
  return HC_OK;
}

hc_status hc_add_mult_device(hcop_t* h, const double* x, double* y) {
  if (!h || !x || !y) return HC_EINVAL;
  const OpJ<double> op{h, h->fac};
  HC_CUDA_TRY(h, op.apply(x, y, nullptr, nullptr, h->stream, false));
  return HC_OK;
}

hc_status hc_add_mult_device_f32(hcop_t* h, const float* x, float* y) {
  if (!h || !x || !y) return HC_EINVAL;
  const OpJ<float> op{h, h->facf};
  HC_CUDA_TRY(h, op.apply(x, y, nullptr, nullptr, h->stream, false));
  return HC_OK;
}

hc_status hc_apply_form_device(hcop_t* h, const double* x, double* y) {
  if (!h || !x || !y) return HC_EINVAL;
  if (h->type == HC_TET) {
    HC_CUDA_TRY(h, cudaMemsetAsync(y, 0, h->ndof * sizeof(double), h->stream));
    HC_CUDA_TRY(h, tet_apply_launch<double>(h, h->tetK64, x, y, 1, false, 1.0, nullptr, h->stream));
    return HC_OK;
  }
  HC_CUDA_TRY(h, cudaMemsetAsync(y, 0, h->ndof * sizeof(double), h->stream));
  HC_CUDA_TRY(h, hex_apply<double>(h->hexdev(), h->fac, x, y, h->has_mass ? 1.0 : 0.0, 1.0, false, nullptr,
                                   nullptr, h->stream, true));
  return HC_OK;
}

static hc_status h2d(hcop* h, double* dst, const double* src) {
  HC_CUDA_TRY(h, cudaMemcpyAsync(dst, src, h->ndof * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  return HC_OK;
}
static hc_status d2h_sync(hcop* h, double* dst, const double* src) {
  HC_CUDA_TRY(h, cudaMemcpyAsync(dst, src, h->ndof * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  HC_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
  return HC_OK;
}

hc_status hc_mult(hcop_t* h, const double* x, double* y) {
  if (!h || !x || !y) return HC_EINVAL;
  hc_status st = h2d(h, h->xbuf, x);
  if (st == HC_OK) st = mult_impl(h, h->xbuf, h->ybuf);
  if (st == HC_OK) st = d2h_sync(h, y, h->ybuf);
  return st;
}

hc_status hc_apply_form(hcop_t* h, const double* x, double* y) {
  if (!h || !x || !y) return HC_EINVAL;
  hc_status st = h2d(h, h->xbuf, x);
  if (st == HC_OK) st = hc_apply_form_device(h, h->xbuf, h->ybuf);
  if (st == HC_OK) st = d2h_sync(h, y, h->ybuf);
  return st;
}

hc_status hc_add_weak_curlcurl(hcop_t* h, const double* x, double* y, double scale) {
  if (!h || !x || !y || !std::isfinite(scale)) return HC_EINVAL;
  if (h->type != HC_HEX) {
    h->err = "hc_add_weak_curlcurl: structured hex grids only in this build";
    return HC_ENOTSUP;
  }
  hc_status st = h2d(h, h->xbuf, x);
  if (st == HC_OK) st = h2d(h, h->ybuf, y);
  if (st != HC_OK) return st;
  // C_nu = (dt C_nu) / dt
  HC_CUDA_TRY(h, hex_apply<double>(h->hexdev(), h->fac, h->xbuf, h->ybuf, 0.0, scale / h->dt, false, nullptr,
                                   nullptr, h->stream, false));
  return d2h_sync(h, y, h->ybuf);
}

hc_status hc_add_weak_curlcurl_device(hcop_t* h, const double* x, double* y, double scale) {
  if (!h || !x || !y || !std::isfinite(scale)) return HC_EINVAL;
  if (h->type != HC_HEX) {
    h->err = "hc_add_weak_curlcurl: structured hex grids only in this build";
    return HC_ENOTSUP;
  }
  HC_CUDA_TRY(h, hex_apply<double>(h->hexdev(), h->fac, x, y, 0.0, scale / h->dt, false, nullptr, nullptr,
                                   h->stream, false));
  return HC_OK;
}

hc_status hc_diag(hcop_t* h, double* d) {
  if (!h || !d) return HC_EINVAL;
  return d2h_sync(h, d, h->diag);
}

// ---- multi right-hand-side apply ------------------------------------------------
hc_status hc_mult_multi_device(hcop_t* h, int precision, int nrhs, const void* X, void* Y) {
  if (!h || !X || !Y) return HC_EINVAL;
  if (nrhs != 1 && nrhs != 2 && nrhs != 4 && nrhs != 8 && nrhs != 16 && nrhs != 32) {
    h->err = "hc_mult_multi_device: nrhs must be 1, 2, 4, 8, 16 or 32";
    return HC_EINVAL;
  }
  if (precision != HC_FP64 && precision != HC_FP32 && precision != HC_BF16) {
    h->err = "hc_mult_multi_device: precision must be HC_FP64, HC_FP32 or HC_BF16";
    return HC_EINVAL;
  }
  if (precision == HC_BF16 && h->type != HC_TET) {
    h->err = "hc_mult_multi_device: HC_BF16 element matrices exist for tet meshes only";
    return HC_ENOTSUP;
  }
  if (h->type != HC_TET) {
    if (nrhs != 1) {
      h->err = "hc_mult_multi_device: hex grids take one right-hand side per call in this build";
      return HC_ENOTSUP;
    }
    return precision == HC_FP64 ? hc_mult_device(h, (const double*)X, (double*)Y)
                                : hc_mult_device_f32(h, (const float*)X, (float*)Y);
  }
  if (precision == HC_FP64) {
    HC_CUDA_TRY(h, init_masked_multi<double>(h->ndof, nrhs, h->ess, (const double*)X, (double*)Y, h->stream));
    HC_CUDA_TRY(h, tet_apply_launch<double>(h, h->tetK64, (const double*)X, (double*)Y, nrhs, true, 1.0, nullptr,
                                            h->stream));
  } else if (precision == HC_FP32) {
    HC_CUDA_TRY(h, init_masked_multi<float>(h->ndof, nrhs, h->ess, (const float*)X, (float*)Y, h->stream));
    HC_CUDA_TRY(h, tet_apply_launch<float>(h, h->tetK32, (const float*)X, (float*)Y, nrhs, true, 1.0, nullptr,
                                           h->stream));
  } else {
    HC_CUDA_TRY(h, tet_ensure_bf16(h));
    HC_CUDA_TRY(h, init_masked_multi<float>(h->ndof, nrhs, h->ess, (const float*)X, (float*)Y, h->stream));
    HC_CUDA_TRY(h, tet_apply_launch_bf16(h, (const float*)X, (float*)Y, nrhs, true, h->stream));
  }
  return HC_OK;
}

int32_t hc_elem_type(const hcop_t* h) { return h ? h->type : -1; }

hc_status hc_tet_element_matrix(hcop_t* h, int64_t e, double* out) {
  if (!h || !out || h->type != HC_TET || e < 0 || e >= h->ne) return HC_EINVAL;
  const int L = h->p == 1 ? 6 : 20;
  HC_CUDA_TRY(h, cudaMemcpy(out, h->tetK64 + e * L * L, L * L * sizeof(double), cudaMemcpyDeviceToHost));
  return HC_OK;
}

// ---- curl, load vector ------------------------------------------------------------
int64_t hc_num_rt_dofs(const hcop_t* h) {
  if (!h || h->type != HC_HEX) return -1;
  int64_t o1, o2, n;
  hex_rt_layout(h->hexdev(), &o1, &o2, &n);
  return n;
}

int64_t hc_hex_rt_dof_index(const hcop_t* h, int c, int64_t i, int64_t j, int64_t k) {
  if (!h || c < 0 || c > 2) return -1;
  const int64_t mx = (int64_t)h->nx * h->p, my = (int64_t)h->ny * h->p, mz = (int64_t)h->nz * h->p;
  const int64_t n0 = mx + (c == 0), n1 = my + (c == 1), n2 = mz + (c == 2);
  if (i < 0 || j < 0 || k < 0 || i >= n0 || j >= n1 || k >= n2) return -1;
  int64_t o1, o2, n;
  hex_rt_layout(h->hexdev(), &o1, &o2, &n);
  const int64_t off = c == 0 ? 0 : (c == 1 ? o1 : o2);
  return off + i + n0 * (j + n1 * k);
}

hc_status hc_curl_device(hcop_t* h, const double* A, double* B) {
  if (!h || !A || !B) return HC_EINVAL;
  if (h->type != HC_HEX) {
    h->err = "hc_curl: structured hex grids only in this build";
    return HC_ENOTSUP;
  }
  HC_CUDA_TRY(h, hex_curl(h->hexdev(), A, B, h->stream));
  return HC_OK;
}

hc_status hc_curl(hcop_t* h, const double* A, double* B) {
  if (!h || !A || !B) return HC_EINVAL;
  if (h->type != HC_HEX) {
    h->err = "hc_curl: structured hex grids only in this build";
    return HC_ENOTSUP;
  }
  const int64_t nrt = hc_num_rt_dofs(h);
  double* dB = nullptr;
  HC_CUDA_TRY(h, cudaMallocAsync((void**)&dB, nrt * sizeof(double), h->stream));
  hc_status st = h2d(h, h->xbuf, A);
  if (st == HC_OK) st = hc_curl_device(h, h->xbuf, dB);
  if (st == HC_OK) {
    cudaMemcpyAsync(B, dB, nrt * sizeof(double), cudaMemcpyDeviceToHost, h->stream);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) st = HC_ECUDA;
  }
  cudaFreeAsync(dB, h->stream);
  return st;
}

hc_status hc_load_coil_device(hcop_t* h, const hc_coil* coil, int q, double* b) {
  if (!h || !coil || !b || q < 1 || q > 8) {
    if (h) h->err = "hc_load_coil: need a coil and 1 <= q <= 8";
    return HC_EINVAL;
  }
  if (h->type == HC_TET) {
    std::vector<double> xq(q), wq(q);
    gl01(q, xq.data(), wq.data());
    const double cv[7] = {coil->I0, coil->xc, coil->yc, coil->r0, coil->r1, coil->z0, coil->z1};
    HC_CUDA_TRY(h, tet_load_coil(h, cv, q, xq.data(), wq.data(), b, h->stream));
    return HC_OK;
  }
  std::vector<double> xq(q), wq(q), bc(q * (h->p + 1)), bo(q * h->p);
  gl01(q, xq.data(), wq.data());
  double xc[kMaxP + 1], xo[kMaxP], wo[kMaxP], d1[kMaxP + 1];
  gll01(h->p + 1, xc);
  gl01(h->p, xo, wo);
  for (int k = 0; k < q; ++k) {
    lagrange(xc, h->p + 1, xq[k], &bc[k * (h->p + 1)], d1);
    lagrange(xo, h->p, xq[k], &bo[k * h->p], d1);
  }
  const double cv[7] = {coil->I0, coil->xc, coil->yc, coil->r0, coil->r1, coil->z0, coil->z1};
  HC_CUDA_TRY(h, hex_load_coil(h->hexdev(), h->verts, cv, q, xq.data(), wq.data(), bc.data(), bo.data(), b,
                               h->stream));
  return HC_OK;
}

// q-point Gauss-Legendre rule on [0,1] and the hex's 1-D bases at its points
struct HexRule {
  std::vector<double> xq, wq, bc, bo;
};
static HexRule hex_rule(const hcop* h, int q) {
  HexRule r;
  r.xq.resize(q);
  r.wq.resize(q);
  r.bc.resize(q * (h->p + 1));
  r.bo.resize(q * h->p);
  gl01(q, r.xq.data(), r.wq.data());
  if (h->type != HC_HEX) return r;
  double xc[kMaxP + 1], xo[kMaxP], wo[kMaxP], d1[kMaxP + 1];
  gll01(h->p + 1, xc);
  gl01(h->p, xo, wo);
  for (int k = 0; k < q; ++k) {
    lagrange(xc, h->p + 1, r.xq[k], &r.bc[k * (h->p + 1)], d1);
    lagrange(xo, h->p, r.xq[k], &r.bo[k * h->p], d1);
  }
  return r;
}

hc_status hc_quad_points_device(hcop_t* h, int q, double* xyz) {
  if (!h || !xyz) return HC_EINVAL;
  if (q < 1 || q > 8) {
    h->err = "hc_quad_points_device: 1 <= q <= 8";
    return HC_EINVAL;
  }
  const HexRule r = hex_rule(h, q);
  if (h->type == HC_TET) {
    HC_CUDA_TRY(h, tet_quad_points(h, q, r.xq.data(), xyz, h->stream));
  } else {
    HC_CUDA_TRY(h, hex_quad_points(h->hexdev(), h->verts, q, r.xq.data(), r.wq.data(), r.bc.data(), r.bo.data(), xyz,
                                   h->stream));
  }
  return HC_OK;
}

hc_status hc_load_field_device(hcop_t* h, int mode, int q, const double* J, double* b) {
  if (!h || !J || !b) return HC_EINVAL;
  if ((mode != HC_FIELD_ELEM && mode != HC_FIELD_QUAD) || q < 1 || q > 8) {
    h->err = "hc_load_field_device: mode must be HC_FIELD_ELEM or HC_FIELD_QUAD and 1 <= q <= 8";
    return HC_EINVAL;
  }
  const HexRule r = hex_rule(h, q);
  const int per_point = mode == HC_FIELD_QUAD ? 1 : 0;
  if (h->type == HC_TET) {
    HC_CUDA_TRY(h, tet_load_field(h, per_point, J, q, r.xq.data(), r.wq.data(), b, h->stream));
  } else {
    HC_CUDA_TRY(h, hex_load_field(h->hexdev(), h->verts, per_point, J, q, r.xq.data(), r.wq.data(), r.bc.data(),
                                  r.bo.data(), b, h->stream));
  }
  return HC_OK;
}

hc_status hc_curl_load_device(hcop_t* h, const double* A, double* b) {
  if (!h || !A || !b) return HC_EINVAL;
  if (h->type == HC_TET) {
    // curl A (degree p - 1) . w_i (degree p) on affine tets: 4 points per
    // direction of the collapsed rule are exact
    const HexRule r = hex_rule(h, 4);
    HC_CUDA_TRY(h, tet_curl_load(h, A, 4, r.xq.data(), r.wq.data(), b, h->stream));
  } else {
    HC_CUDA_TRY(h, hex_curl_load(h->hexdev(), h->nu, A, b, h->stream));
  }
  return HC_OK;
}

hc_status hc_tet_curl_points_device(hcop_t* h, const double* A, int npts, const double* xi, double* B) {
  if (!h || !A || !xi || !B) return HC_EINVAL;
  if (h->type != HC_TET) {
    h->err = "hc_tet_curl_points_device: tet meshes only (hex grids: hc_curl_device)";
    return HC_ENOTSUP;
  }
  if (npts < 1 || npts > 16) {
    h->err = "hc_tet_curl_points_device: 1 <= npts <= 16";
    return HC_EINVAL;
  }
  HC_CUDA_TRY(h, tet_curl_points(h, A, npts, xi, B, h->stream));
  return HC_OK;
}

hc_status hc_tet_gradient_device(hcop_t* h, const double* u, double* y) {
  if (!h || !u || !y) return HC_EINVAL;
  if (h->type != HC_TET) {
    h->err = "hc_tet_gradient_device: tet meshes only";
    return HC_ENOTSUP;
  }
  HC_CUDA_TRY(h, tet_gradient(h, u, y, h->stream));
  return HC_OK;
}

hc_status hc_load_coil(hcop_t* h, const hc_coil* coil, int q, double* b) {
  if (!h || !b) return HC_EINVAL;
  hc_status st = hc_load_coil_device(h, coil, q, h->ybuf);
  if (st != HC_OK) return st;
  return d2h_sync(h, b, h->ybuf);
}

// ---- solves ---------------------------------------------------------------------
static hc_status check_params(hcop* h, const hc_solve_params* p) {
  if (!p) {
    h->err = "null solve parameters";
    return HC_EINVAL;
  }
  if (p->precision != HC_FP64 && p->precision != HC_MIXED && p->precision != HC_MIXED_RR) {
    h->err = "precision must be HC_FP64, HC_MIXED or HC_MIXED_RR";
    return HC_EINVAL;
  }
  if (p->precond < HC_PRECOND_NONE || p->precond > HC_PRECOND_AUX_MULT) {
    h->err = "unknown preconditioner";
    return HC_EINVAL;
  }
  if (p->precond == HC_PRECOND_CHEBYSHEV && p->cheb_degree < 1) {
    h->err = "cheb_degree must be >= 1";
    return HC_EINVAL;
  }
  if (p->precond == HC_PRECOND_AUX_MULT && h->type != HC_HEX) {
    h->err = "HC_PRECOND_AUX_MULT is built for hex handles";
    return HC_ENOTSUP;
  }
  if (!(p->rtol >= 0.0) || !(p->atol >= 0.0) || p->maxit < 1) {
    h->err = "rtol, atol must be >= 0 and maxit >= 1";
    return HC_EINVAL;
  }
  return HC_OK;
}

hc_status hc_precond_apply_device(hcop_t* h, int32_t precond, const double* r, double* z) {
  if (!h || !r || !z) return HC_EINVAL;
  if (precond != HC_PRECOND_JACOBI && precond != HC_PRECOND_AUX) {
    h->err = "hc_precond_apply_device: precond must be HC_PRECOND_JACOBI or HC_PRECOND_AUX";
    return HC_EINVAL;
  }
  if (precond == HC_PRECOND_AUX && h->type != HC_HEX) {
    h->err = "hc_precond_apply_device: HC_PRECOND_AUX is built for hex handles here";
    return HC_ENOTSUP;
  }
  if (precond == HC_PRECOND_AUX) {
    const hc_status st = auxmg_setup(h);
    if (st != HC_OK) return st;
  }
  HC_CUDA_TRY(h, jacobi_apply(h->ndof, h->dinv, r, z, h->stream));
  if (precond == HC_PRECOND_AUX) {
    const float coef[4] = {1.0f, 0.0f, 0.0f, 0.0f};
    const cudaError_t e = auxmg_apply<double, 1>(h, r, nullptr, z, nullptr, coef, nullptr, h->stream);
    HC_CUDA_TRY(h, e);
  }
  return HC_OK;
}

hc_status hc_lanczos_lmax(hcop_t* h, int steps, double* lmax) {
  if (!h || !lmax) return HC_EINVAL;
  return lanczos_device<double>(h, steps, lmax);
}

hc_status hc_solve_device(hcop_t* h, const hc_solve_params* prm, const double* b, double* x,
                          hc_solve_info* info) {
  if (!h || !b || !x) return HC_EINVAL;
  hc_status st = check_params(h, prm);
  if (st != HC_OK) return st;
  hc_solve_info loc{};
  if (!info) info = &loc;
  std::memset(info, 0, sizeof(*info));
  if (prm->precond == HC_PRECOND_AUX && h->type == HC_TET) {  // one-column block PCG with the tet AMG
    if ((reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(x)) % 16 != 0) {
      h->err = "hc_solve_device: b and x must be 16-byte aligned for tet AUX solves";
      return HC_EINVAL;
    }
    return multi_solve_device(h, prm, 1, b, x, info);
  }
  if (prm->precond == HC_PRECOND_AUX || prm->precond == HC_PRECOND_AUX_MULT) {
    st = auxmg_setup(h);
    if (st != HC_OK) return st;
  }
  if (prm->precision == HC_MIXED) return mixed_device(h, prm, b, x, info);
  if (prm->precision == HC_MIXED_RR) return mixed_rr_device(h, prm, b, x, info);
  SolveCfg cfg;
  cfg.precond = prm->precond;
  cfg.cheb_degree = prm->cheb_degree > 0 ? prm->cheb_degree : 2;
  cfg.cheb_ratio = prm->cheb_ratio > 0 ? prm->cheb_ratio : 30.0;
  cfg.rtol = prm->rtol;
  cfg.atol = prm->atol;
  cfg.maxit = prm->maxit;
  cfg.lmax = prm->cheb_lmax;
  if ((cfg.precond == HC_PRECOND_CHEBYSHEV || cfg.precond == HC_PRECOND_AUX_MULT) && cfg.lmax <= 0) {
    if (h->lmax64 <= 0) {
      double lm = 0;
      st = lanczos_device<double>(h, 20, &lm);
      if (st != HC_OK) return st;
      h->lmax64 = 1.1 * lm;
    }
    cfg.lmax = h->lmax64;
  }
  int it = 0, ap = 0;
  st = pcg_device<double>(h, cfg, b, x, &it, &ap, nullptr);
  info->status = st;
  info->iterations = it;
  info->outer_iterations = 1;
  info->applies = ap;
  info->lmax = cfg.lmax;
  // recursive residual norm of the last batch read
  const KrylovScalars* hs = h->hscal;
  info->rel_residual = hs->bb > 0 ? std::sqrt(hs->rr / hs->bb) : std::sqrt(hs->rr);
  return st;
}

hc_status hc_solve(hcop_t* h, const hc_solve_params* prm, const double* b, double* x, hc_solve_info* info) {
  if (!h || !b || !x) return HC_EINVAL;
  hc_status st = h2d(h, h->ybuf, b);
  if (st == HC_OK) st = h2d(h, h->xbuf, x);
  if (st != HC_OK) return st;
  hc_status sst = hc_solve_device(h, prm, h->ybuf, h->xbuf, info);
  if (sst == HC_EINVAL || sst == HC_ECUDA || sst == HC_ENOMEM) return sst;
  st = d2h_sync(h, x, h->xbuf);
  return st != HC_OK ? st : sst;
}

}  // extern "C"

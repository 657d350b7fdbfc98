// hcurl_oracle.cpp -- FP64 CPU oracle (test infrastructure only; see hcurl_oracle.h).
//
// Everything here is plain, unoptimised-for-clarity FP64 C++: full-quadrature
// element matrices, CSR assembly, CSR SpMV, textbook PCG.  It shares no code
// with the CUDA product path, which uses sum factorisation and never forms a
// matrix; agreement between the two is the parity evidence.
#include "hcurl_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

namespace {

using i64 = int64_t;
constexpr double kPi = 3.14159265358979323846;

// ---------------------------------------------------------------------------
// threading helper
// ---------------------------------------------------------------------------
void parallel_for(i64 n, int nthreads, const std::function<void(i64, i64)>& fn) {
  if (nthreads <= 1 || n < 4096) {
    fn(0, n);
    return;
  }
  std::vector<std::thread> th;
  i64 chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; ++t) {
    i64 b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    th.emplace_back(fn, b, e);
  }
  for (auto& x : th) x.join();
}

// ---------------------------------------------------------------------------
// 1-D rules on [0,1]
// ---------------------------------------------------------------------------
// Gauss-Legendre: Newton on the three-term Legendre recurrence.
void gauss_legendre01(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = std::cos(kPi * (i + 0.75) / (n + 0.5));
    double p0 = 0, p1 = 0, dp = 0;
    for (int it = 0; it < 100; ++it) {
      p0 = 1.0;
      p1 = 0.0;
      for (int k = 1; k <= n; ++k) {
        double p2 = p1;
        p1 = p0;
        p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
      }
      dp = n * (z * p0 - p1) / (z * z - 1.0);
      double dz = p0 / dp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    p0 = 1.0;
    p1 = 0.0;
    for (int k = 1; k <= n; ++k) {
      double p2 = p1;
      p1 = p0;
      p0 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p2) / k;
    }
    dp = n * (z * p0 - p1) / (z * z - 1.0);
    x[n - 1 - i] = 0.5 * (1.0 + z);
    w[n - 1 - i] = 1.0 / ((1.0 - z * z) * dp * dp);
  }
}

// Gauss-Lobatto nodes: Newton iteration x <- x - (x P_N - P_{N-1}) / ((N+1) P_N)
// started from the Chebyshev-Gauss-Lobatto points.
void gauss_lobatto01(int n, double* x) {
  const int N = n - 1;
  std::vector<double> z(n);
  for (int i = 0; i < n; ++i) z[i] = std::cos(kPi * i / N);
  for (int it = 0; it < 200; ++it) {
    double md = 0;
    for (int i = 0; i < n; ++i) {
      double pm = 1.0, pc = z[i];
      for (int k = 2; k <= N; ++k) {
        double pn = ((2.0 * k - 1.0) * z[i] * pc - (k - 1.0) * pm) / k;
        pm = pc;
        pc = pn;
      }
      double d = (z[i] * pc - pm) / (n * pc);
      z[i] -= d;
      md = std::max(md, std::fabs(d));
    }
    if (md < 1e-16) break;
  }
  for (int i = 0; i < n; ++i) x[N - i] = 0.5 * (1.0 + z[i]);
  x[0] = 0.0;
  x[N] = 1.0;
}

struct Lagrange {
  std::vector<double> nodes;
  void eval(double t, double* v, double* d) const {
    const int m = (int)nodes.size();
    for (int j = 0; j < m; ++j) {
      double pv = 1.0;
      for (int k = 0; k < m; ++k)
        if (k != j) pv *= (t - nodes[k]) / (nodes[j] - nodes[k]);
      v[j] = pv;
      double s = 0.0;
      for (int l = 0; l < m; ++l) {
        if (l == j) continue;
        double pr = 1.0 / (nodes[j] - nodes[l]);
        for (int k = 0; k < m; ++k)
          if (k != j && k != l) pr *= (t - nodes[k]) / (nodes[j] - nodes[k]);
        s += pr;
      }
      d[j] = s;
    }
  }
};

// 3x3 helpers (row-major)
double det3(const double* J) {
  return J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
         J[2] * (J[3] * J[7] - J[4] * J[6]);
}
void inv3(const double* J, double* Ji) {
  double d = det3(J);
  Ji[0] = (J[4] * J[8] - J[5] * J[7]) / d;
  Ji[1] = (J[2] * J[7] - J[1] * J[8]) / d;
  Ji[2] = (J[1] * J[5] - J[2] * J[4]) / d;
  Ji[3] = (J[5] * J[6] - J[3] * J[8]) / d;
  Ji[4] = (J[0] * J[8] - J[2] * J[6]) / d;
  Ji[5] = (J[2] * J[3] - J[0] * J[5]) / d;
  Ji[6] = (J[3] * J[7] - J[4] * J[6]) / d;
  Ji[7] = (J[1] * J[6] - J[0] * J[7]) / d;
  Ji[8] = (J[0] * J[4] - J[1] * J[3]) / d;
}
void cross3(const double* a, const double* b, double* c) {
  c[0] = a[1] * b[2] - a[2] * b[1];
  c[1] = a[2] * b[0] - a[0] * b[2];
  c[2] = a[0] * b[1] - a[1] * b[0];
}

// Manufactured problem of test/integration/test_aform_source.cpp:26-49.
double mms_nu(const double* x, double s) {
  return 1.0 + s * std::cos(kPi * x[0]) * std::cos(kPi * x[1]);
}
void mms_source(const double* x, double t, double s, double* f) {
  const double sx = std::sin(kPi * x[0]), cx = std::cos(kPi * x[0]);
  const double sy = std::sin(kPi * x[1]), cy = std::cos(kPi * x[1]);
  const double sz = std::sin(kPi * x[2]), cz = std::cos(kPi * x[2]);
  f[0] = t * kPi * kPi * sy * sz * (3 * s * cx * cy + 2) + sy * sz;
  f[1] = -s * kPi * kPi * t * sx * cy * cy * sz;
  f[2] = -0.5 * s * kPi * kPi * t * sx * std::sin(2 * kPi * x[1]) * cz;
}
void mms_exact(const double* x, double t, double* A) {
  A[0] = std::sin(kPi * x[1]) * std::sin(kPi * x[2]) * t;
  A[1] = 0;
  A[2] = 0;
}

// ---------------------------------------------------------------------------
// Problem base: element dofs, coefficients, CSR, essential mask.
// ---------------------------------------------------------------------------
struct Prob {
  i64 ndof = 0, ne = 0;
  int L = 0;
  std::vector<i64> edofs;
  std::vector<double> alpha, beta;  // per element constants
  bool mms = false;
  double mms_dt = 0, mms_s = 0, mms_sigma = 0;
  std::vector<i64> rp, ci;
  std::vector<double> va;
  std::vector<uint8_t> ess;
  std::vector<double> dmask;  // diagonal of the eliminated operator
  std::vector<double> ebuf;   // cached element matrices (tets / mms)
  // eliminated operator as hypre holds it: ess rows/cols dropped, unit
  // diagonal on ess rows, 32-bit column indices
  std::vector<int64_t> erp;
  std::vector<int32_t> eci;
  std::vector<double> eva;
  int q_curl = 0, q_mass = 0;  // points per direction for element matrices (0 = exact default)

  virtual ~Prob() = default;
  // reference quadrature (points in reference coordinates, weights sum to ref volume)
  virtual void ref_quad(int q, std::vector<double>& xi, std::vector<double>& w) const = 0;
  // physical point, |det J|, physical basis values/curls (L x 3 each) at reference xi
  virtual void eval_phys(i64 e, const double* xi, double* x, double* adet, double* val,
                         double* curl) const = 0;
  virtual int elem_quad_order() const = 0;

  // Element matrix by direct quadrature (general; used by tets and MMS).
  void elem_matrix_quad(i64 e, double* K) const {
    std::fill(K, K + (size_t)L * L, 0.0);
    if (q_curl == q_mass) {
      elem_matrix_term(e, q_curl ? q_curl : elem_quad_order(), true, true, K);
    } else {
      elem_matrix_term(e, q_curl ? q_curl : elem_quad_order(), true, false, K);
      elem_matrix_term(e, q_mass ? q_mass : elem_quad_order(), false, true, K);
    }
  }
  void elem_matrix_term(i64 e, int qo, bool with_curl, bool with_mass, double* K) const {
    std::vector<double> xi, w;
    ref_quad(qo, xi, w);
    std::vector<double> val(L * 3), cu(L * 3);
    for (size_t q = 0; q < w.size(); ++q) {
      double x[3], ad;
      eval_phys(e, &xi[3 * q], x, &ad, val.data(), cu.data());
      double a, b;
      if (mms) {
        a = mms_dt * mms_nu(x, mms_s);
        b = mms_sigma;
      } else {
        a = alpha.empty() ? 0.0 : alpha[e];
        b = beta.empty() ? 0.0 : beta[e];
      }
      if (!with_curl) a = 0.0;
      if (!with_mass) b = 0.0;
      const double wq = w[q] * ad;
      for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j) {
          double m = val[3 * i] * val[3 * j] + val[3 * i + 1] * val[3 * j + 1] +
                     val[3 * i + 2] * val[3 * j + 2];
          double c = cu[3 * i] * cu[3 * j] + cu[3 * i + 1] * cu[3 * j + 1] +
                     cu[3 * i + 2] * cu[3 * j + 2];
          K[i * L + j] += wq * (b * m + a * c);
        }
    }
  }
  virtual void elem_matrix(i64 e, double* K) const { elem_matrix_quad(e, K); }
  // one row of the element matrix; default reads the cache
  virtual void elem_row(i64 e, int li, double* row) const {
    std::memcpy(row, &ebuf[((size_t)e * L + li) * L], sizeof(double) * L);
  }
  virtual bool needs_cache() const { return true; }

  int assemble(int nthreads) {
    if (needs_cache()) {
      ebuf.assign((size_t)ne * L * L, 0.0);
      parallel_for(ne, nthreads, [&](i64 b, i64 e) {
        for (i64 k = b; k < e; ++k) elem_matrix(k, &ebuf[(size_t)k * L * L]);
      });
    }
    // dof -> (element, local) adjacency
    std::vector<i64> cnt(ndof + 1, 0);
    for (i64 k = 0; k < ne * L; ++k) cnt[edofs[k] + 1]++;
    for (i64 i = 0; i < ndof; ++i) cnt[i + 1] += cnt[i];
    std::vector<i64> adj(ne * L), fill(cnt.begin(), cnt.end() - 1);
    for (i64 k = 0; k < ne * L; ++k) adj[fill[edofs[k]]++] = k;
    // row lengths
    std::vector<i64> len(ndof, 0);
    parallel_for(ndof, nthreads, [&](i64 b, i64 e) {
      std::vector<i64> tmp;
      for (i64 i = b; i < e; ++i) {
        tmp.clear();
        for (i64 a = cnt[i]; a < cnt[i + 1]; ++a) {
          i64 el = adj[a] / L;
          for (int j = 0; j < L; ++j) tmp.push_back(edofs[el * L + j]);
        }
        std::sort(tmp.begin(), tmp.end());
        len[i] = std::unique(tmp.begin(), tmp.end()) - tmp.begin();
      }
    });
    rp.assign(ndof + 1, 0);
    for (i64 i = 0; i < ndof; ++i) rp[i + 1] = rp[i] + len[i];
    ci.assign(rp[ndof], 0);
    va.assign(rp[ndof], 0.0);
    parallel_for(ndof, nthreads, [&](i64 b, i64 e) {
      std::vector<i64> tmp;
      std::vector<double> row(L);
      for (i64 i = b; i < e; ++i) {
        tmp.clear();
        for (i64 a = cnt[i]; a < cnt[i + 1]; ++a) {
          i64 el = adj[a] / L;
          for (int j = 0; j < L; ++j) tmp.push_back(edofs[el * L + j]);
        }
        std::sort(tmp.begin(), tmp.end());
        tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
        std::copy(tmp.begin(), tmp.end(), ci.begin() + rp[i]);
        for (i64 a = cnt[i]; a < cnt[i + 1]; ++a) {
          i64 el = adj[a] / L;
          int li = (int)(adj[a] % L);
          elem_row(el, li, row.data());
          for (int j = 0; j < L; ++j) {
            i64 c = edofs[el * L + j];
            i64 pos = std::lower_bound(ci.begin() + rp[i], ci.begin() + rp[i + 1], c) - ci.begin();
            va[pos] += row[j];
          }
        }
      }
    });
    ebuf.clear();
    ebuf.shrink_to_fit();
    set_ess_default();
    return 0;
  }

  void set_ess_default() {
    if ((i64)ess.size() != ndof) ess.assign(ndof, 0);
    dmask.assign(ndof, 1.0);
    for (i64 i = 0; i < ndof; ++i) {
      if (ess[i]) continue;
      for (i64 k = rp[i]; k < rp[i + 1]; ++k)
        if (ci[k] == i) dmask[i] = va[k];
    }
  }

  void spmv(const double* x, double* y, int nthreads) const {
    parallel_for(ndof, nthreads, [&](i64 b, i64 e) {
      for (i64 i = b; i < e; ++i) {
        double s = 0.0;
        for (i64 k = rp[i]; k < rp[i + 1]; ++k) s += va[k] * x[ci[k]];
        y[i] = s;
      }
    });
  }
  void build_eliminated() {
    erp.assign(ndof + 1, 0);
    eci.clear();
    eva.clear();
    for (i64 i = 0; i < ndof; ++i) {
      if (ess[i]) {
        eci.push_back((int32_t)i);
        eva.push_back(1.0);
      } else {
        for (i64 k = rp[i]; k < rp[i + 1]; ++k)
          if (!ess[ci[k]]) {
            eci.push_back((int32_t)ci[k]);
            eva.push_back(va[k]);
          }
      }
      erp[i + 1] = (i64)eci.size();
    }
  }
  void spmv_eliminated(const double* x, double* y, int nthreads) const {
    parallel_for(ndof, nthreads, [&](i64 b, i64 e) {
      for (i64 i = b; i < e; ++i) {
        double s = 0.0;
        for (i64 k = erp[i]; k < erp[i + 1]; ++k) s += eva[k] * x[eci[k]];
        y[i] = s;
      }
    });
  }
  // J x = P K P x + (I - P) x  (MFEM FormLinearSystem with DIAG_ONE)
  void apply_masked(const double* x, double* y, int nthreads) const {
    parallel_for(ndof, nthreads, [&](i64 b, i64 e) {
      for (i64 i = b; i < e; ++i) {
        if (ess[i]) {
          y[i] = x[i];
          continue;
        }
        double s = 0.0;
        for (i64 k = rp[i]; k < rp[i + 1]; ++k)
          if (!ess[ci[k]]) s += va[k] * x[ci[k]];
        y[i] = s;
      }
    });
  }
};

// ---------------------------------------------------------------------------
// Structured hex grid, Nedelec order p.
//   local dof order:  comp 0 (x): a + p (b + (p+1) c)       a open,   b,c closed
//                     comp 1 (y): a + (p+1)(b + p c)         b open,   a,c closed
//                     comp 2 (z): a + (p+1)(b + (p+1) c)     c open,   a,b closed
//   global:  comp 0 at (ex p + a) + (nx p)((ey p + b) + (ny p + 1)(ez p + c)), etc.
// ---------------------------------------------------------------------------
struct HexProb : Prob {
  int nx, ny, nz, p;
  std::vector<double> verts;
  std::vector<double> Jm, Ji, dets;  // per element affine map
  Lagrange cl, op;
  std::vector<double> RM, RC;  // reference matrices [9][L][L]
  i64 off[3];

  HexProb(int nx_, int ny_, int nz_, int p_, const double* v) : nx(nx_), ny(ny_), nz(nz_), p(p_) {
    const i64 nv = (i64)(nx + 1) * (ny + 1) * (nz + 1);
    verts.resize(nv * 3);
    for (int k = 0; k <= nz; ++k)
      for (int j = 0; j <= ny; ++j)
        for (int i = 0; i <= nx; ++i) {
          i64 id = i + (i64)(nx + 1) * (j + (i64)(ny + 1) * k);
          if (v) {
            for (int d = 0; d < 3; ++d) verts[3 * id + d] = v[3 * id + d];
          } else {
            verts[3 * id] = double(i) / nx;
            verts[3 * id + 1] = double(j) / ny;
            verts[3 * id + 2] = double(k) / nz;
          }
        }
    L = 3 * p * (p + 1) * (p + 1);
    ne = (i64)nx * ny * nz;
    const i64 nxo = (i64)nx * p, nyo = (i64)ny * p, nzo = (i64)nz * p;
    off[0] = 0;
    off[1] = nxo * (nyo + 1) * (nzo + 1);
    off[2] = off[1] + (nxo + 1) * nyo * (nzo + 1);
    ndof = off[2] + (nxo + 1) * (nyo + 1) * nzo;
    cl.nodes.resize(p + 1);
    gauss_lobatto01(p + 1, cl.nodes.data());
    op.nodes.resize(p);
    std::vector<double> w(p);
    gauss_legendre01(p, op.nodes.data(), w.data());
    // element dofs
    edofs.resize(ne * L);
    const int pp = p + 1;
    for (int ez = 0; ez < nz; ++ez)
      for (int ey = 0; ey < ny; ++ey)
        for (int ex = 0; ex < nx; ++ex) {
          i64 e = ex + (i64)nx * (ey + (i64)ny * ez);
          i64* d = &edofs[e * L];
          int l = 0;
          for (int c = 0; c < pp; ++c)
            for (int b = 0; b < pp; ++b)
              for (int a = 0; a < p; ++a)
                d[l++] = off[0] + (ex * p + a) + nxo * ((ey * p + b) + (nyo + 1) * (i64)(ez * p + c));
          for (int c = 0; c < pp; ++c)
            for (int b = 0; b < p; ++b)
              for (int a = 0; a < pp; ++a)
                d[l++] = off[1] + (ex * p + a) + (nxo + 1) * ((ey * p + b) + nyo * (i64)(ez * p + c));
          for (int c = 0; c < p; ++c)
            for (int b = 0; b < pp; ++b)
              for (int a = 0; a < pp; ++a)
                d[l++] =
                    off[2] + (ex * p + a) + (nxo + 1) * ((ey * p + b) + (nyo + 1) * (i64)(ez * p + c));
        }
    // geometry
    Jm.resize(ne * 9);
    Ji.resize(ne * 9);
    dets.resize(ne);
    for (int ez = 0; ez < nz; ++ez)
      for (int ey = 0; ey < ny; ++ey)
        for (int ex = 0; ex < nx; ++ex) {
          i64 e = ex + (i64)nx * (ey + (i64)ny * ez);
          auto V = [&](int di, int dj, int dk) {
            return &verts[3 * ((ex + di) + (i64)(nx + 1) * ((ey + dj) + (i64)(ny + 1) * (ez + dk)))];
          };
          const double *v0 = V(0, 0, 0), *vx = V(1, 0, 0), *vy = V(0, 1, 0), *vz = V(0, 0, 1);
          double* J = &Jm[9 * e];
          for (int r = 0; r < 3; ++r) {
            J[3 * r + 0] = vx[r] - v0[r];
            J[3 * r + 1] = vy[r] - v0[r];
            J[3 * r + 2] = vz[r] - v0[r];
          }
          dets[e] = det3(J);
          inv3(J, &Ji[9 * e]);
        }
    build_ref_matrices();
  }

  // reference values and curls of all local basis functions at xi
  void eval_ref(const double* xi, double* val, double* curl) const {
    double cv[3][8], cd[3][8], ov[3][8], od[3][8];
    for (int d = 0; d < 3; ++d) {
      cl.eval(xi[d], cv[d], cd[d]);
      op.eval(xi[d], ov[d], od[d]);
    }
    const int pp = p + 1;
    int l = 0;
    for (int c = 0; c < pp; ++c)
      for (int b = 0; b < pp; ++b)
        for (int a = 0; a < p; ++a, ++l) {
          double f = ov[0][a] * cv[1][b] * cv[2][c];
          double fy = ov[0][a] * cd[1][b] * cv[2][c];
          double fz = ov[0][a] * cv[1][b] * cd[2][c];
          val[3 * l] = f, val[3 * l + 1] = 0, val[3 * l + 2] = 0;
          curl[3 * l] = 0, curl[3 * l + 1] = fz, curl[3 * l + 2] = -fy;
        }
    for (int c = 0; c < pp; ++c)
      for (int b = 0; b < p; ++b)
        for (int a = 0; a < pp; ++a, ++l) {
          double g = cv[0][a] * ov[1][b] * cv[2][c];
          double gx = cd[0][a] * ov[1][b] * cv[2][c];
          double gz = cv[0][a] * ov[1][b] * cd[2][c];
          val[3 * l] = 0, val[3 * l + 1] = g, val[3 * l + 2] = 0;
          curl[3 * l] = -gz, curl[3 * l + 1] = 0, curl[3 * l + 2] = gx;
        }
    for (int c = 0; c < p; ++c)
      for (int b = 0; b < pp; ++b)
        for (int a = 0; a < pp; ++a, ++l) {
          double h = cv[0][a] * cv[1][b] * ov[2][c];
          double hx = cd[0][a] * cv[1][b] * ov[2][c];
          double hy = cv[0][a] * cd[1][b] * ov[2][c];
          val[3 * l] = 0, val[3 * l + 1] = 0, val[3 * l + 2] = h;
          curl[3 * l] = hy, curl[3 * l + 1] = -hx, curl[3 * l + 2] = 0;
        }
  }

  void ref_quad(int q, std::vector<double>& xi, std::vector<double>& w) const override {
    std::vector<double> x(q), wq(q);
    gauss_legendre01(q, x.data(), wq.data());
    xi.clear();
    w.clear();
    for (int k = 0; k < q; ++k)
      for (int j = 0; j < q; ++j)
        for (int i = 0; i < q; ++i) {
          xi.push_back(x[i]);
          xi.push_back(x[j]);
          xi.push_back(x[k]);
          w.push_back(wq[i] * wq[j] * wq[k]);
        }
  }
  int elem_quad_order() const override { return p + 2; }

  void eval_phys(i64 e, const double* xi, double* x, double* adet, double* val,
                 double* curl) const override {
    const i64 ex = e % nx, ey = (e / nx) % ny, ez = e / ((i64)nx * ny);
    const double* v0 = &verts[3 * (ex + (i64)(nx + 1) * (ey + (i64)(ny + 1) * ez))];
    const double* J = &Jm[9 * e];
    const double* I = &Ji[9 * e];
    for (int r = 0; r < 3; ++r) x[r] = v0[r] + J[3 * r] * xi[0] + J[3 * r + 1] * xi[1] + J[3 * r + 2] * xi[2];
    const double d = dets[e];
    *adet = std::fabs(d);
    std::vector<double> rv(L * 3), rc(L * 3);
    eval_ref(xi, rv.data(), rc.data());
    for (int l = 0; l < L; ++l) {
      // covariant Piola: J^{-T} v ;  curl: J c / det
      for (int r = 0; r < 3; ++r) {
        val[3 * l + r] = I[r] * rv[3 * l] + I[3 + r] * rv[3 * l + 1] + I[6 + r] * rv[3 * l + 2];
        curl[3 * l + r] = (J[3 * r] * rc[3 * l] + J[3 * r + 1] * rc[3 * l + 1] + J[3 * r + 2] * rc[3 * l + 2]) / d;
      }
    }
  }

  void build_ref_matrices() {
    std::vector<double> xi, w;
    ref_quad(p + 2, xi, w);
    RM.assign((size_t)9 * L * L, 0.0);
    RC.assign((size_t)9 * L * L, 0.0);
    std::vector<double> val(L * 3), cu(L * 3);
    for (size_t q = 0; q < w.size(); ++q) {
      eval_ref(&xi[3 * q], val.data(), cu.data());
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b)
          for (int i = 0; i < L; ++i)
            for (int j = 0; j < L; ++j) {
              RM[((size_t)(3 * a + b) * L + i) * L + j] += w[q] * val[3 * i + a] * val[3 * j + b];
              RC[((size_t)(3 * a + b) * L + i) * L + j] += w[q] * cu[3 * i + a] * cu[3 * j + b];
            }
    }
  }
  // Mfac = beta |det| J^-1 J^-T ; Cfac = alpha / |det| J^T J
  void factors(i64 e, double* Mf, double* Cf) const {
    const double* J = &Jm[9 * e];
    const double* I = &Ji[9 * e];
    const double ad = std::fabs(dets[e]);
    const double a = alpha.empty() ? 0.0 : alpha[e], b = beta.empty() ? 0.0 : beta[e];
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) {
        double m = 0, k = 0;
        for (int s = 0; s < 3; ++s) {
          m += I[3 * r + s] * I[3 * c + s];
          k += J[3 * s + r] * J[3 * s + c];
        }
        Mf[3 * r + c] = b * ad * m;
        Cf[3 * r + c] = a / ad * k;
      }
  }
  void elem_row(i64 e, int li, double* row) const override {
    if (mms) {
      Prob::elem_row(e, li, row);
      return;
    }
    double Mf[9], Cf[9];
    factors(e, Mf, Cf);
    for (int j = 0; j < L; ++j) row[j] = 0.0;
    for (int ab = 0; ab < 9; ++ab) {
      const double* rm = &RM[((size_t)ab * L + li) * L];
      const double* rc = &RC[((size_t)ab * L + li) * L];
      for (int j = 0; j < L; ++j) row[j] += Mf[ab] * rm[j] + Cf[ab] * rc[j];
    }
  }
  void elem_matrix(i64 e, double* K) const override {
    if (mms) {
      elem_matrix_quad(e, K);
      return;
    }
    for (int i = 0; i < L; ++i) elem_row(e, i, K + (size_t)i * L);
  }
  bool needs_cache() const override { return mms; }

  void ess_mask(int bits, uint8_t* m) const {
    const i64 nxo = (i64)nx * p, nyo = (i64)ny * p, nzo = (i64)nz * p;
    auto on = [&](int attr) { return (bits >> (attr - 1)) & 1; };
    // comp 0: tangential on y- and z-faces
    for (i64 k = 0; k <= nzo; ++k)
      for (i64 j = 0; j <= nyo; ++j)
        for (i64 i = 0; i < nxo; ++i) {
          bool b = (j == 0 && on(3)) || (j == nyo && on(4)) || (k == 0 && on(5)) || (k == nzo && on(6));
          m[off[0] + i + nxo * (j + (nyo + 1) * k)] = b;
        }
    for (i64 k = 0; k <= nzo; ++k)
      for (i64 j = 0; j < nyo; ++j)
        for (i64 i = 0; i <= nxo; ++i) {
          bool b = (i == 0 && on(1)) || (i == nxo && on(2)) || (k == 0 && on(5)) || (k == nzo && on(6));
          m[off[1] + i + (nxo + 1) * (j + nyo * k)] = b;
        }
    for (i64 k = 0; k < nzo; ++k)
      for (i64 j = 0; j <= nyo; ++j)
        for (i64 i = 0; i <= nxo; ++i) {
          bool b = (i == 0 && on(1)) || (i == nxo && on(2)) || (j == 0 && on(3)) || (j == nyo && on(4));
          m[off[2] + i + (nxo + 1) * (j + (nyo + 1) * k)] = b;
        }
  }
};

// ---------------------------------------------------------------------------
// Tetrahedral mesh, Nedelec order 1 or 2, hierarchical basis on vertices
// sorted by global index.  Edge and face numbering: lexicographic order of
// sorted vertex tuples.
//   local dofs p=1: edges (01,02,03,12,13,23) -> W_ij
//   local dofs p=2: edge k -> [lambda_i W_ij, lambda_j W_ij];
//                   face (ijk) in (012,013,023,123) -> [lambda_k W_ij, lambda_j W_ik]
// ---------------------------------------------------------------------------
const int kTetEdges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
const int kTetFaces[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};

struct TetProb : Prob {
  int p;
  std::vector<double> verts;
  std::vector<i64> tv;  // sorted vertex ids per tet
  std::vector<std::pair<i64, i64>> edges;
  std::vector<std::array<i64, 3>> faces;
  std::vector<double> G, dets, x0;  // per element grad lambda (4x3), det J, v0

  TetProb(i64 nv, const double* v, i64 ne_, const i64* t, int p_) : p(p_) {
    verts.assign(v, v + 3 * nv);
    ne = ne_;
    tv.resize(ne * 4);
    for (i64 e = 0; e < ne; ++e) {
      i64 s[4] = {t[4 * e], t[4 * e + 1], t[4 * e + 2], t[4 * e + 3]};
      std::sort(s, s + 4);
      for (int k = 0; k < 4; ++k) tv[4 * e + k] = s[k];
    }
    edges.reserve(ne * 6);
    for (i64 e = 0; e < ne; ++e)
      for (auto& ed : kTetEdges) edges.push_back({tv[4 * e + ed[0]], tv[4 * e + ed[1]]});
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    if (p >= 2) {
      faces.reserve(ne * 4);
      for (i64 e = 0; e < ne; ++e)
        for (auto& f : kTetFaces) faces.push_back({tv[4 * e + f[0]], tv[4 * e + f[1]], tv[4 * e + f[2]]});
      std::sort(faces.begin(), faces.end());
      faces.erase(std::unique(faces.begin(), faces.end()), faces.end());
    }
    const i64 nE = edges.size(), nF = faces.size();
    L = (p == 1) ? 6 : 20;
    ndof = (p == 1) ? nE : 2 * nE + 2 * nF;
    edofs.resize(ne * L);
    for (i64 e = 0; e < ne; ++e) {
      i64* d = &edofs[e * L];
      for (int k = 0; k < 6; ++k) {
        std::pair<i64, i64> key{tv[4 * e + kTetEdges[k][0]], tv[4 * e + kTetEdges[k][1]]};
        i64 g = std::lower_bound(edges.begin(), edges.end(), key) - edges.begin();
        if (p == 1) {
          d[k] = g;
        } else {
          d[2 * k] = 2 * g;
          d[2 * k + 1] = 2 * g + 1;
        }
      }
      if (p >= 2)
        for (int f = 0; f < 4; ++f) {
          std::array<i64, 3> key{tv[4 * e + kTetFaces[f][0]], tv[4 * e + kTetFaces[f][1]],
                                 tv[4 * e + kTetFaces[f][2]]};
          i64 g = std::lower_bound(faces.begin(), faces.end(), key) - faces.begin();
          d[12 + 2 * f] = 2 * nE + 2 * g;
          d[12 + 2 * f + 1] = 2 * nE + 2 * g + 1;
        }
    }
    G.resize(ne * 12);
    dets.resize(ne);
    x0.resize(ne * 3);
    for (i64 e = 0; e < ne; ++e) {
      const double* v0 = &verts[3 * tv[4 * e]];
      double J[9], I[9];
      for (int c = 0; c < 3; ++c) {
        const double* vc = &verts[3 * tv[4 * e + c + 1]];
        for (int r = 0; r < 3; ++r) J[3 * r + c] = vc[r] - v0[r];
      }
      dets[e] = det3(J);
      inv3(J, I);
      double* g = &G[12 * e];
      for (int k = 1; k <= 3; ++k)
        for (int r = 0; r < 3; ++r) g[3 * k + r] = I[3 * (k - 1) + r];
      for (int r = 0; r < 3; ++r) g[r] = -(g[3 + r] + g[6 + r] + g[9 + r]);
      for (int r = 0; r < 3; ++r) x0[3 * e + r] = v0[r];
    }
  }

  void ref_quad(int q, std::vector<double>& xi, std::vector<double>& w) const override {
    // collapsed (Duffy) Gauss-Legendre rule; weights sum to 1/6
    std::vector<double> x(q), wq(q);
    gauss_legendre01(q, x.data(), wq.data());
    xi.clear();
    w.clear();
    for (int a = 0; a < q; ++a)
      for (int b = 0; b < q; ++b)
        for (int c = 0; c < q; ++c) {
          double u = x[a], v = x[b], t = x[c];
          xi.push_back(u);
          xi.push_back(v * (1 - u));
          xi.push_back(t * (1 - u) * (1 - v));
          w.push_back(wq[a] * wq[b] * wq[c] * (1 - u) * (1 - u) * (1 - v));
        }
  }
  int elem_quad_order() const override { return p + 3; }

  void eval_phys(i64 e, const double* xi, double* x, double* adet, double* val,
                 double* curl) const override {
    const double lam[4] = {1.0 - xi[0] - xi[1] - xi[2], xi[0], xi[1], xi[2]};
    const double* g = &G[12 * e];
    const double* v0 = &x0[3 * e];
    // x = v0 + sum_k lam_k (v_k - v0)
    for (int r = 0; r < 3; ++r) {
      x[r] = v0[r];
      for (int k = 1; k <= 3; ++k) x[r] += lam[k] * (verts[3 * tv[4 * e + k] + r] - v0[r]);
    }
    *adet = std::fabs(dets[e]);
    // W_ij and its curl
    auto W = [&](int i, int j, double* out) {
      for (int r = 0; r < 3; ++r) out[r] = lam[i] * g[3 * j + r] - lam[j] * g[3 * i + r];
    };
    auto LW = [&](int a, int i, int j, double* vv, double* cc) {
      double w[3], gc[3], c1[3];
      W(i, j, w);
      cross3(&g[3 * a], w, c1);
      cross3(&g[3 * i], &g[3 * j], gc);
      for (int r = 0; r < 3; ++r) {
        vv[r] = lam[a] * w[r];
        cc[r] = c1[r] + 2.0 * lam[a] * gc[r];
      }
    };
    if (p == 1) {
      for (int k = 0; k < 6; ++k) {
        int i = kTetEdges[k][0], j = kTetEdges[k][1];
        W(i, j, &val[3 * k]);
        cross3(&g[3 * i], &g[3 * j], &curl[3 * k]);
        for (int r = 0; r < 3; ++r) curl[3 * k + r] *= 2.0;
      }
      return;
    }
    for (int k = 0; k < 6; ++k) {
      int i = kTetEdges[k][0], j = kTetEdges[k][1];
      LW(i, i, j, &val[3 * (2 * k)], &curl[3 * (2 * k)]);
      LW(j, i, j, &val[3 * (2 * k + 1)], &curl[3 * (2 * k + 1)]);
    }
    for (int f = 0; f < 4; ++f) {
      int i = kTetFaces[f][0], j = kTetFaces[f][1], k = kTetFaces[f][2];
      LW(k, i, j, &val[3 * (12 + 2 * f)], &curl[3 * (12 + 2 * f)]);
      LW(j, i, k, &val[3 * (13 + 2 * f)], &curl[3 * (13 + 2 * f)]);
    }
  }

  void ess_mask(i64 nb, const i64* tris, const int* attr, int bits, uint8_t* m) const {
    const i64 nE = edges.size();
    for (i64 b = 0; b < nb; ++b) {
      if (!((bits >> (attr[b] - 1)) & 1)) continue;
      i64 s[3] = {tris[3 * b], tris[3 * b + 1], tris[3 * b + 2]};
      std::sort(s, s + 3);
      const int pr[3][2] = {{0, 1}, {0, 2}, {1, 2}};
      for (auto& q : pr) {
        std::pair<i64, i64> key{s[q[0]], s[q[1]]};
        i64 g = std::lower_bound(edges.begin(), edges.end(), key) - edges.begin();
        if (p == 1) {
          m[g] = 1;
        } else {
          m[2 * g] = 1;
          m[2 * g + 1] = 1;
        }
      }
      if (p >= 2) {
        std::array<i64, 3> key{s[0], s[1], s[2]};
        i64 g = std::lower_bound(faces.begin(), faces.end(), key) - faces.begin();
        m[2 * nE + 2 * g] = 1;
        m[2 * nE + 2 * g + 1] = 1;
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Krylov pieces on the eliminated operator
// ---------------------------------------------------------------------------
double dot(const std::vector<double>& a, const std::vector<double>& b) {
  double s = 0;
  for (size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
  return s;
}

// Largest eigenvalue of a symmetric tridiagonal matrix by Sturm bisection.
double tridiag_max_eig(const std::vector<double>& a, const std::vector<double>& b) {
  const int m = (int)a.size();
  double lo = 1e300, hi = -1e300;
  for (int i = 0; i < m; ++i) {
    double r = (i > 0 ? std::fabs(b[i - 1]) : 0) + (i + 1 < m ? std::fabs(b[i]) : 0);
    lo = std::min(lo, a[i] - r);
    hi = std::max(hi, a[i] + r);
  }
  auto count_below = [&](double x) {
    int c = 0;
    double d = 1.0;
    for (int i = 0; i < m; ++i) {
      double bb = i > 0 ? b[i - 1] * b[i - 1] : 0.0;
      d = a[i] - x - (i > 0 ? bb / d : 0.0);
      if (d == 0.0) d = 1e-300;
      if (d < 0) ++c;
    }
    return c;
  };
  for (int it = 0; it < 200; ++it) {
    double mid = 0.5 * (lo + hi);
    if (count_below(mid) >= m) hi = mid;
    else lo = mid;
  }
  return hi;
}

// Deterministic start vector shared by the oracle and the device path:
// v_i = frac(i * golden) - 1/2.
double start_vec(i64 i) {
  double t = (double)i * 0.6180339887498949;
  return t - std::floor(t) - 0.5;
}

double lanczos_lmax(const Prob& P, int steps, int nt) {
  const i64 n = P.ndof;
  std::vector<double> v(n), w(n), vp(n, 0.0), s(n), tmp(n);
  for (i64 i = 0; i < n; ++i) s[i] = 1.0 / std::sqrt(P.dmask[i]);
  for (i64 i = 0; i < n; ++i) v[i] = start_vec(i);
  double nv = std::sqrt(dot(v, v));
  for (auto& x : v) x /= nv;
  std::vector<double> al, be;
  double bprev = 0.0;
  for (int j = 0; j < steps; ++j) {
    for (i64 i = 0; i < n; ++i) tmp[i] = s[i] * v[i];
    P.apply_masked(tmp.data(), w.data(), nt);
    for (i64 i = 0; i < n; ++i) w[i] *= s[i];
    double a = dot(w, v);
    for (i64 i = 0; i < n; ++i) w[i] -= a * v[i] + bprev * vp[i];
    double b = std::sqrt(dot(w, w));
    al.push_back(a);
    if (j + 1 < steps) be.push_back(b);
    if (b == 0.0) break;
    vp = v;
    for (i64 i = 0; i < n; ++i) v[i] = w[i] / b;
    bprev = b;
  }
  be.resize(al.size() > 0 ? al.size() - 1 : 0);
  return tridiag_max_eig(al, be);
}

// Chebyshev iteration on D^-1 J z = D^-1 r over [lmax/ratio, lmax], zero start
// (Saad, Iterative Methods for Sparse Linear Systems, Alg. 12.1).
void cheb_apply(const Prob& P, int degree, double lmax, double ratio, const double* r, double* z,
                int nt) {
  const i64 n = P.ndof;
  const double lmin = lmax / ratio;
  const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
  const double sigma1 = theta / delta;
  double rho = 1.0 / sigma1;
  std::vector<double> d(n), res(n), Az(n);
  for (i64 i = 0; i < n; ++i) {
    d[i] = r[i] / P.dmask[i] / theta;
    z[i] = d[i];
  }
  for (int k = 1; k < degree; ++k) {
    P.apply_masked(z, Az.data(), nt);
    const double rho_n = 1.0 / (2.0 * sigma1 - rho);
    for (i64 i = 0; i < n; ++i) {
      res[i] = r[i] - Az[i];
      d[i] = rho_n * rho * d[i] + (2.0 * rho_n / delta) * res[i] / P.dmask[i];
      z[i] += d[i];
    }
    rho = rho_n;
  }
}

}  // namespace

// ===========================================================================
// C API
// ===========================================================================
extern "C" {

void* orc_hex_new(int nx, int ny, int nz, int p, const double* verts) {
  if (nx < 1 || ny < 1 || nz < 1 || p < 1 || p > 4) return nullptr;
  return new HexProb(nx, ny, nz, p, verts);
}
void* orc_tet_new(int64_t nv, const double* verts, int64_t ne, const int64_t* tets, int p) {
  if (p < 1 || p > 2) return nullptr;
  return new TetProb(nv, verts, ne, tets, p);
}
void orc_free(void* h) { delete static_cast<Prob*>(h); }
int64_t orc_ndof(void* h) { return static_cast<Prob*>(h)->ndof; }
int64_t orc_nelem(void* h) { return static_cast<Prob*>(h)->ne; }
int orc_ldof(void* h) { return static_cast<Prob*>(h)->L; }
void orc_elem_dofs(void* h, int64_t* out) {
  auto* P = static_cast<Prob*>(h);
  std::copy(P->edofs.begin(), P->edofs.end(), out);
}
int64_t orc_tet_nedges(void* h) { return (int64_t) static_cast<TetProb*>(h)->edges.size(); }
int64_t orc_tet_nfaces(void* h) { return (int64_t) static_cast<TetProb*>(h)->faces.size(); }

void orc_set_coef(void* h, const double* alpha, const double* beta) {
  auto* P = static_cast<Prob*>(h);
  P->mms = false;
  P->alpha.assign(alpha, alpha + P->ne);
  if (beta) P->beta.assign(beta, beta + P->ne);
  else P->beta.clear();
}
void orc_set_quad(void* h, int q_curl, int q_mass) {
  auto* P = static_cast<Prob*>(h);
  P->q_curl = q_curl;
  P->q_mass = q_mass;
}
void orc_set_coef_mms(void* h, double dt, double s, double sigma) {
  auto* P = static_cast<Prob*>(h);
  P->mms = true;
  P->mms_dt = dt;
  P->mms_s = s;
  P->mms_sigma = sigma;
}
int orc_assemble(void* h, int nthreads) { return static_cast<Prob*>(h)->assemble(nthreads); }
int64_t orc_nnz(void* h) { return (int64_t) static_cast<Prob*>(h)->ci.size(); }
void orc_csr(void* h, int64_t* rowptr, int64_t* col, double* val) {
  auto* P = static_cast<Prob*>(h);
  std::copy(P->rp.begin(), P->rp.end(), rowptr);
  std::copy(P->ci.begin(), P->ci.end(), col);
  std::copy(P->va.begin(), P->va.end(), val);
}
void orc_element_matrix(void* h, int64_t e, double* out) { static_cast<Prob*>(h)->elem_matrix(e, out); }

void orc_hex_ess_mask(void* h, int attr_bits, uint8_t* mask) {
  static_cast<HexProb*>(h)->ess_mask(attr_bits, mask);
}
void orc_tet_ess_mask(void* h, int64_t nb, const int64_t* tris, const int* attr, int attr_bits,
                      uint8_t* mask) {
  static_cast<TetProb*>(h)->ess_mask(nb, tris, attr, attr_bits, mask);
}
void orc_set_ess(void* h, const uint8_t* mask) {
  auto* P = static_cast<Prob*>(h);
  P->ess.assign(mask, mask + P->ndof);
  if (!P->rp.empty()) P->set_ess_default();
}
void orc_apply(void* h, const double* x, double* y, int nthreads) {
  static_cast<Prob*>(h)->spmv(x, y, nthreads);
}
void orc_apply_masked(void* h, const double* x, double* y, int nthreads) {
  static_cast<Prob*>(h)->apply_masked(x, y, nthreads);
}
void orc_diag_masked(void* h, double* d) {
  auto* P = static_cast<Prob*>(h);
  std::copy(P->dmask.begin(), P->dmask.end(), d);
}
void orc_apply_curlcurl(void* h, const double* x, double* y) {
  // element-by-element with beta switched off
  auto* P = static_cast<Prob*>(h);
  std::vector<double> saved = P->beta;
  P->beta.clear();
  const int L = P->L;
  std::vector<double> K((size_t)L * L);
  std::fill(y, y + P->ndof, 0.0);
  for (i64 e = 0; e < P->ne; ++e) {
    P->elem_matrix(e, K.data());
    for (int i = 0; i < L; ++i) {
      double s = 0;
      for (int j = 0; j < L; ++j) s += K[(size_t)i * L + j] * x[P->edofs[e * L + j]];
      y[P->edofs[e * L + i]] += s;
    }
  }
  P->beta = saved;
}

int64_t orc_build_eliminated(void* h) {
  auto* P = static_cast<Prob*>(h);
  if (P->ndof > 2147483647LL) return -1;
  P->build_eliminated();
  return (int64_t)P->eci.size();
}
void orc_spmv_eliminated(void* h, const double* x, double* y, int nthreads) {
  static_cast<Prob*>(h)->spmv_eliminated(x, y, nthreads);
}

double orc_lanczos_lmax(void* h, int steps, int nthreads) {
  return lanczos_lmax(*static_cast<Prob*>(h), steps, nthreads);
}
void orc_cheb_apply(void* h, int degree, double lmax, double ratio, const double* r, double* z,
                    int nthreads) {
  cheb_apply(*static_cast<Prob*>(h), degree, lmax, ratio, r, z, nthreads);
}

int orc_pcg(void* h, const double* b, double* x, int precond, int cheb_degree, double cheb_lmax,
            double cheb_ratio, double rtol, double atol, int maxit, int nt, int* iters,
            double* relres) {
  const Prob& P = *static_cast<Prob*>(h);
  const i64 n = P.ndof;
  if (precond == 2 && cheb_lmax <= 0) cheb_lmax = 1.1 * lanczos_lmax(P, 20, nt);
  std::vector<double> r(n), z(n), p(n), q(n), bb(b, b + n), xv(x, x + n);
  auto M = [&](const std::vector<double>& in, std::vector<double>& out) {
    if (precond == 0) out = in;
    else if (precond == 1)
      for (i64 i = 0; i < n; ++i) out[i] = in[i] / P.dmask[i];
    else cheb_apply(P, cheb_degree, cheb_lmax, cheb_ratio, in.data(), out.data(), nt);
  };
  P.apply_masked(xv.data(), q.data(), nt);
  for (i64 i = 0; i < n; ++i) r[i] = bb[i] - q[i];
  const double nb = std::sqrt(dot(bb, bb));
  double nr = std::sqrt(dot(r, r));
  const double tol = std::max(rtol * nb, atol);
  int it = 0, status = 4;
  if (nr <= tol) status = 0;
  else {
    M(r, z);
    p = z;
    double rz = dot(r, z);
    for (it = 1; it <= maxit; ++it) {
      P.apply_masked(p.data(), q.data(), nt);
      double pq = dot(p, q);
      if (!(pq > 0) || !std::isfinite(pq)) {
        status = 5;
        break;
      }
      double a = rz / pq;
      for (i64 i = 0; i < n; ++i) {
        xv[i] += a * p[i];
        r[i] -= a * q[i];
      }
      nr = std::sqrt(dot(r, r));
      if (!std::isfinite(nr)) {
        status = 5;
        break;
      }
      if (nr <= tol) {
        status = 0;
        break;
      }
      M(r, z);
      double rzn = dot(r, z);
      double be = rzn / rz;
      rz = rzn;
      for (i64 i = 0; i < n; ++i) p[i] = z[i] + be * p[i];
    }
    if (it > maxit) it = maxit;
  }
  std::copy(xv.begin(), xv.end(), x);
  if (iters) *iters = it;
  if (relres) *relres = nb > 0 ? nr / nb : nr;
  return status;
}

static void load_generic(Prob& P, int q, const std::function<void(const double*, double*)>& J, double* b) {
  std::vector<double> xi, w;
  P.ref_quad(q, xi, w);
  const int L = P.L;
  std::vector<double> val(L * 3), cu(L * 3);
  std::fill(b, b + P.ndof, 0.0);
  for (i64 e = 0; e < P.ne; ++e)
    for (size_t k = 0; k < w.size(); ++k) {
      double x[3], ad, f[3];
      P.eval_phys(e, &xi[3 * k], x, &ad, val.data(), cu.data());
      J(x, f);
      const double wq = w[k] * ad;
      for (int i = 0; i < L; ++i)
        b[P.edofs[e * L + i]] += wq * (f[0] * val[3 * i] + f[1] * val[3 * i + 1] + f[2] * val[3 * i + 2]);
    }
}

void orc_load_coil(void* h, double I0, double xc, double yc, double r0, double r1, double z0,
                   double z1, int q, double* b) {
  load_generic(*static_cast<Prob*>(h), q,
               [=](const double* x, double* f) {
                 const double dx = x[0] - xc, dy = x[1] - yc;
                 const double r = std::sqrt(dx * dx + dy * dy);
                 if (r >= r0 && r <= r1 && x[2] >= z0 && x[2] <= z1) {
                   f[0] = -I0 * dy;
                   f[1] = I0 * dx;
                 } else {
                   f[0] = 0.0;
                   f[1] = 0.0;
                 }
                 f[2] = 0.0;
               },
               b);
}
void orc_load_mms(void* h, double t, double s, int q, double* b) {
  load_generic(*static_cast<Prob*>(h), q, [=](const double* x, double* f) { mms_source(x, t, s, f); }, b);
}
// b_i = (J, w_i) for a source constant on each element (J: ne x 3), the
// VectorFEDomainLFIntegrator load of DivFreeSource::Apply
// (src/sources/div_free_source.cpp:77-80) for an element-wise source.
void orc_load_elem_field(void* h, const double* J, int q, double* b) {
  Prob& P = *static_cast<Prob*>(h);
  std::vector<double> xi, w;
  P.ref_quad(q, xi, w);
  const int L = P.L;
  std::vector<double> val(L * 3), cu(L * 3);
  std::fill(b, b + P.ndof, 0.0);
  for (i64 e = 0; e < P.ne; ++e)
    for (size_t k = 0; k < w.size(); ++k) {
      double x[3], ad;
      P.eval_phys(e, &xi[3 * k], x, &ad, val.data(), cu.data());
      const double* f = J + 3 * e;
      const double wq = w[k] * ad;
      for (int i = 0; i < L; ++i)
        b[P.edofs[e * L + i]] += wq * (f[0] * val[3 * i] + f[1] * val[3 * i + 1] + f[2] * val[3 * i + 2]);
    }
}
// b_i = (J, w_i) for the affine source J(x) = a + B x (B row-major 3x3).
void orc_load_affine(void* h, const double* a, const double* B, int q, double* b) {
  const double a0 = a[0], a1 = a[1], a2 = a[2];
  double Bm[9];
  std::memcpy(Bm, B, sizeof(Bm));
  load_generic(*static_cast<Prob*>(h), q,
               [=](const double* x, double* f) {
                 const double aa[3] = {a0, a1, a2};
                 for (int r = 0; r < 3; ++r) f[r] = aa[r] + Bm[3 * r] * x[0] + Bm[3 * r + 1] * x[1] + Bm[3 * r + 2] * x[2];
               },
               b);
}
// b_i = (nu curl A, w_i) with nu constant per element: the right-hand side of
// ScaledCurlVectorGridFunctionAux's projection (MixedVectorCurlIntegrator(nu),
// src/auxsolvers/scaled_curl_vector_gridfunction_aux.cpp:21-27), by quadrature.
void orc_curl_load(void* h, const double* nu, const double* A, int q, double* b) {
  Prob& P = *static_cast<Prob*>(h);
  std::vector<double> xi, w;
  P.ref_quad(q, xi, w);
  const int L = P.L;
  std::vector<double> val(L * 3), cu(L * 3);
  std::fill(b, b + P.ndof, 0.0);
  for (i64 e = 0; e < P.ne; ++e)
    for (size_t k = 0; k < w.size(); ++k) {
      double x[3], ad, c[3] = {0, 0, 0};
      P.eval_phys(e, &xi[3 * k], x, &ad, val.data(), cu.data());
      for (int i = 0; i < L; ++i)
        for (int r = 0; r < 3; ++r) c[r] += A[P.edofs[e * L + i]] * cu[3 * i + r];
      const double wq = w[k] * ad * nu[e];
      for (int i = 0; i < L; ++i)
        b[P.edofs[e * L + i]] += wq * (c[0] * val[3 * i] + c[1] * val[3 * i + 1] + c[2] * val[3 * i + 2]);
    }
}
double orc_l2err_mms(void* h, const double* A, double t, int q) {
  Prob& P = *static_cast<Prob*>(h);
  std::vector<double> xi, w;
  P.ref_quad(q, xi, w);
  const int L = P.L;
  std::vector<double> val(L * 3), cu(L * 3);
  double err = 0;
  for (i64 e = 0; e < P.ne; ++e)
    for (size_t k = 0; k < w.size(); ++k) {
      double x[3], ad, ex[3], ah[3] = {0, 0, 0};
      P.eval_phys(e, &xi[3 * k], x, &ad, val.data(), cu.data());
      mms_exact(x, t, ex);
      for (int i = 0; i < L; ++i)
        for (int r = 0; r < 3; ++r) ah[r] += A[P.edofs[e * L + i]] * val[3 * i + r];
      for (int r = 0; r < 3; ++r) err += w[k] * ad * (ah[r] - ex[r]) * (ah[r] - ex[r]);
    }
  return std::sqrt(err);
}
void orc_eval(void* h, const double* A, int64_t e, const double* xi, double* val, double* curl) {
  Prob& P = *static_cast<Prob*>(h);
  const int L = P.L;
  std::vector<double> v(L * 3), c(L * 3);
  double x[3], ad;
  P.eval_phys(e, xi, x, &ad, v.data(), c.data());
  for (int r = 0; r < 3; ++r) {
    val[r] = 0;
    curl[r] = 0;
    for (int i = 0; i < L; ++i) {
      val[r] += A[P.edofs[e * L + i]] * v[3 * i + r];
      curl[r] += A[P.edofs[e * L + i]] * c[3 * i + r];
    }
  }
}

}  // extern "C"

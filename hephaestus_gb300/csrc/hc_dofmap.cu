// hc_dofmap.cu -- the correspondence between a caller's dof numbering (MFEM's
// true dofs of an ND space) and this library's, for the drop-in operator.
//
// The reference hands the Jacobian solver vectors in MFEM's true-dof numbering
// (EquationSystem::FormLinearSystem / Mult, src/equation_systems/equation_system.cpp:117-210).
// Where both sides use the same local basis on each element -- MFEM's default
// ND hex basis (closed Gauss-Lobatto, open Gauss-Legendre) read in MFEM's
// lexicographic element order, and the order-1 (Whitney) tet basis -- the two
// global numberings differ by a signed permutation: element e's local
// function l is +/- one caller basis function (MFEM encodes -1 - d for the
// minus sign) and exactly one library basis function (the library orients
// every dof globally).  The map is built from both sides' element dof lists
// and checked: every library dof must be reached with one caller dof and one
// sign, and the correspondence must be one to one.  Host code only: no device
// is needed to build or apply it.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "hc_internal.h"
#include "hc_tet_topo.h"

struct hc_dofmap {
  int64_t n = 0;
  std::vector<int64_t> lib_of;  // caller dof -> library dof
  std::vector<int8_t> sign;     // per caller dof: x_lib[lib_of[d]] = sign[d] * x_caller[d]
};

namespace {
thread_local std::string g_map_err;
hc_status fail(const std::string& m, hc_status st = HC_EINVAL) {
  g_map_err = m;
  return st;
}
}  // namespace

extern "C" {

hc_status hc_dofmap_last_error(char* buf, size_t n) {
  if (!buf || n == 0) return HC_EINVAL;
  std::snprintf(buf, n, "%s", g_map_err.c_str());
  return HC_OK;
}

hc_status hc_hex_elem_dofs(int32_t order, int32_t nx, int32_t ny, int32_t nz, int64_t* out) {
  if (!out || order < 1 || order > hc::kMaxP || nx < 1 || ny < 1 || nz < 1)
    return fail("hc_hex_elem_dofs: need out, 1 <= order <= 3 and nx, ny, nz >= 1");
  const int p = order, C = p + 1, O = p;
  const int64_t mx = (int64_t)nx * p, my = (int64_t)ny * p, mz = (int64_t)nz * p;
  const int64_t n0 = mx * (my + 1) * (mz + 1), n1 = (mx + 1) * my * (mz + 1);
  const int L = 3 * O * C * C;
  for (int64_t ez = 0; ez < nz; ++ez)
    for (int64_t ey = 0; ey < ny; ++ey)
      for (int64_t ex = 0; ex < nx; ++ex) {
        int64_t* d = out + (ex + nx * (ey + (int64_t)ny * ez)) * L;
        int l = 0;
        // comp 0: (a < p, b <= p, c <= p); comp 1: (a <= p, b < p, c <= p); comp 2: (a <= p, b <= p, c < p)
        for (int c = 0; c < C; ++c)
          for (int b = 0; b < C; ++b)
            for (int a = 0; a < O; ++a)
              d[l++] = (ex * p + a) + mx * ((ey * p + b) + (my + 1) * (ez * p + c));
        for (int c = 0; c < C; ++c)
          for (int b = 0; b < O; ++b)
            for (int a = 0; a < C; ++a)
              d[l++] = n0 + (ex * p + a) + (mx + 1) * ((ey * p + b) + my * (ez * p + c));
        for (int c = 0; c < O; ++c)
          for (int b = 0; b < C; ++b)
            for (int a = 0; a < C; ++a)
              d[l++] = n0 + n1 + (ex * p + a) + (mx + 1) * ((ey * p + b) + (my + 1) * (ez * p + c));
      }
  return HC_OK;
}

hc_status hc_tet_elem_dofs(int32_t order, int64_t n_vert, int64_t n_elem, const int64_t* elem_verts, int64_t* out,
                           int64_t* n_dof) {
  if (!elem_verts || !out || !n_dof || (order != 1 && order != 2) || n_vert < 4 || n_elem < 1)
    return fail("hc_tet_elem_dofs: need elem_verts, out, n_dof, order 1 or 2, n_vert >= 4, n_elem >= 1");
  hc::topo::TetTopology T;
  std::string msg;
  const int st = hc::topo::build_tet_topology(n_elem, n_vert, elem_verts, order, nullptr, 0, nullptr, nullptr, 0, T,
                                              msg);
  if (st != hc::topo::kOk) return fail("hc_tet_elem_dofs: " + msg, st == hc::topo::kTooLarge ? HC_ENOTSUP : HC_EINVAL);
  std::copy(T.edofs.begin(), T.edofs.end(), out);
  *n_dof = T.ndof;
  return HC_OK;
}

hc_status hc_dofmap_create(int64_t n_dof, int64_t n_elem, int32_t ldofs, const int64_t* lib_elem_dofs,
                           const int32_t* caller_elem_dofs, hc_dofmap_t** out) {
  if (!out) return fail("hc_dofmap_create: null output");
  *out = nullptr;
  if (!lib_elem_dofs || !caller_elem_dofs || n_dof < 1 || n_elem < 1 || ldofs < 1)
    return fail("hc_dofmap_create: need both element dof lists, n_dof, n_elem, ldofs >= 1");
  std::vector<int64_t> caller_of(n_dof, -1);  // library dof -> caller dof
  std::vector<int8_t> sgn(n_dof, 0);
  for (int64_t e = 0; e < n_elem; ++e)
    for (int l = 0; l < ldofs; ++l) {
      const int64_t lib = lib_elem_dofs[e * ldofs + l];
      const int32_t enc = caller_elem_dofs[e * ldofs + l];
      const int64_t c = enc >= 0 ? enc : -1 - (int64_t)enc;
      const int8_t s = enc >= 0 ? 1 : -1;
      if (lib < 0 || lib >= n_dof || c >= n_dof)
        return fail("hc_dofmap_create: element " + std::to_string(e) + " local dof " + std::to_string(l) +
                    " is out of range");
      if (caller_of[lib] < 0) {
        caller_of[lib] = c;
        sgn[lib] = s;
      } else if (caller_of[lib] != c || sgn[lib] != s) {
        return fail("hc_dofmap_create: library dof " + std::to_string(lib) + " is reached as caller dof " +
                    std::to_string(caller_of[lib]) + (sgn[lib] > 0 ? " (+)" : " (-)") + " and as " +
                    std::to_string(c) + (s > 0 ? " (+)" : " (-)") + " (element " + std::to_string(e) +
                    "): the local bases or the element order differ");
      }
    }
  hc_dofmap* m = new hc_dofmap();
  m->n = n_dof;
  m->lib_of.assign(n_dof, -1);
  m->sign.assign(n_dof, 0);
  for (int64_t lib = 0; lib < n_dof; ++lib) {
    const int64_t c = caller_of[lib];
    if (c < 0) {
      delete m;
      return fail("hc_dofmap_create: library dof " + std::to_string(lib) + " belongs to no element");
    }
    if (m->lib_of[c] >= 0) {
      const int64_t other = m->lib_of[c];
      delete m;
      return fail("hc_dofmap_create: caller dof " + std::to_string(c) + " maps to library dofs " +
                  std::to_string(other) + " and " + std::to_string(lib));
    }
    m->lib_of[c] = lib;
    m->sign[c] = sgn[lib];
  }
  *out = m;
  return HC_OK;
}

hc_status hc_dofmap_to_lib(const hc_dofmap_t* m, const double* x_caller, double* x_lib) {
  if (!m || !x_caller || !x_lib || x_caller == x_lib) return fail("hc_dofmap_to_lib: null or aliased vectors");
  for (int64_t d = 0; d < m->n; ++d) x_lib[m->lib_of[d]] = m->sign[d] * x_caller[d];
  return HC_OK;
}

hc_status hc_dofmap_from_lib(const hc_dofmap_t* m, const double* x_lib, double* x_caller) {
  if (!m || !x_caller || !x_lib || x_caller == x_lib) return fail("hc_dofmap_from_lib: null or aliased vectors");
  for (int64_t d = 0; d < m->n; ++d) x_caller[d] = m->sign[d] * x_lib[m->lib_of[d]];
  return HC_OK;
}

hc_status hc_dofmap_ess_mask(const hc_dofmap_t* m, int64_t n_ess, const int32_t* ess_tdofs, uint8_t* mask) {
  if (!m || !mask || (n_ess > 0 && !ess_tdofs) || n_ess < 0) return fail("hc_dofmap_ess_mask: bad arguments");
  std::memset(mask, 0, (size_t)m->n);
  for (int64_t k = 0; k < n_ess; ++k) {
    const int32_t d = ess_tdofs[k];
    if (d < 0 || d >= m->n) return fail("hc_dofmap_ess_mask: essential dof " + std::to_string(d) + " out of range");
    mask[m->lib_of[d]] = 1;
  }
  return HC_OK;
}

int64_t hc_dofmap_size(const hc_dofmap_t* m) { return m ? m->n : -1; }

void hc_dofmap_destroy(hc_dofmap_t* m) { delete m; }

}  // extern "C"

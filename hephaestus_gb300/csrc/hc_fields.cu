// hc_fields.cu -- work around the solve that stays on the device:
//  * H = nu curl A projected into the Nedelec space (the reference's
//    ScaledCurlVectorGridFunctionAux: M H = (nu curl A, w), Jacobi PCG on the
//    unit-coefficient mass, src/auxsolvers/scaled_vector_gridfunction_aux.cpp:73-99);
//  * backward-Euler steps on device-resident state: b = P (f - C_nu A),
//    solve J dA = b, A += dt dA (TimeDomainEquationSystemProblemOperator::
//    ImplicitSolve, time_domain_equation_system_problem_operator.cpp:31-51;
//    BackwardEulerSolver, time_domain_problem_builder.cpp:59-64;
//    WeakCurlCurlKernel, weak_curl_curl_kernel.cpp:27-31).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "hc_internal.h"

namespace hc {

#define GS_LOOP(i, n) \
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

static inline unsigned fgrid(int64_t n) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)(b < 1 ? 1 : (b > 4 * 152 ? 4 * 152 : b));
}

__global__ void k_zero_ess(int64_t n, const uint8_t* __restrict__ ess, double* __restrict__ b) {
  GS_LOOP(i, n) if (ess[i]) b[i] = 0.0;
}
__global__ void k_axpy64(int64_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
  GS_LOOP(i, n) y[i] += a * x[i];
}

// The unit-coefficient Nedelec mass on the handle's space (nu = 0, sigma = 1,
// no essential dofs): same mesh, same dof numbering.  Built from the
// handle's device copies of the geometry on first use.
static hc_status ensure_mass_child(hcop* h) {
  if (h->mass_child) {
    if (h->mass_child->stream != h->stream) {
      HC_CUDA_TRY(h, cudaStreamSynchronize(h->mass_child->stream));
      h->mass_child->stream = h->stream;
    }
    return HC_OK;
  }
  hc_problem_desc d;
  std::memset(&d, 0, sizeof(d));
  d.elem_type = h->type;
  d.order = h->p;
  d.dt = 1.0;
  std::vector<double> nu((size_t)h->ne, 0.0), sigma((size_t)h->ne, 1.0), verts;
  std::vector<int64_t> ev;
  d.nu = nu.data();
  d.sigma = sigma.data();
  if (h->type == HC_HEX) {
    d.nx = h->nx;
    d.ny = h->ny;
    d.nz = h->nz;
    verts.resize((size_t)(h->nx + 1) * (h->ny + 1) * (h->nz + 1) * 3);
    HC_CUDA_TRY(h, cudaMemcpyAsync(verts.data(), h->verts, verts.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                   h->stream));
    HC_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    d.vertices = verts.data();
  } else {
    verts.resize((size_t)h->n_vert * 3);
    std::vector<int32_t> sv((size_t)h->ne * 4);
    HC_CUDA_TRY(h, cudaMemcpyAsync(verts.data(), h->verts, verts.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                   h->stream));
    HC_CUDA_TRY(h, cudaMemcpyAsync(sv.data(), h->tet_sv, sv.size() * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                   h->stream));
    HC_CUDA_TRY(h, cudaStreamSynchronize(h->stream));
    ev.assign(sv.begin(), sv.end());
    d.n_vert = h->n_vert;
    d.n_elem = h->ne;
    d.vertices = verts.data();
    d.elem_verts = ev.data();
  }
  hcop_t* c = nullptr;
  const hc_status st = hc_create(&d, &c);
  if (st != HC_OK) {
    char buf[256];
    hc_last_error(nullptr, buf, sizeof(buf));
    h->err = std::string("unit-coefficient mass operator: ") + buf;
    return st;
  }
  if (c->ndof != h->ndof) {
    hc_destroy(c);
    h->err = "unit-coefficient mass operator: dof count differs from the handle's";
    return HC_ECUDA;
  }
  c->stream = h->stream;
  h->mass_child = c;
  return HC_OK;
}

}  // namespace hc

using namespace hc;

extern "C" {

hc_status hc_magnetic_field_device(hcop_t* h, const double* A, double* H, double rtol, hc_solve_info* info) {
  if (!h || !A || !H || !(rtol > 0.0)) {
    if (h) h->err = "hc_magnetic_field_device: need A, H and rtol > 0";
    return HC_EINVAL;
  }
  hc_status st = ensure_mass_child(h);
  if (st != HC_OK) return st;
  st = hc_curl_load_device(h, A, h->ybuf);
  if (st != HC_OK) return st;
  hc_solve_params prm;
  std::memset(&prm, 0, sizeof(prm));
  prm.precision = HC_FP64;
  prm.precond = HC_PRECOND_JACOBI;
  prm.rtol = rtol;
  prm.atol = 0.0;
  prm.maxit = 5000;
  st = hc_solve_device(h->mass_child, &prm, h->ybuf, H, info);
  if (st != HC_OK && st != HC_NOT_CONVERGED && st != HC_BREAKDOWN) h->err = h->mass_child->err;
  return st;
}

hc_status hc_be_rhs_device(hcop_t* h, const double* f, const double* A, double* b) {
  if (!h || !f || !A || !b) return HC_EINVAL;
  if (h->type != HC_HEX) {
    h->err = "hc_be_rhs_device: structured hex grids only (tet element matrices combine dt C + M)";
    return HC_ENOTSUP;
  }
  const int64_t n = h->ndof;
  if (b != f) HC_CUDA_TRY(h, cudaMemcpyAsync(b, f, n * sizeof(double), cudaMemcpyDeviceToDevice, h->stream));
  // C_nu = (dt C_nu) / dt; the full A (boundary values included), as the
  // reference's curl-curl form applies it to the grid function
  HC_CUDA_TRY(h, hex_apply<double>(h->hexdev(), h->fac, A, b, 0.0, -1.0 / h->dt, false, nullptr, nullptr, h->stream,
                                   false));
  k_zero_ess<<<fgrid(n), 256, 0, h->stream>>>(n, h->ess, b);
  HC_CUDA_TRY(h, cudaGetLastError());
  return HC_OK;
}

hc_status hc_be_update_device(hcop_t* h, double* A, const double* dA) {
  if (!h || !A || !dA) return HC_EINVAL;
  const int64_t n = h->ndof;
  k_axpy64<<<fgrid(n), 256, 0, h->stream>>>(n, h->dt, dA, A);
  HC_CUDA_TRY(h, cudaGetLastError());
  return HC_OK;
}

hc_status hc_be_steps_device(hcop_t* h, const hc_solve_params* prm, int32_t nsteps, const double* f, double* A,
                             double* dA, double* b, hc_solve_info* info) {
  if (!h || !prm || !f || !A || !dA || !b || nsteps < 1) {
    if (h) h->err = "hc_be_steps_device: null argument or nsteps < 1";
    return HC_EINVAL;
  }
  if (h->type != HC_HEX) {
    h->err = "hc_be_steps_device: structured hex grids only";
    return HC_ENOTSUP;
  }
  if (info) {
    std::memset(info, 0, sizeof(hc_solve_info) * (size_t)nsteps);
    for (int k = 0; k < nsteps; ++k) info[k].status = -1;  // steps not taken
  }
  for (int k = 0; k < nsteps; ++k) {
    hc_status st = hc_be_rhs_device(h, f, A, b);
    if (st != HC_OK) return st;
    HC_CUDA_TRY(h, cudaMemsetAsync(dA, 0, h->ndof * sizeof(double), h->stream));
    hc_solve_info loc;
    st = hc_solve_device(h, prm, b, dA, info ? &info[k] : &loc);
    if (st != HC_OK) return st;
    st = hc_be_update_device(h, A, dA);
    if (st != HC_OK) return st;
  }
  return HC_OK;
}

}  // extern "C"

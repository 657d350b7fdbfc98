// hcurl_mfem.hpp -- header-only MFEM adapter over the C ABI of hcurl_op.h.
//
// Drop-in for the reference's H(curl) operator and Jacobian solve:
//  * GpuHCurlOperator : mfem::Operator   replaces the HypreParMatrix that
//    EquationSystem::GetGradient returns (src/equation_systems/equation_system.cpp:201-210);
//    Mult() is hc_mult, i.e. y = (P K P + I - P) x with K = dt C_nu + M_sigma.
//  * GpuHCurlSolver : mfem::Solver       replaces the HyprePCG + HypreAMS pair built by
//    HCurlFormulation::ConstructJacobianSolver / ConstructJacobianPreconditioner
//    (src/formulations/HCurl/hcurl_formulation.cpp:69-85); Mult() is hc_solve.
//  * WeakCurlCurl(u, lf) is WeakCurlCurlKernel::Apply (src/kernels/weak_curl_curl_kernel.cpp:27-31).
//
// Errors are reported the MFEM way (MFEM_ABORT with the library's message),
// as the reference does for its own failures (src/named_fields_map/named_fields_map.hpp:117).
// Vectors are passed as host data (the reference configures no mfem::Device).
#pragma once
#include <cstdio>
#include <string>
#include <vector>

#include "hcurl_op.h"
#include "mfem.hpp"

namespace hcurl {

inline std::string last_error(const hcop_t* h) {
  char buf[512];
  hc_last_error(h, buf, sizeof(buf));
  return std::string(buf);
}

class GpuHCurlOperator : public mfem::Operator {
public:
  explicit GpuHCurlOperator(const hc_problem_desc& desc) {
    const hc_status st = hc_create(&desc, &h_);
    if (st != HC_OK) MFEM_ABORT("hc_create failed: " << last_error(nullptr));
    height = width = (int)hc_num_dofs(h_);
  }
  ~GpuHCurlOperator() override { hc_destroy(h_); }
  GpuHCurlOperator(const GpuHCurlOperator&) = delete;
  GpuHCurlOperator& operator=(const GpuHCurlOperator&) = delete;

  void Mult(const mfem::Vector& x, mfem::Vector& y) const override {
    Check(hc_mult(h_, x.HostRead(), y.HostWrite()));
  }
  // The operator is linear: its gradient is itself (EquationSystem::GetGradient).
  mfem::Operator& GetGradient(const mfem::Vector&) const override {
    return const_cast<GpuHCurlOperator&>(*this);
  }
  // lf += scale * C_nu u   (WeakCurlCurlKernel::Apply uses scale = -1)
  void AddWeakCurlCurl(const mfem::Vector& u, mfem::Vector& lf, double scale = -1.0) const {
    Check(hc_add_weak_curlcurl(h_, u.HostRead(), lf.HostReadWrite(), scale));
  }
  void AssembleDiagonal(mfem::Vector& diag) const override { Check(hc_diag(h_, diag.HostWrite())); }
  hcop_t* Handle() const { return h_; }

private:
  void Check(hc_status st) const {
    if (st != HC_OK) MFEM_ABORT("hcurl: " << last_error(h_));
  }
  hcop_t* h_ = nullptr;
};

// Solver options use the reference's names and defaults
// (DefaultJacobiPCGSolver, src/solvers/hephaestus_solvers.hpp:34-57).
struct GpuHCurlSolverOptions {
  double tolerance = 1e-9;
  double abs_tolerance = 1e-16;
  int max_iter = 1000;
  int precision = HC_FP64;               // HC_FP64 (drop-in) or HC_MIXED
  int preconditioner = HC_PRECOND_JACOBI;
  int cheb_degree = 2;
  double inner_tolerance = 1e-4;
};

class GpuHCurlSolver : public mfem::Solver {
public:
  explicit GpuHCurlSolver(const GpuHCurlSolverOptions& o = GpuHCurlSolverOptions()) {
    prm_.precision = o.precision;
    prm_.precond = o.preconditioner;
    prm_.cheb_degree = o.cheb_degree;
    prm_.cheb_ratio = 30.0;
    prm_.cheb_lmax = 0.0;
    prm_.rtol = o.tolerance;
    prm_.atol = o.abs_tolerance;
    prm_.maxit = o.max_iter;
    prm_.inner_rtol = o.inner_tolerance;
    prm_.max_outer = 50;
  }
  void SetOperator(const mfem::Operator& op) override {
    op_ = dynamic_cast<const GpuHCurlOperator*>(&op);
    if (!op_) MFEM_ABORT("GpuHCurlSolver needs a GpuHCurlOperator");
    height = width = op.Height();
  }
  // x holds the initial guess (iterative_mode semantics of HyprePCG).
  void Mult(const mfem::Vector& b, mfem::Vector& x) const override {
    if (!iterative_mode) x = 0.0;
    const hc_status st = hc_solve(op_->Handle(), &prm_, b.HostRead(), x.HostReadWrite(), &info_);
    if (st != HC_OK && st != HC_NOT_CONVERGED) MFEM_ABORT("hc_solve: " << last_error(op_->Handle()));
  }
  const hc_solve_info& Info() const { return info_; }

  // Solve for the columns of B together (hc_solve_multi: one block PCG whose
  // iterations share every operator apply; tet meshes).  B and X are
  // ndof x nrhs, nrhs in {1, 2, 4, 8, 16, 32}; X holds the initial guesses
  // (iterative_mode) and receives the solutions; Infos() has one report per column.
  void MultBlock(const mfem::DenseMatrix& B, mfem::DenseMatrix& X) const {
    const int n = B.Height(), r = B.Width();
    if (X.Height() != n || X.Width() != r) MFEM_ABORT("GpuHCurlSolver::MultBlock: B and X shapes differ");
    std::vector<double> b((size_t)n * r), x((size_t)n * r, 0.0);
    for (int k = 0; k < r; ++k)
      for (int i = 0; i < n; ++i) {
        b[(size_t)i * r + k] = B(i, k);
        if (iterative_mode) x[(size_t)i * r + k] = X(i, k);
      }
    infos_.assign(r, hc_solve_info{});
    const hc_status st = hc_solve_multi(op_->Handle(), &prm_, r, b.data(), x.data(), infos_.data());
    if (st != HC_OK && st != HC_NOT_CONVERGED) MFEM_ABORT("hc_solve_multi: " << last_error(op_->Handle()));
    for (int k = 0; k < r; ++k)
      for (int i = 0; i < n; ++i) X(i, k) = x[(size_t)i * r + k];
  }
  const std::vector<hc_solve_info>& Infos() const { return infos_; }

private:
  const GpuHCurlOperator* op_ = nullptr;
  hc_solve_params prm_{};
  mutable hc_solve_info info_{};
  mutable std::vector<hc_solve_info> infos_;
};

}  // namespace hcurl

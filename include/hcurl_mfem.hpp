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
//  * DofMap + MfemHexLexicographicDofs / MfemTetOrder1Dofs: the signed
//    permutation between MFEM's true dofs and the library's, applied around
//    Mult and the solve (hex spaces of any order with MFEM's default ND basis,
//    order-1 tet spaces); the whole mesh lives on one rank.
//
// Errors are reported the MFEM way (MFEM_ABORT with the library's message),
// as the reference does for its own failures (src/named_fields_map/named_fields_map.hpp:117).
// Vectors are passed as host data (the reference configures no mfem::Device).
#pragma once
#include <algorithm>
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

// Signed permutation between MFEM's true dofs and the library's (hc_dofmap_*).
// The shim takes the whole mesh on one rank (run the reference with
// mpirun -n 1): true dofs are the local dofs of the ND space.
class DofMap {
public:
  DofMap(int64_t n_dof, int64_t n_elem, int ldofs, const std::vector<int64_t>& lib_elem_dofs,
         const std::vector<int32_t>& mfem_elem_dofs) {
    if (hc_dofmap_create(n_dof, n_elem, ldofs, lib_elem_dofs.data(), mfem_elem_dofs.data(), &m_) != HC_OK) {
      char buf[512];
      hc_dofmap_last_error(buf, sizeof(buf));
      MFEM_ABORT("hcurl::DofMap: " << buf);
    }
  }
  ~DofMap() { hc_dofmap_destroy(m_); }
  DofMap(const DofMap&) = delete;
  DofMap& operator=(const DofMap&) = delete;
  int64_t Size() const { return hc_dofmap_size(m_); }
  void ToLib(const double* x_mfem, double* x_lib) const { hc_dofmap_to_lib(m_, x_mfem, x_lib); }
  void FromLib(const double* x_lib, double* x_mfem) const { hc_dofmap_from_lib(m_, x_lib, x_mfem); }
  // hc_problem_desc::ess_mask from the ess_tdof_list of GetEssentialTrueDofs
  std::vector<uint8_t> EssMask(const std::vector<int32_t>& ess_tdofs) const {
    std::vector<uint8_t> mask((size_t)Size(), 0);
    if (hc_dofmap_ess_mask(m_, (int64_t)ess_tdofs.size(), ess_tdofs.data(), mask.data()) != HC_OK)
      MFEM_ABORT("hcurl::DofMap::EssMask: essential dof out of range");
    return mask;
  }

private:
  hc_dofmap_t* m_ = nullptr;
};

// MFEM's signed global dof of every element and lexicographic local dof of an
// ND hex space: the element's native dofs (GetElementDofs, -1 - d for a
// reversed function) read through the element's lexicographic dof map
// (TensorBasisElement::GetDofMap: lexicographic index -> native index, -1 - n
// where the lexicographic function is minus the native one).  Elements must
// be in the library's structured order (MakeCartesian3D: x fastest).
inline std::vector<int32_t> MfemHexLexicographicDofs(const mfem::FiniteElementSpace& fes) {
  std::vector<int32_t> out;
  mfem::Array<int> dofs;
  for (int e = 0; e < fes.GetNE(); ++e) {
    fes.GetElementDofs(e, dofs);
    const auto* tfe = dynamic_cast<const mfem::VectorTensorFiniteElement*>(fes.GetFE(e));
    if (!tfe) MFEM_ABORT("MfemHexLexicographicDofs: not a tensor-product ND element");
    const mfem::Array<int>& dmap = tfe->GetDofMap();
    for (int l = 0; l < dmap.Size(); ++l) {
      int nd = dmap[l], s = 1;
      if (nd < 0) {
        nd = -1 - nd;
        s = -s;
      }
      int g = dofs[nd];
      if (g < 0) {
        g = -1 - g;
        s = -s;
      }
      out.push_back(s > 0 ? g : -1 - g);
    }
  }
  return out;
}

// MFEM's signed global dof of every order-1 ND tet element in the library's
// local order (the 6 edges of the element's vertices sorted by global id,
// each oriented from the lower id): the element's local edge (i, j) of
// Geometry::Constants<TETRAHEDRON>::Edges carries MFEM's function with
// tangent v_i -> v_j; it is minus the library's when v_i > v_j.
inline std::vector<int32_t> MfemTetOrder1Dofs(const mfem::FiniteElementSpace& fes, const mfem::Mesh& mesh) {
  using Geo = mfem::Geometry::Constants<mfem::Geometry::TETRAHEDRON>;
  std::vector<int32_t> out;
  mfem::Array<int> dofs, v;
  const int lib_edges[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
  for (int e = 0; e < fes.GetNE(); ++e) {
    fes.GetElementDofs(e, dofs);
    mesh.GetElementVertices(e, v);
    int sv[4] = {v[0], v[1], v[2], v[3]};
    std::sort(sv, sv + 4);
    for (int k = 0; k < 6; ++k) {
      const int a = sv[lib_edges[k][0]], b = sv[lib_edges[k][1]];  // a < b
      int found = -1, s = 1;
      for (int m = 0; m < 6; ++m) {
        const int vi = v[Geo::Edges[m][0]], vj = v[Geo::Edges[m][1]];
        if ((vi == a && vj == b) || (vi == b && vj == a)) {
          found = m;
          s = vi == a ? 1 : -1;
        }
      }
      if (found < 0) MFEM_ABORT("MfemTetOrder1Dofs: edge not found");
      int g = dofs[found];
      if (g < 0) {
        g = -1 - g;
        s = -s;
      }
      out.push_back(s > 0 ? g : -1 - g);
    }
  }
  return out;
}

class GpuHCurlOperator : public mfem::Operator {
public:
  // map: MFEM true dofs <-> library dofs (nullptr when the caller already
  // uses the library's numbering); it must outlive the operator.
  explicit GpuHCurlOperator(const hc_problem_desc& desc, const DofMap* map = nullptr) : map_(map) {
    const hc_status st = hc_create(&desc, &h_);
    if (st != HC_OK) MFEM_ABORT("hc_create failed: " << last_error(nullptr));
    height = width = (int)hc_num_dofs(h_);
    if (map_ && map_->Size() != height) MFEM_ABORT("hcurl::GpuHCurlOperator: dof map size differs from the space");
    if (map_) {
      xl_.resize(height);
      yl_.resize(height);
    }
  }
  ~GpuHCurlOperator() override { hc_destroy(h_); }
  GpuHCurlOperator(const GpuHCurlOperator&) = delete;
  GpuHCurlOperator& operator=(const GpuHCurlOperator&) = delete;

  void Mult(const mfem::Vector& x, mfem::Vector& y) const override {
    if (!map_) {
      Check(hc_mult(h_, x.HostRead(), y.HostWrite()));
      return;
    }
    map_->ToLib(x.HostRead(), xl_.data());
    Check(hc_mult(h_, xl_.data(), yl_.data()));
    map_->FromLib(yl_.data(), y.HostWrite());
  }
  const DofMap* Map() const { return map_; }
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
  const DofMap* map_ = nullptr;
  mutable std::vector<double> xl_, yl_;
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
    const DofMap* m = op_->Map();
    if (!m) {
      const hc_status st = hc_solve(op_->Handle(), &prm_, b.HostRead(), x.HostReadWrite(), &info_);
      if (st != HC_OK && st != HC_NOT_CONVERGED) MFEM_ABORT("hc_solve: " << last_error(op_->Handle()));
      return;
    }
    std::vector<double> bl((size_t)height), xl((size_t)height);
    m->ToLib(b.HostRead(), bl.data());
    m->ToLib(x.HostRead(), xl.data());
    const hc_status st = hc_solve(op_->Handle(), &prm_, bl.data(), xl.data(), &info_);
    if (st != HC_OK && st != HC_NOT_CONVERGED) MFEM_ABORT("hc_solve: " << last_error(op_->Handle()));
    m->FromLib(xl.data(), x.HostReadWrite());
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

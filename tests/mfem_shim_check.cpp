// Type-checks include/hcurl_mfem.hpp against the MFEM stub and links it with
// the CUDA library: construct the shim objects the way a formulation would.
#include "hcurl_mfem.hpp"

int shim_smoke(hc_problem_desc d) {
  hcurl::GpuHCurlOperator op(d);
  hcurl::GpuHCurlSolverOptions o;
  o.precision = HC_MIXED;
  hcurl::GpuHCurlSolver solver(o);
  solver.SetOperator(op.GetGradient(mfem::Vector(op.Height())));
  mfem::Vector b(op.Height()), x(op.Height());
  solver.Mult(b, x);
  op.Mult(x, b);
  mfem::DenseMatrix B(op.Height(), 16), X(op.Height(), 16);
  solver.MultBlock(B, X);
  return solver.Info().iterations + (int)solver.Infos().size();
}

// MFEM-numbered operator and solve through the dof map
int shim_mapped(hc_problem_desc d, const mfem::FiniteElementSpace& fes, const mfem::Mesh& mesh) {
  const int p = d.order;
  std::vector<int64_t> lib((size_t)d.nx * d.ny * d.nz * 3 * p * (p + 1) * (p + 1));
  hc_hex_elem_dofs(p, d.nx, d.ny, d.nz, lib.data());
  const std::vector<int32_t> mf = hcurl::MfemHexLexicographicDofs(fes);
  const int64_t n = *std::max_element(lib.begin(), lib.end()) + 1;
  hcurl::DofMap map(n, (int64_t)d.nx * d.ny * d.nz, 3 * p * (p + 1) * (p + 1), lib, mf);
  const std::vector<uint8_t> mask = map.EssMask(std::vector<int32_t>{0, 1, 2});
  d.ess_mask = mask.data();
  hcurl::GpuHCurlOperator op(d, &map);
  hcurl::GpuHCurlSolver solver;
  solver.SetOperator(op);
  mfem::Vector b(op.Height()), x(op.Height());
  solver.Mult(b, x);
  op.Mult(x, b);
  return (int)hcurl::MfemTetOrder1Dofs(fes, mesh).size();
}

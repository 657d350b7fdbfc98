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

// Test driver for hc_amg_host.h: reads an SPD CSR matrix, runs one level of the
// smoothed-aggregation set-up and the dense scaled inverse, writes the results.
// Input  (binary): int32 n, int32 nnz, int32 rp[n+1], int32 ci[nnz], float64 va[nnz]
// Output (binary): float64 lmax, int32 na, int32 agg[n], CSR P (n x na), CSR Ac (na x na),
//                  int32 ok, float32 inv[na*na], float32 sc[na]   (CSR: int32 rows, nnz, rp, ci; float64 va)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "hc_amg_host.h"

using hc::amg::HCsr;

static void wcsr(FILE* f, const HCsr& M) {
  const int nnz = (int)M.ci.size();
  fwrite(&M.n, 4, 1, f);
  fwrite(&nnz, 4, 1, f);
  fwrite(M.rp.data(), 4, M.rp.size(), f);
  fwrite(M.ci.data(), 4, nnz, f);
  fwrite(M.va.data(), 8, nnz, f);
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 3;
  HCsr A;
  int nnz = 0;
  if (fread(&A.n, 4, 1, f) != 1 || fread(&nnz, 4, 1, f) != 1) return 4;
  A.m = A.n;
  A.rp.resize(A.n + 1);
  A.ci.resize(nnz);
  A.va.resize(nnz);
  if (fread(A.rp.data(), 4, A.n + 1, f) != (size_t)A.n + 1 || fread(A.ci.data(), 4, nnz, f) != (size_t)nnz ||
      fread(A.va.data(), 8, nnz, f) != (size_t)nnz)
    return 5;
  fclose(f);
  const std::vector<double> dg = hc::amg::diagonal(A);
  const double lmax = hc::amg::lmax_scaled(A, dg);
  std::vector<int> agg;
  const int na = hc::amg::aggregate(A, dg, 0.08, agg);
  const HCsr P = hc::amg::smooth_prolongator(A, dg, agg, na, 4.0 / (3.0 * lmax));
  const HCsr R = hc::amg::transpose(P);
  const HCsr Ac = hc::amg::spgemm(R, hc::amg::spgemm(A, P));
  std::vector<float> inv, sc;
  const int ok = hc::amg::dense_scaled_inverse(Ac, hc::amg::diagonal(Ac), inv, sc) ? 1 : 0;
  FILE* o = fopen(argv[2], "wb");
  if (!o) return 6;
  fwrite(&lmax, 8, 1, o);
  fwrite(&na, 4, 1, o);
  fwrite(agg.data(), 4, agg.size(), o);
  wcsr(o, P);
  wcsr(o, Ac);
  fwrite(&ok, 4, 1, o);
  fwrite(inv.data(), 4, inv.size(), o);
  fwrite(sc.data(), 4, sc.size(), o);
  fclose(o);
  return 0;
}

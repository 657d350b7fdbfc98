// Test driver for hc_tetaux_host.h.  Input (binary): int64 p, ne, N, n_edges;
// int32 sv[ne*4], int32 ed[ne*L], uint8 ess[N], float64 Ae[ne*nout].
// Output (binary): int32 ok, nfree, nfe, nn; int64 nface0; int32 gnode[3N];
// int32 gedge[3N or 0]; CSR Gt (int32 rows, nnz, rp, ci; float64 va);
// CSR A (same); float32 dl[nn or 0].
#include <cstdio>
#include <vector>

#include "hc_tetaux_host.h"

static void wcsr(FILE* f, const hc::amg::HCsr& M) {
  const int nnz = (int)M.ci.size();
  std::fwrite(&M.n, 4, 1, f);
  std::fwrite(&nnz, 4, 1, f);
  std::fwrite(M.rp.data(), 4, M.rp.size(), f);
  std::fwrite(M.ci.data(), 4, nnz, f);
  std::fwrite(M.va.data(), 8, nnz, f);
}

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int64_t hdr[4];
  if (std::fread(hdr, 8, 4, f) != 4) return 4;
  const int p = (int)hdr[0];
  const int64_t ne = hdr[1], N = hdr[2], nE = hdr[3];
  const int L = p == 1 ? 6 : 20, nout = p == 1 ? 10 : 16;
  std::vector<int32_t> sv(ne * 4), ed(ne * L);
  std::vector<uint8_t> ess(N);
  std::vector<double> Ae(ne * nout);
  if (std::fread(sv.data(), 4, sv.size(), f) != sv.size() || std::fread(ed.data(), 4, ed.size(), f) != ed.size() ||
      std::fread(ess.data(), 1, ess.size(), f) != ess.size() || std::fread(Ae.data(), 8, Ae.size(), f) != Ae.size())
    return 5;
  std::fclose(f);
  hc::AuxStructure S;
  std::string msg;
  const int32_t ok = hc::build_aux_structure(p, ne, N, nE, sv.data(), ed.data(), ess.data(), Ae.data(), S, msg) ? 1 : 0;
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 6;
  const int32_t h4[4] = {ok, S.nfree, S.nfe, S.nn};
  std::fwrite(h4, 4, 4, o);
  std::fwrite(&S.nface0, 8, 1, o);
  if (ok) {
    std::fwrite(S.gnode.data(), 4, S.gnode.size(), o);
    std::fwrite(S.gedge.data(), 4, S.gedge.size(), o);
    wcsr(o, S.Gt);
    wcsr(o, S.A);
    std::fwrite(S.dl.data(), 4, S.dl.size(), o);
  }
  std::fclose(o);
  return 0;
}

// Prints the local discrete-gradient tables of hc_tet_grad.h: for order p,
// rows = local dofs, columns = 4 vertex hats (and, for p = 2, 6 edge bubbles).
#include <cstdio>
#include <cstdlib>

#include "hc_tet_grad.h"

int main(int argc, char** argv) {
  const int p = argc > 1 ? std::atoi(argv[1]) : 2;
  const int L = p == 1 ? 6 : 20;
  for (int I = 0; I < L; ++I) {
    float row[10] = {0};
    int v[3];
    float c[3];
    const int nn = hc::ta_local(p, I, hc::kHEdges, hc::kHFaces, v, c);
    for (int k = 0; k < nn; ++k) row[v[k]] += c[k];
    if (p == 2)
      for (int ke = 0; ke < 6; ++ke) row[4 + ke] = hc::ta_bubble(I, ke, hc::kHEdges, hc::kHFaces);
    for (int k = 0; k < (p == 2 ? 10 : 4); ++k) std::printf("%g ", row[k]);
    std::printf("\n");
  }
  return 0;
}

// Test driver for hc_tet_topo.h.  Input (binary): int64 ne, nv, p, bits, n_bdr;
// int64 elem_verts[ne*4], int64 bdr_tris[n_bdr*3], int32 bdr_attr[n_bdr].
// Output (binary): int32 status, int32 len, char msg[len], int64 ndof, n_edges,
// n_faces; int32 edofs[ne*L]; uint8 ess[ndof]   (arrays only when status == 0).
#include <cstdio>
#include <vector>

#include "hc_tet_topo.h"

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  int64_t hdr[5];
  if (std::fread(hdr, 8, 5, f) != 5) return 4;
  const int64_t ne = hdr[0], nv = hdr[1], p = hdr[2], bits = hdr[3], nb = hdr[4];
  std::vector<int64_t> ev(ne * 4), bt(nb * 3);
  std::vector<int32_t> ba(nb);
  if (std::fread(ev.data(), 8, ev.size(), f) != ev.size() || std::fread(bt.data(), 8, bt.size(), f) != bt.size() ||
      std::fread(ba.data(), 4, ba.size(), f) != ba.size())
    return 5;
  std::fclose(f);
  hc::topo::TetTopology T;
  std::string msg;
  const int st = hc::topo::build_tet_topology(ne, nv, ev.data(), (int)p, nullptr, nb, bt.data(), ba.data(), (int)bits,
                                              T, msg);
  FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 6;
  const int32_t s32 = st, len = (int32_t)msg.size();
  std::fwrite(&s32, 4, 1, o);
  std::fwrite(&len, 4, 1, o);
  std::fwrite(msg.data(), 1, msg.size(), o);
  const int64_t sizes[3] = {T.ndof, T.n_edges, T.n_faces};
  std::fwrite(sizes, 8, 3, o);
  if (st == 0) {
    std::fwrite(T.edofs.data(), 4, T.edofs.size(), o);
    std::fwrite(T.ess.data(), 1, T.ess.size(), o);
  }
  std::fclose(o);
  return 0;
}

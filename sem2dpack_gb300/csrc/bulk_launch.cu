// bulk_launch.cu -- NGLL dispatch and tile-shape selection for the bulk kernel.
#include <cstdio>
#include <cstdlib>
#include <string>

#include "bulk_launch.h"

namespace sem2d {

thread_local std::string g_bulk_err;

const char *bulk_last_error() { return g_bulk_err.c_str(); }

int launch_bulk(const BulkConfig &c) {
  switch (c.N) {
    case 5: return launch_bulk_n5(c);
    case 6: return launch_bulk_n6(c);
    case 9: return launch_bulk_n9(c);
    default: g_bulk_err = "NGLL not compiled"; return 1;
  }
}

int configure_bulk(const BulkConfig &c) {
  switch (c.N) {
    case 5: return configure_bulk_n5(c);
    case 6: return configure_bulk_n6(c);
    case 9: return configure_bulk_n9(c);
    default: g_bulk_err = "NGLL not compiled"; return 1;
  }
}

size_t bulk_smem(int N, int ndof, int mixed, int tn, int nmat, int kv, int me) {
  switch (N) {
    case 5: return bulk_smem_n5(ndof, mixed, tn, nmat, kv, me);
    case 6: return bulk_smem_n6(ndof, mixed, tn, nmat, kv, me);
    case 9: return bulk_smem_n9(ndof, mixed, tn, nmat, kv, me);
    default: return size_t(-1);
  }
}

int tile_nodes_for(int N, int nx, int nz, const int *row0, int TX, int TZ) {
  int best = 0;
  for (int ez0 = 0; ez0 < nz; ez0 += TZ) {
    const int ez1 = ez0 + TZ < nz ? ez0 + TZ : nz;
    const int hz = (ez0 > 0 && row0[ez0] == row0[ez0 - 1] + (N - 1)) ? 1 : 0;
    const int TH = row0[ez1 - 1] + N - row0[ez0 - hz];
    for (int ex0 = 0; ex0 < nx; ex0 += TX) {
      const int ex1 = ex0 + TX < nx ? ex0 + TX : nx;
      const int hx = ex0 > 0 ? 1 : 0;
      const int TW = (ex1 - 1) * (N - 1) + N - (ex0 - hx) * (N - 1);
      if (TW * TH > best) best = TW * TH;
    }
  }
  return best;
}

int choose_tiles(int N, int ndof, int mixed, int nx, int nz, const int *row0, int nmat, int has_kv,
                 int mat_elem, int *TX, int *TZ, int *tile_nodes) {
  const size_t kSmemCap = 113 * 1024;  // two CTAs per SM
  const char *env = std::getenv("SEM2D_TILE");
  if (env) {
    int tx = 0, tz = 0;
    if (std::sscanf(env, "%dx%d", &tx, &tz) == 2 && tx > 0 && tz > 0) {
      const int tn = tile_nodes_for(N, nx, nz, row0, tx, tz);
      if (bulk_smem(N, ndof, mixed, tn, nmat, has_kv, mat_elem) <= 227 * 1024) {
        *TX = tx;
        *TZ = tz;
        *tile_nodes = tn;
        return 0;
      }
      g_bulk_err = "SEM2D_TILE does not fit in shared memory";
      return 1;
    }
  }
  static const int cand[][2] = {{16, 8}, {8, 8}, {8, 4}, {4, 4}, {4, 2}, {2, 2}, {1, 1}};
  for (const auto &c : cand) {
    const long long ntiles = (long long)((nx + c[0] - 1) / c[0]) * ((nz + c[1] - 1) / c[1]);
    const int tn = tile_nodes_for(N, nx, nz, row0, c[0], c[1]);
    if (bulk_smem(N, ndof, mixed, tn, nmat, has_kv, mat_elem) > kSmemCap) continue;
    if (ntiles < 2 * 152 && !(c[0] == 1 && c[1] == 1)) continue;  // keep every SM busy
    *TX = c[0];
    *TZ = c[1];
    *tile_nodes = tn;
    return 0;
  }
  // small meshes: the smallest tile that fits
  for (int k = int(sizeof(cand) / sizeof(cand[0])) - 1; k >= 0; --k) {
    const int tn = tile_nodes_for(N, nx, nz, row0, cand[k][0], cand[k][1]);
    if (bulk_smem(N, ndof, mixed, tn, nmat, has_kv, mat_elem) <= kSmemCap) {
      *TX = cand[k][0];
      *TZ = cand[k][1];
      *tile_nodes = tn;
      return 0;
    }
  }
  g_bulk_err = "no tile fits in shared memory";
  return 1;
}

}  // namespace sem2d

// bulk_launch.cu -- NGLL dispatch and tile-shape selection for the bulk kernel.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

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

size_t bulk_smem(int N, int ndof, int mixed, int tn, int on, int nmat, int kv, int me) {
  switch (N) {
    case 5: return bulk_smem_n5(ndof, mixed, tn, on, nmat, kv, me);
    case 6: return bulk_smem_n6(ndof, mixed, tn, on, nmat, kv, me);
    case 9: return bulk_smem_n9(ndof, mixed, tn, on, nmat, kv, me);
    default: return size_t(-1);
  }
}

std::vector<int> tile_rows(int N, int nz, const int *row0, int TZ) {
  std::vector<int> b;
  for (int z = 0; z < nz; z += TZ) b.push_back(z);
  b.push_back(nz);
  auto split = [&](int z) { return z > 0 && z < nz && row0[z] == row0[z - 1] + N; };
  for (size_t k = 1; k + 1 < b.size(); ++k) {
    if (!split(b[k])) continue;
    if (b[k] + 1 < b[k + 1] && !split(b[k] + 1)) b[k] += 1;        // lower tile takes the row
    else if (b[k] - 1 > b[k - 1] && !split(b[k] - 1)) b[k] -= 1;   // upper tile takes the row
    else {                                                          // merge the two tiles
      b.erase(b.begin() + long(k));
      --k;
    }
  }
  return b;
}

void tile_sizes(int N, int nx, const int *row0, int TX, const std::vector<int> &zt, int *tile_nodes,
                int *own_nodes) {
  int best = 0, own = 0;
  const int LX = nx * (N - 1) + 1;
  for (size_t y = 0; y + 1 < zt.size(); ++y) {
    const int ez0 = zt[y], ez1 = zt[y + 1];
    const int hz = (ez0 > 0 && row0[ez0] == row0[ez0 - 1] + (N - 1)) ? 1 : 0;
    const int TH = row0[ez1 - 1] + N - row0[ez0 - hz];
    const int OH = row0[ez1] - row0[ez0];
    for (int ex0 = 0; ex0 < nx; ex0 += TX) {
      const int ex1 = ex0 + TX < nx ? ex0 + TX : nx;
      const int hx = ex0 > 0 ? 1 : 0;
      const int TW = (ex1 - 1) * (N - 1) + N - (ex0 - hx) * (N - 1);
      const int OW = (ex1 == nx ? LX : ex1 * (N - 1)) - ex0 * (N - 1);
      best = std::max(best, TW * TH);
      own = std::max(own, OW * OH);
    }
  }
  *tile_nodes = best;
  *own_nodes = own;
}

int choose_tiles(int N, int ndof, int mixed, int nx, int nz, const int *row0, int nmat, int has_kv,
                 int mat_elem, int *TX, int *TZ) {
  const size_t kSmemCap = 113 * 1024;  // two CTAs per SM
  auto fits = [&](int tx, int tz, size_t cap) {
    int tn, on;
    tile_sizes(N, nx, row0, tx, tile_rows(N, nz, row0, tz), &tn, &on);
    return bulk_smem(N, ndof, mixed, tn, on, nmat, has_kv, mat_elem) <= cap;
  };
  const char *env = std::getenv("SEM2D_TILE");
  if (env) {
    int tx = 0, tz = 0;
    if (std::sscanf(env, "%dx%d", &tx, &tz) == 2 && tx > 0 && tz > 0) {
      if (fits(tx, tz, 227 * 1024)) {
        *TX = tx;
        *TZ = tz;
        return 0;
      }
      g_bulk_err = "SEM2D_TILE does not fit in shared memory";
      return 1;
    }
  }
  static const int cand[][2] = {{16, 8}, {8, 8}, {8, 4}, {4, 4}, {4, 2}, {2, 2}, {1, 1}};
  for (const auto &c : cand) {
    const long long ntiles = (long long)((nx + c[0] - 1) / c[0]) * ((nz + c[1] - 1) / c[1]);
    if (!fits(c[0], c[1], kSmemCap)) continue;
    if (ntiles < 2 * 152 && !(c[0] == 1 && c[1] == 1)) continue;  // keep every SM busy
    *TX = c[0];
    *TZ = c[1];
    return 0;
  }
  for (int k = int(sizeof(cand) / sizeof(cand[0])) - 1; k >= 0; --k)
    if (fits(cand[k][0], cand[k][1], kSmemCap)) {
      *TX = cand[k][0];
      *TZ = cand[k][1];
      return 0;
    }
  g_bulk_err = "no tile fits in shared memory";
  return 1;
}

}  // namespace sem2d

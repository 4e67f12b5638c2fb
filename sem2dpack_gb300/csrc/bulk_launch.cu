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

int occupancy_bulk(const BulkConfig &c) {
  switch (c.N) {
    case 5: return occupancy_bulk_n5(c);
    case 6: return occupancy_bulk_n6(c);
    case 9: return occupancy_bulk_n9(c);
    default: return 0;
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
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 1;
  auto eval = [&](int tx, int tz, double *cost) -> bool {
    const std::vector<int> zt = tile_rows(N, nz, row0, tz);
    BulkConfig c;
    c.N = N;
    c.ndof = ndof;
    c.mixed = mixed;
    c.nmat = nmat;
    c.has_kv = has_kv;
    c.mat_elem = mat_elem;
    tile_sizes(N, nx, row0, tx, zt, &c.tile_nodes, &c.own_nodes);
    if (bulk_smem(N, ndof, mixed, c.tile_nodes, c.own_nodes, nmat, has_kv, mat_elem) > 227 * 1024) return false;
    const int per_sm = occupancy_bulk(c);
    if (per_sm <= 0) return false;
    const long long ntiles = (long long)((nx + tx - 1) / tx) * (long long)(zt.size() - 1);
    const long long waves = (ntiles + (long long)per_sm * nsm - 1) / ((long long)per_sm * nsm);
    // work of the slowest SM: waves x elements computed per tile (with halo)
    const double per_tile = double(std::min(tx, nx) + (nx > tx ? 1 : 0)) * double(std::min(tz, nz) + (nz > tz ? 1 : 0));
    *cost = double(waves) * per_tile + 1e-3 * per_tile;
    return true;
  };
  const char *env = std::getenv("SEM2D_TILE");
  if (env) {
    int tx = 0, tz = 0;
    double cost;
    if (std::sscanf(env, "%dx%d", &tx, &tz) == 2 && tx > 0 && tz > 0) {
      if (eval(tx, tz, &cost)) {
        *TX = tx;
        *TZ = tz;
        return 0;
      }
      g_bulk_err = "SEM2D_TILE does not fit";
      return 1;
    }
  }
  double best = 1e300;
  int bx = 0, bz = 0;
  for (int tx = 1; tx <= 32; ++tx)
    for (int tz = 1; tz <= 16; ++tz) {
      if (tx > nx || tz > nz) continue;
      double cost;
      if (!eval(tx, tz, &cost)) continue;
      if (cost < best) {
        best = cost;
        bx = tx;
        bz = tz;
      }
    }
  if (bx == 0) {
    g_bulk_err = "no tile fits in shared memory";
    return 1;
  }
  *TX = bx;
  *TZ = bz;
  return 0;
}

}  // namespace sem2d

// bulk_launch.cu -- NGLL dispatch and chunk selection for the step kernel.
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
    case 3: return launch_bulk_n3(c);
    case 9: return launch_bulk_n9(c);
    default: g_bulk_err = "NGLL not compiled"; return 1;
  }
}

int configure_bulk(const BulkConfig &c) {
  switch (c.N) {
    case 5: return configure_bulk_n5(c);
    case 6: return configure_bulk_n6(c);
    case 3: return configure_bulk_n3(c);
    case 9: return configure_bulk_n9(c);
    default: g_bulk_err = "NGLL not compiled"; return 1;
  }
}

int occupancy_bulk(const BulkConfig &c) {
  switch (c.N) {
    case 5: return occupancy_bulk_n5(c);
    case 6: return occupancy_bulk_n6(c);
    case 3: return occupancy_bulk_n3(c);
    case 9: return occupancy_bulk_n9(c);
    default: return 0;
  }
}

size_t bulk_smem(int N, int ndof, int mixed, int nplanes) {
  switch (N) {
    case 5: return bulk_smem_n5(ndof, mixed, nplanes);
    case 6: return bulk_smem_n6(ndof, mixed, nplanes);
    case 3: return bulk_smem_n3(ndof, mixed, nplanes);
    case 9: return bulk_smem_n9(ndof, mixed, nplanes);
    default: return size_t(-1);
  }
}

int launch_batch(const BulkConfig &c, const BatchLaunch &b) {
  switch (c.N) {
    case 5: return launch_batch_n5(c, b);
    case 6: return launch_batch_n6(c, b);
    case 3: return launch_batch_n3(c, b);
    case 9: return launch_batch_n9(c, b);
    default: g_bulk_err = "NGLL not compiled"; return 1;
  }
}

size_t params_bytes(int N, int mixed) {
  switch (N) {
    case 5: return params_bytes_n5(mixed);
    case 6: return params_bytes_n6(mixed);
    case 3: return params_bytes_n3(mixed);
    case 9: return params_bytes_n9(mixed);
    default: return 0;
  }
}

int fill_params_block(const BulkConfig &c, void *out) {
  switch (c.N) {
    case 5: fill_params_n5(c, out); return 0;
    case 6: fill_params_n6(c, out); return 0;
    case 3: fill_params_n3(c, out); return 0;
    case 9: fill_params_n9(c, out); return 0;
    default: g_bulk_err = "NGLL not compiled"; return 1;
  }
}

int strip_batch_rows(int N) {
  switch (N) {
    case 5: return strip_batch_rows_n5();
    case 6: return strip_batch_rows_n6();
    case 3: return strip_batch_rows_n3();
    case 9: return strip_batch_rows_n9();
    default: return 1;
  }
}

int strip_width(int N) {
  switch (N) {
    case 5: return strip_width_n5();
    case 6: return strip_width_n6();
    case 3: return strip_width_n3();
    case 9: return strip_width_n9();
    default: return 0;
  }
}

int strip_plane_count(int ndof, int nmat, int mat_elem, int scheme) {
  // displacement, node material, velocity, acceleration (Newmark), inverse mass
  return ndof + (mat_elem == 0 ? nmat : 0) + ndof + (scheme != 0 ? ndof : 0) + 1;
}

std::vector<int> tile_rows(int N, int nz, const int *row0, int TZ) {
  std::vector<int> b;
  for (int z = 0; z < nz; z += TZ) b.push_back(z);
  b.push_back(nz);
  auto split = [&](int z) { return z > 0 && z < nz && row0[z] == row0[z - 1] + N; };
  for (size_t k = 1; k + 1 < b.size(); ++k) {
    if (!split(b[k])) continue;
    if (b[k] + 1 < b[k + 1] && !split(b[k] + 1)) b[k] += 1;        // lower chunk takes the row
    else if (b[k] - 1 > b[k - 1] && !split(b[k] - 1)) b[k] -= 1;   // upper chunk takes the row
    else {                                                          // merge the two chunks
      b.erase(b.begin() + long(k));
      --k;
    }
  }
  return b;
}

int choose_tiles(const BulkConfig &c, const int *row0, int *TZ) {
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0) nsm = 1;
  const int N = c.N, nx = c.nx, nz = c.nz, SW = strip_width(N);
  if (SW <= 0) {
    g_bulk_err = "NGLL not compiled";
    return 1;
  }
  if (bulk_smem(N, c.ndof, c.mixed, c.nplanes) > 227 * 1024) {
    g_bulk_err = "the stage buffers do not fit in shared memory";
    return 1;
  }
  const int per_sm = occupancy_bulk(c);
  if (per_sm <= 0) {
    g_bulk_err = std::string("no resident CTA: ") + g_bulk_err;
    return 1;
  }
  const int R = strip_batch_rows(N);
  const long long nstrips = (nx + SW - 1) / SW;
  auto eval = [&](int tz) {
    const std::vector<int> zt = tile_rows(N, nz, row0, tz);
    const long long nchunks = (long long)zt.size() - 1;
    long long batches = 0;  // the slowest chunk
    for (size_t y = 0; y + 1 < zt.size(); ++y) {
      const int ez0 = zt[y], ez1 = zt[y + 1];
      const int hz = (ez0 > 0 && row0[ez0] == row0[ez0 - 1] + (N - 1)) ? 1 : 0;
      batches = std::max(batches, (long long)((ez1 - ez0 + hz + R - 1) / R));
    }
    const long long ctas = nstrips * nchunks;
    const long long conc = (long long)per_sm * nsm;
    const long long waves = (ctas + conc - 1) / conc;
    // time ~ waves x batches per CTA, plus the pipeline fill of each CTA
    return double(waves) * (double(batches) + 1.0);
  };
  // chunks of at most kMaxChunkRows element rows (two merged around a fault
  // split plus the halo row stay within the kernel's row tables)
  const int tzmax = std::min(nz, kMaxChunkRows);
  const char *env = std::getenv("SEM2D_CHUNK");
  if (env) {
    const int tz = std::atoi(env);
    if (tz > 0) {
      *TZ = std::min(tz, tzmax);
      return 0;
    }
  }
  double best = 1e300;
  int bz = tzmax;
  for (int tz = 1; tz <= tzmax; ++tz) {
    const double cost = eval(tz);
    if (cost <= best + 1e-9) {  // ties: the taller chunk (less halo work)
      best = cost;
      bz = tz;
    }
  }
  *TZ = bz;
  return 0;
}

}  // namespace sem2d

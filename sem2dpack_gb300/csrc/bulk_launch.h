// bulk_launch.h -- host interface of the bulk kernel instantiations.
#pragma once

#include <cuda_runtime.h>

#include <vector>

namespace sem2d {

// Everything the bulk kernel needs, type-erased; the launcher for the
// (NGLL, ndof, precision) of the problem fills the typed parameter block.
struct BulkConfig {
  int N = 0, ndof = 0, mixed = 0;
  int tile_nodes = 0, own_nodes = 0, nmat = 0, has_kv = 0, mat_elem = 0, mat_iso = 0;
  int grid_x = 0, grid_y = 0;
  int LX = 0, LZ = 0, pitch = 0;
  long long plane = 0;
  int nx = 0, nz = 0;
  const int *row0 = nullptr;
  int TX = 0;
  const int *ztile = nullptr;  // device [grid_y+1]
  const double *H = nullptr, *w = nullptr;  // host arrays
  void *Dcur = nullptr, *Dnext = nullptr, *Vcur = nullptr, *Vnext = nullptr;
  void *Acur = nullptr, *Anext = nullptr;
  void *mat[4] = {nullptr, nullptr, nullptr, nullptr};
  void *kveta = nullptr, *rmass = nullptr;
  void *geo[4] = {nullptr, nullptr, nullptr, nullptr};  // xix, etaz, dxdxi, dzdeta
  void *per_rm = nullptr, *per_Ca = nullptr, *per_Cb = nullptr;
  int jf1 = -1, jf2 = -1;
  int has_fault = 0;
  const void *flt = nullptr;  // host FaultParams<real> of the problem's precision
  int nsrc = 0;
  const int *src_I = nullptr, *src_J = nullptr;
  const double *src_amp = nullptr;
  int nt = 0;
  int *step = nullptr;
  unsigned *done = nullptr;
  int rec_nsamp = 0, rec_isamp = 1, rec_nrec = 0, rec_npts = 1;
  char rec_field = 'V';
  const int *rec_tile_start = nullptr, *rec_ids = nullptr, *rec_I = nullptr, *rec_J = nullptr;
  const double *rec_w = nullptr;
  double *sis = nullptr;
  int scheme = 0, kd2 = 0;
  double dt = 0, cv = 0, cpred = 0, cd2 = 0;
  cudaStream_t stream = nullptr;
};

// launches one time step of the bulk kernel; 0 or non-zero on error
int launch_bulk(const BulkConfig &c);
// sets the kernel's dynamic shared-memory limit (once per handle, before
// any launch or stream capture)
int configure_bulk(const BulkConfig &c);
const char *bulk_last_error();

// tile-row boundaries (element rows) of height TZ, moved off split rows
// (row0[b] == row0[b-1] + N) so that both rows of a fault stay in one tile
std::vector<int> tile_rows(int N, int nz, const int *row0, int TZ);
// largest staged tile and largest owned block over all CTAs
void tile_sizes(int N, int nx, const int *row0, int TX, const std::vector<int> &zt,
                int *tile_nodes, int *own_nodes);
// dynamic shared memory (bytes) of one CTA
size_t bulk_smem(int N, int ndof, int mixed, int tile_nodes, int own_nodes, int nmat, int has_kv,
                 int mat_elem);

// picks the tile shape minimising (waves x recomputed elements per tile)
// for the device's SM count and the kernel's occupancy; SEM2D_TILE=TXxTZ
// overrides.  0 on success.
int choose_tiles(int N, int ndof, int mixed, int nx, int nz, const int *row0, int nmat, int has_kv,
                 int mat_elem, int *TX, int *TZ);

// per-NGLL launchers
int launch_bulk_n5(const BulkConfig &c);
int launch_bulk_n6(const BulkConfig &c);
int launch_bulk_n9(const BulkConfig &c);
int configure_bulk_n5(const BulkConfig &c);
int configure_bulk_n6(const BulkConfig &c);
int configure_bulk_n9(const BulkConfig &c);
int occupancy_bulk_n5(const BulkConfig &c);
int occupancy_bulk_n6(const BulkConfig &c);
int occupancy_bulk_n9(const BulkConfig &c);
// resident CTAs per SM for the configuration's shared memory (0 if none)
int occupancy_bulk(const BulkConfig &c);
size_t bulk_smem_n5(int ndof, int mixed, int tile_nodes, int own_nodes, int nmat, int has_kv, int mat_elem);
size_t bulk_smem_n6(int ndof, int mixed, int tile_nodes, int own_nodes, int nmat, int has_kv, int mat_elem);
size_t bulk_smem_n9(int ndof, int mixed, int tile_nodes, int own_nodes, int nmat, int has_kv, int mat_elem);

}  // namespace sem2d

// bulk_launch.h -- host interface of the step-kernel instantiations.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

namespace sem2d {

// largest chunk height the host picks (the kernel holds the row tables of
// up to 256 element rows: two chunks merged around a fault split + a halo)
constexpr int kMaxChunkRows = 120;

// Everything the bulk kernel needs, type-erased; the launcher for the
// (NGLL, ndof, precision) of the problem fills the typed parameter block.
struct BulkConfig {
  int N = 0, ndof = 0, mixed = 0;
  int nplanes = 0, nmat = 0, has_kv = 0, mat_elem = 0, mat_iso = 0;
  int fast = 0;  // isotropic, leapfrog, no Kelvin-Voigt, no 2.5D term
  int grid_x = 0, grid_y = 0;
  int LX = 0, LZ = 0, pitch = 0;
  long long plane = 0;
  int nx = 0, nz = 0;
  const int *row0 = nullptr;
  int TX = 0;                  // element columns per strip (strip_width)
  const int *ztile = nullptr;  // device [grid_y+1] element-row chunk boundaries
  const double *H = nullptr, *w = nullptr;  // host arrays
  void *Dcur = nullptr, *Dnext = nullptr, *Vcur = nullptr, *Vnext = nullptr;
  void *Acur = nullptr, *Anext = nullptr;
  void *Fcur = nullptr, *Fnext = nullptr;  // force state planes (march kernel)
  void *mat[4] = {nullptr, nullptr, nullptr, nullptr};
  void *gen = nullptr;           // general coefficients (mat_elem == kMatGeneral)
  long long gen_stride = 0;
  void *kveta = nullptr, *rmass = nullptr;
  void *geo[4] = {nullptr, nullptr, nullptr, nullptr};  // xix, etaz, dxdxi, dzdeta
  void *per_rm = nullptr, *per_Ca = nullptr, *per_Cb = nullptr;
  void *per_kd = nullptr;  // Stacey P3 forces [c*nslot + slot], or null
  const int *per_dir = nullptr;  // zero-Dirichlet bits c by perimeter slot, or null
  void *perio_f = nullptr;       // raw forces of the periodic columns, or null
  int perio_tb = 0;              // the periodic sides are the bottom and top rows
  void *per_bf = nullptr;        // incident wave and Neumann tractions of this step [c*nslot + slot], or null
  int jf1 = -1, jf2 = -1;
  int has_fault = 0;
  const void *flt = nullptr;  // host FaultParams<real> of the problem's precision
  void *fault_force = nullptr;  // march kernel: forces of the fault rows
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
  double dt = 0, cv = 0, cpred = 0, cd2 = 0, cb = 0;
  double cal = 0, cpa = 0;  // HHT-alpha: 1 - alpha; alpha (1 - gamma) dt
  double width = 0;  // 2.5D seismogenic width, 0 = 2D
  int *error = nullptr;  // device error flag
  int spin_limit = 1 << 22;  // polls of a stage's mbarrier before giving up
  int chunk_shift = 0;   // chunk scheduled first (the fault's)
  int march_warps = 4;   // march kernels: warps per CTA (1, 2 or 4)
  int march_fst = 0;     // march kernels: force state (1) or displacement state (0)
  cudaStream_t stream = nullptr;
};

// a batched step: device array of per-problem parameter blocks for this
// step's buffer parity, the work units and the batch's counters
struct BatchLaunch {
  const void *params = nullptr;  // [nsim] parameter blocks (params_bytes each)
  const void *units = nullptr;   // [nunits] int4 (problem, strip, chunk, strips per row)
  int nunits = 0, grid = 0;
  int *step = nullptr;
  unsigned *done = nullptr;
};

// one reverse step of the adjoint (adjoint_kernel.cuh), type-erased
struct AdjConfig {
  int ndof = 0, mixed = 0, grid_x = 0, grid_y = 0;
  int LX = 0, LZ = 0, pitch = 0;
  long long plane = 0;
  int nx = 0, nz = 0;
  const int *row0 = nullptr, *ztile = nullptr;
  const double *H = nullptr, *w = nullptr;  // host
  void *geo[4] = {nullptr, nullptr, nullptr, nullptr};
  int nmat = 0;
  void *mat[2] = {nullptr, nullptr};
  void *rmass = nullptr, *per_rm = nullptr, *per_Ca = nullptr, *per_Cb = nullptr;
  void *Db = nullptr, *Vb = nullptr, *Dbn = nullptr, *Vbn = nullptr;
  void *d = nullptr, *vprev = nullptr, *a = nullptr;
  void *g_la = nullptr, *g_mu = nullptr, *g_M = nullptr, *g_C = nullptr;
  int nrec = 0, nsamp = 0, isamp = 1;
  char field = 'V';
  const int *rec_I = nullptr, *rec_J = nullptr;
  const double *resid = nullptr;
  double dt = 0;
  int kd2 = 0, it = 0;
  int *error = nullptr;
  cudaStream_t stream = nullptr;
};
int configure_adjoint(const AdjConfig &c);
int launch_adjoint(const AdjConfig &c);
// acc64[k] += (double)part[k]; part[k] = 0, for n values
int launch_fold(void *part, double *acc64, long long n, int mixed, cudaStream_t s);
// node gradients from the accumulated terms (see adjoint.cu)
struct ChainConfig {
  int ndof = 0, mixed = 0, LX = 0, LZ = 0, pitch = 0;
  double dt = 0;
  const void *rho = nullptr, *la = nullptr, *mu = nullptr, *rmass = nullptr;
  const void *per_rm = nullptr, *per_Ca = nullptr, *per_Cb = nullptr;
  const double *g_la = nullptr, *g_mu = nullptr, *g_M = nullptr, *g_C = nullptr;
  double *grad_rho = nullptr, *grad_vp = nullptr, *grad_vs = nullptr;  // lattice planes
  cudaStream_t stream = nullptr;
};
int launch_chain(const ChainConfig &c);

// launches one time step of the step kernel; 0 or non-zero on error
int launch_bulk(const BulkConfig &c);
// launches one time step of a batch (c describes the shared kernel shape:
// N, ndof, precision, material layout, planes, fast path, H, w, stream)
int launch_batch(const BulkConfig &c, const BatchLaunch &b);
// size of one parameter block and the block of a problem
size_t params_bytes(int N, int mixed);
int fill_params_block(const BulkConfig &c, void *out);
// sets the kernel's dynamic shared-memory limit (once per handle, before
// any launch or stream capture)
int configure_bulk(const BulkConfig &c);
const char *bulk_last_error();
// the message sem2d_gpu_last_error(NULL) returns
void set_library_error(const std::string &msg);

// element columns per strip and element rows per batch for NGLL N
int strip_width(int N);
int strip_batch_rows(int N);
// lattice planes staged per batch
int strip_plane_count(int ndof, int nmat, int mat_elem, int scheme);

// chunk boundaries (element rows) of height TZ, moved off split rows
// (row0[b] == row0[b-1] + N) so that both rows of a fault stay in one chunk
std::vector<int> tile_rows(int N, int nz, const int *row0, int TZ);
// dynamic shared memory (bytes) of one CTA
size_t bulk_smem(int N, int ndof, int mixed, int nplanes);

// picks the chunk height minimising (waves x batches per chunk) for the
// device's SM count and the kernel's occupancy; SEM2D_CHUNK=TZ overrides.
// 0 on success.
int choose_tiles(const BulkConfig &c, const int *row0, int *TZ);

// per-NGLL launchers
int launch_bulk_n5(const BulkConfig &c);
int launch_bulk_n6(const BulkConfig &c);
int launch_bulk_n9(const BulkConfig &c);
int launch_bulk_n3(const BulkConfig &c);
int configure_bulk_n5(const BulkConfig &c);
int configure_bulk_n6(const BulkConfig &c);
int configure_bulk_n9(const BulkConfig &c);
int configure_bulk_n3(const BulkConfig &c);
int occupancy_bulk_n5(const BulkConfig &c);
int occupancy_bulk_n6(const BulkConfig &c);
int occupancy_bulk_n9(const BulkConfig &c);
int occupancy_bulk_n3(const BulkConfig &c);
// resident CTAs per SM for the configuration's shared memory (0 if none)
int occupancy_bulk(const BulkConfig &c);
size_t bulk_smem_n5(int ndof, int mixed, int nplanes);
size_t bulk_smem_n6(int ndof, int mixed, int nplanes);
size_t bulk_smem_n9(int ndof, int mixed, int nplanes);
size_t bulk_smem_n3(int ndof, int mixed, int nplanes);
int strip_width_n5();
int strip_width_n6();
int strip_width_n9();
int strip_width_n3();
int strip_batch_rows_n5();
int strip_batch_rows_n6();
int strip_batch_rows_n9();
int strip_batch_rows_n3();
int launch_batch_n5(const BulkConfig &c, const BatchLaunch &b);
int launch_batch_n6(const BulkConfig &c, const BatchLaunch &b);
int launch_batch_n9(const BulkConfig &c, const BatchLaunch &b);
int launch_batch_n3(const BulkConfig &c, const BatchLaunch &b);
// The FP32 NGLL=5 fast path with one element per thread (march_kernel.cuh).
// Units are MarchUnit records {problem, strip, z0, z1, rec0, rec1}.
constexpr int kMarchColsHost = 31;   // element columns owned by one unit
constexpr int kMarchUnitInts = 6;    // ints per unit record
constexpr int kMarchWarpsHost = 4;   // warps per CTA of the march kernels
struct MarchLaunch {
  const void *units = nullptr;  // [nunits] unit records
  int nunits = 0;
  const void *sims = nullptr;   // [nsim] BulkParams<float, 5> (batch launches)
  int *step = nullptr;          // batch launches
  unsigned *done = nullptr;
};
// true when the march kernel covers the configuration
bool march_supported(const BulkConfig &c);
int launch_march(const BulkConfig &c, const MarchLaunch &m);
int launch_march_batch(const BulkConfig &c, const MarchLaunch &m);
// the fault node pairs of a march step (one thread per pair, after the step)
int launch_march_fault(const BulkConfig &c);
// the fault-side units of a march step and the fault node pairs in one
// launch (a CTA per strip; nrows fault-side units per strip, at most 4)
int launch_march_fault_side(const BulkConfig &c, const MarchLaunch &m, int nstrips, int nrows);
// one reverse step of the adjoint with the march kernels (FP32, NGLL=5,
// isotropic node material; march_adjoint.cuh): `bc` is the forward step's
// configuration with (lambda^n, w^{n+1}) as (Dcur, Vcur) and (lambda^{n-1},
// w^n) as (Dnext, Vnext), sources and receivers off; `c` the rest
struct MarchAdjConfig {
  const void *a = nullptr, *vprev = nullptr;  // forward a^n, v^{n-1}
  const void *d = nullptr;                    // forward d^n
  void *g_la = nullptr, *g_mu = nullptr, *g_M = nullptr, *g_C = nullptr;
  int nrec = 0, nsamp = 0, isamp = 1;
  char field = 'V';
  const int *rec_I = nullptr, *rec_J = nullptr;
  const double *resid = nullptr;
  int it = 0;
  const void *units = nullptr;
  int nunits = 0;
};
// reverse step c.it; *launches receives the number of kernels launched
int launch_march_adjoint(const BulkConfig &bc, const MarchAdjConfig &c, int *launches);
// lambda^{nt} from the velocity misfit of the last step (into Dcur of bc)
int launch_march_adjoint_seed(const BulkConfig &bc, const MarchAdjConfig &c, int *launches);
// resident warps per SM of the march kernel for the configuration; also
// sets the kernels' shared-memory limit (call before any launch or capture)
int march_warps_per_sm(const BulkConfig &c);

size_t params_bytes_n5(int mixed);
size_t params_bytes_n6(int mixed);
size_t params_bytes_n9(int mixed);
size_t params_bytes_n3(int mixed);
void fill_params_n5(const BulkConfig &c, void *out);
void fill_params_n6(const BulkConfig &c, void *out);
void fill_params_n9(const BulkConfig &c, void *out);
void fill_params_n3(const BulkConfig &c, void *out);

}  // namespace sem2d

// sem2d_gpu.cu -- C-ABI of include/sem2d_gpu.h: upload, layout, launches.
//
// create():  validates the descriptor, recovers the structured GLL lattice
//            behind the reference's global numbering (ibool + coord), picks
//            the material layout, uploads everything.
// step():    per time step launches (1) the fused bulk kernel, (2) the fault
//            kernel -- or a counter bump when there is no fault -- and (3) the
//            receiver kernel; runs of 2*kGraphPairs steps are captured once in
//            a CUDA graph and replayed.
// get_*():   synchronise and map results back to the reference numbering.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/sem2d_gpu.h"
#include "../../include/sem2d_host.h"
#include "bulk_launch.h"
#include "fault_kernel.cuh"
#include "sem2d_common.cuh"
#include "stf.cuh"

using namespace sem2d;

namespace {

std::string g_create_err;
constexpr int kGraphPairs = 8;  // a captured graph covers 16 steps

}  // namespace

void sem2d::set_library_error(const std::string &msg) { g_create_err = msg; }

struct FaultScalars {
  double coefA2V = 0, coefA2D = 0, normal_V = 0, normal_T = 1, normal_L = 1;
  int opening = 0, swf_kind = 1, swf_healing = 0, rsf_kind = 1, normal_kind = 1;
  int oit = 0, oitd = 1, oix1 = 1, oixd = 1;
  int twf_kind = 0;
  double twf_mus = 0.6, twf_mud = 0.5, twf_mu0 = 0.6, twf_X = 0, twf_Z = 0, twf_V = 1e3, twf_L = 1,
         twf_T = 0, twf_Dc = 0;
};

struct sem2d_handle {
  // problem
  std::vector<double> H, w;          // GLL derivative matrix and weights
  int kd2 = 0;
  double width = 0;  // 2.5D seismogenic width, 0 = 2D
  FaultScalars fs;
  int N = 0, ndof = 0, nelem = 0, npoin = 0, nt = 0, mixed = 0, scheme = 0;  // scheme 2: HHT-alpha
  double dt = 0, beta = 0, gamma = 0.5, alpha = 1.0;
  int nx = 0, nz = 0, LX = 0, LZ = 0, pitch = 0;
  long long plane = 0;
  std::vector<int> row0;             // [nz+1]
  std::vector<long long> glob2lat;   // global node -> J*pitch + I
  long long *d_glob2lat = nullptr;   // the same on the device (the adjoint's output), when needed
  std::vector<int> elem_ex, elem_ez; // reference element -> structured position
  int TX = 8, TZ = 8, nplanes = 0, nmat = 0, mat_iso = 0, mat_elem = 0, has_kv = 0;
  std::vector<int> ztile;            // chunk boundaries (element rows)
  int fault_chunk = 0;               // chunk holding the fault rows
  int *d_ztile = nullptr;
  bool keep_accel = false;
  // device memory
  cudaStream_t stream = nullptr;
  std::vector<void *> allocs;
  void *D[2] = {nullptr, nullptr}, *V[2] = {nullptr, nullptr}, *A[2] = {nullptr, nullptr};
  void *mat[4] = {nullptr, nullptr, nullptr, nullptr};
  void *kveta = nullptr, *rmass = nullptr, *geo[4] = {nullptr, nullptr, nullptr, nullptr};
  void *per_rm = nullptr, *per_Ca = nullptr, *per_Cb = nullptr;
  // Stacey P3 terms grouped by perimeter slot, and their forces
  int st_nslot = 0, st_nterm = 0;
  int *d_st_slot = nullptr, *d_st_ptr = nullptr, *d_st_k = nullptr, *d_st_lat = nullptr;
  void *d_st_K = nullptr, *d_st_H = nullptr, *per_kd = nullptr;
  // zero-Dirichlet force components: bits c of a perimeter slot, and bits
  // (side*2 + c) of a fault node when the zero follows the fault
  int ndir = 0;
  int *per_dir = nullptr;
  unsigned char *d_fdir = nullptr;
  // periodic columns I = 0 and LX-1: raw forces left by the step kernel
  int nperio = 0, perio_tb = 0;  // perio_tb: the rows J = 0 and LZ-1 instead
  // a grid that is not flat: general coefficients a_k per element GLL point
  int general = 0;
  void *gen = nullptr;
  void *perio_f = nullptr;
  // perimeter forces with their own time functions: the incident plane
  // wave and the time-dependent Neumann tractions (bf.W null: none),
  // evaluated into per_bf [c*nslot + slot] before every step
  BoundaryForces bf;
  void *per_bf = nullptr;
  int *d_row0 = nullptr, *d_step = nullptr, *d_error = nullptr;
  unsigned *d_done = nullptr;
  // sources
  int nsrc = 0;
  int *src_I = nullptr, *src_J = nullptr;
  double *src_amp = nullptr;
  // receivers
  int nrec = 0, rec_isamp = 1, rec_nsamp = 0, rec_npts = 1;
  char rec_field = 'V';
  bool rec_separate = false;          // interpolated V/A: own kernel after the step
  int *rec_lat = nullptr;
  double *rec_w = nullptr, *sis = nullptr;
  int *rec_tile_start = nullptr, *rec_ids = nullptr, *rec_I = nullptr, *rec_J = nullptr;
  // fault
  int nflt = 0, two = 0, jf1 = -1, jf2 = -1, onx = 0, fnsamp = 0, friction = 0;
  bool potency = false;              // fault potency recorded every step
  std::vector<double> h_fault_init;  // V0, theta for reset
  double *fd[64] = {nullptr};        // fault arrays, see enum below
  // time stepping
  int cur = 0;       // ping-pong index of the current displacement predictor
  int steps = 0;     // steps queued
  // run-time checks: polls of an mbarrier before a step gives up
  // (SEM2D_SPIN_LIMIT), Newton iteration cap, and the max|v|, max|d|
  // watchdog every info_every steps (<= 0: off) into d_info
  int spin_limit = 1 << 22, nr_maxit = 200, info_every = 100;
  double *d_info = nullptr;  // [2]: max|v|, max|d| of the last check
  int info_step = 0;         // step of the last check
  long long launches = 0;
  cudaGraphExec_t graph_exec = nullptr;
  std::string err;
  // a batch of independent problems advanced by one launch per step: the
  // members hold the problems, the batch holds their parameter blocks (by
  // buffer parity), the work units and the step counters
  std::vector<sem2d_handle *> subs;
  sem2d_handle *owner = nullptr;    // the batch a member belongs to
  bool owns_stream = true;
  void *d_params[2] = {nullptr, nullptr};
  void *d_watch[2] = {nullptr, nullptr};  // batch: (V, D, n) of every member by buffer parity
  void *d_units = nullptr;
  // the one-element-per-thread kernel (FP32, NGLL = 5 fast path): work
  // units (strip, chunk) and the receivers each unit samples
  bool march = false;
  int march_warps = 4;  // warps per CTA (SEM2D_MARCH_WARPS)
  int march_fst = 0;    // force state (problems with a fault; SEM2D_FORCE_STATE=0 keeps the displacement state)
  // a time function other than Ricker drives the sources or the boundary:
  // its net impulse can leave a static displacement, which FP32 does not
  // resolve against the dynamic one (the force state is used then too)
  bool static_load = false;
  // the strip kernel's force state (mixed precision, leapfrog, no
  // Kelvin-Voigt, with a fault or a static load): F planes as for the march
  // kernel
  int strip_fst = 0;
  void *F[2] = {nullptr, nullptr};  // force state planes, ping-pong like D and V
  int tune_source = 0;  // launch shape: 0 analytic, 1 timed on the first run, 2 from the tuning cache
  int tune_pending = 0;  // the shape is timed on the next run of at least kTuneSteps steps
  int march_cz = 0, march_nunits = 0;
  void *d_march_units = nullptr;
  int *d_march_rec = nullptr;
  std::vector<int> march_units_host;
  std::vector<int> march_rec_ex, march_rec_ez;  // element of every receiver (units are rebuilt by the tuner)
  float *d_fault_force = nullptr;
  // with a fault: the first march_fault_units units are the fault chunk's,
  // launched as their own kernel with their own step/done counters; the
  // fault chunk and the fault kernel run on fstream, overlapping the next
  // step's other units (march_overlap)
  int march_fault_units = 0;
  // slip/time weakening: the fault-side units and the fault node pairs in
  // one launch (a CTA per strip); rate-and-state keeps the separate fault
  // kernel, whose Newton solves want one warp per SM
  bool march_fused = false;
  int march_nstrips = 0, march_nfch = 0;
  int *d_step_c = nullptr;
  unsigned *d_done_c = nullptr;
  bool march_overlap = false;
  cudaStream_t fstream = nullptr;
  cudaEvent_t ev_m[2] = {nullptr, nullptr}, ev_c[2] = {nullptr, nullptr}, ev_f = nullptr;   // forces of the fault rows, finished by the fault kernel
  int nunits = 0, batch_grid = 0;
  bool batch_open = false;          // members may still be added
  // gradient workflow (sem2d_gpu_adjoint)
  int adjoint = 0;
  void *rho_plane = nullptr;        // density at the nodes
  int ckpt_every = 0;               // forward states kept every ckpt_every steps
  std::vector<void *> ckpt;         // [slot] D then V (ndof planes each)
  int ckpt_saved = -1;              // last slot written
};

namespace {

enum FaultArr {
  F_D64, F_V64, F_A64, F_RM, F_N1, F_B, F_INVM1, F_INVM2, F_Z, F_T0, F_COH,
  F_SWF_DC, F_SWF_MUS, F_SWF_MUD, F_SWF_P, F_SWF_ALPHA,
  F_RSF_DC, F_RSF_MUS, F_RSF_A, F_RSF_B, F_RSF_VSTAR, F_RSF_VC, F_RSF_TC, F_RSF_COEFT,
  F_D, F_V, F_T, F_TSTICK, F_MU, F_THETA, F_SIGMA, F_SERIES, F_XZ, F_POT, F_POTSERIES, F_COUNT
};

#define CK(call)                                                                       \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess) {                                                           \
      h->err = std::string(#call) + ": " + cudaGetErrorString(e_);                     \
      return SEM2D_E_CUDA;                                                             \
    }                                                                                  \
  } while (0)

// the common case the step kernel compiles separately: isotropic material,
// leapfrog, no Kelvin-Voigt, no 2.5D term
bool fast_path(const sem2d_handle *h) {
  return h->mat_iso && h->scheme == 0 && !h->has_kv && !(h->width > 0);
}

int set_err(sem2d_handle *h, int code, const std::string &m) {
  h->err = m;
  return code;
}

template <typename T>
int dalloc(sem2d_handle *h, T **out, size_t n, bool zero = true) {
  void *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T));
  if (e != cudaSuccess) return set_err(h, SEM2D_E_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  h->allocs.push_back(p);
  if (zero) {
    e = cudaMemset(p, 0, n * sizeof(T));
    if (e != cudaSuccess) return set_err(h, SEM2D_E_CUDA, cudaGetErrorString(e));
  }
  *out = static_cast<T *>(p);
  return SEM2D_OK;
}

template <typename T>
int dupload(sem2d_handle *h, T **out, const std::vector<T> &v) {
  int st = dalloc(h, out, v.size(), false);
  if (st) return st;
  if (!v.empty()) CK(cudaMemcpy(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return SEM2D_OK;
}

// real-typed upload of a double vector
int upload_real(sem2d_handle *h, void **out, const std::vector<double> &v) {
  if (h->mixed) {
    std::vector<float> f(v.begin(), v.end());
    float *p;
    int st = dupload(h, &p, f);
    *out = p;
    return st;
  }
  double *p;
  int st = dupload(h, &p, v);
  *out = p;
  return st;
}

double ricker(double t, double f0, double t0, double ampli) {
  const double kPi = 3.141592653589793;
  double arg = kPi * f0 * (t - t0);
  arg = arg * arg;
  return -((ampli * (1.0 - 2.0 * arg)) * std::exp(-arg));
}

// ---------------------------------------------------------------------
// Recover the lattice: element columns/rows from the element corner
// coordinates, shared or split rows from ibool.
// Element positions on a structured grid that is not flat, from the
// connectivity: the right neighbour shares the right edge's corner nodes,
// the upper one the top edge's, or, across a split (fault) row, has its
// bottom corners at the same coordinates.
int topology_positions(sem2d_handle *h, const sem2d_problem_desc *d, std::vector<int> &grid) {
  const int N = d->ngll, ne = d->nelem, np = d->npoin;
  auto ib = [&](int i, int j, int e) { return d->ibool[i + N * (j + (size_t)N * e)] - 1; };
  std::vector<int> by00(np, -1);
  for (int e = 0; e < ne; ++e) {
    const int a = ib(0, 0, e);
    if (by00[a] >= 0) return set_err(h, SEM2D_E_UNSUPPORTED, "two elements share a lower-left corner");
    by00[a] = e;
  }
  auto same_xz = [&](int a, int b) {
    return d->coord[2 * (size_t)a] == d->coord[2 * (size_t)b] && d->coord[2 * (size_t)a + 1] == d->coord[2 * (size_t)b + 1];
  };
  std::vector<std::pair<std::pair<double, double>, int>> c00;
  for (int e = 0; e < ne; ++e) {
    const int a = ib(0, 0, e);
    c00.push_back({{d->coord[2 * (size_t)a], d->coord[2 * (size_t)a + 1]}, e});
  }
  std::sort(c00.begin(), c00.end());
  std::vector<int> right(ne, -1), up(ne, -1), has_left(ne, 0), has_below(ne, 0);
  for (int e = 0; e < ne; ++e) {
    const int r = by00[ib(N - 1, 0, e)];
    if (r >= 0 && ib(0, N - 1, r) == ib(N - 1, N - 1, e)) right[e] = r;
    int u = by00[ib(0, N - 1, e)];
    if (u >= 0 && ib(N - 1, 0, u) != ib(N - 1, N - 1, e)) u = -1;
    if (u < 0) {  // a split row: the element whose bottom corners sit on this top edge
      const int a = ib(0, N - 1, e);
      const std::pair<double, double> key{d->coord[2 * (size_t)a], d->coord[2 * (size_t)a + 1]};
      auto it = std::lower_bound(c00.begin(), c00.end(), std::make_pair(key, -1));
      for (; it != c00.end() && it->first == key; ++it)
        if (it->second != e && same_xz(ib(N - 1, 0, it->second), ib(N - 1, N - 1, e))) u = it->second;
    }
    up[e] = u;
  }
  for (int e = 0; e < ne; ++e) {
    if (right[e] >= 0) has_left[right[e]]++;
    if (up[e] >= 0) has_below[up[e]]++;
  }
  int origin = -1;
  for (int e = 0; e < ne; ++e)
    if (!has_left[e] && !has_below[e]) {
      if (origin >= 0) return set_err(h, SEM2D_E_UNSUPPORTED, "mesh is not a structured grid of elements");
      origin = e;
    }
  if (origin < 0) return set_err(h, SEM2D_E_UNSUPPORTED, "mesh is not a structured grid of elements");
  int nx = 0;
  for (int e = origin; e >= 0; e = right[e]) ++nx;
  if (nx <= 0 || ne % nx) return set_err(h, SEM2D_E_UNSUPPORTED, "mesh is not a structured grid of elements");
  const int nz = ne / nx;
  h->nx = nx;
  h->nz = nz;
  h->elem_ex.assign(ne, -1);
  h->elem_ez.assign(ne, -1);
  grid.assign((size_t)nx * nz, -1);
  int start = origin;
  for (int ez = 0; ez < nz; ++ez) {
    if (start < 0) return set_err(h, SEM2D_E_UNSUPPORTED, "mesh is not a structured grid of elements");
    int e = start;
    for (int ex = 0; ex < nx; ++ex) {
      if (e < 0 || h->elem_ex[e] >= 0) return set_err(h, SEM2D_E_UNSUPPORTED, "mesh is not a structured grid of elements");
      h->elem_ex[e] = ex;
      h->elem_ez[e] = ez;
      grid[(size_t)ez * nx + ex] = e;
      e = right[e];
    }
    if (e >= 0) return set_err(h, SEM2D_E_UNSUPPORTED, "element rows of unequal length");
    start = up[start];
  }
  return SEM2D_OK;
}

int detect_lattice(sem2d_handle *h, const sem2d_problem_desc *d) {
  const int N = d->ngll, ne = d->nelem;
  auto ib = [&](int i, int j, int e) { return d->ibool[i + N * (j + (size_t)N * e)] - 1; };
  std::vector<double> x0(ne), z0(ne), x1(ne), z1(ne);
  for (int e = 0; e < ne; ++e) {
    const int a = ib(0, 0, e), b = ib(N - 1, N - 1, e);
    if (a < 0 || a >= d->npoin || b < 0 || b >= d->npoin)
      return set_err(h, SEM2D_E_ARG, "ibool out of range");
    x0[e] = d->coord[2 * (size_t)a];
    z0[e] = d->coord[2 * (size_t)a + 1];
    x1[e] = d->coord[2 * (size_t)b];
    z1[e] = d->coord[2 * (size_t)b + 1];
  }
  std::vector<int> grid;
  if (d->xjaci) {
    if (!d->dvol) return set_err(h, SEM2D_E_ARG, "xjaci without dvol");
    int st = topology_positions(h, d, grid);
    if (st) return st;
  } else {
  std::vector<double> xs(x0), zs(z0);
  std::sort(xs.begin(), xs.end());
  xs.erase(std::unique(xs.begin(), xs.end()), xs.end());
  std::sort(zs.begin(), zs.end());
  zs.erase(std::unique(zs.begin(), zs.end()), zs.end());
  const int nx = int(xs.size()), nz = int(zs.size());
  if ((long long)nx * nz != ne)
    return set_err(h, SEM2D_E_UNSUPPORTED, "mesh is not a structured rectilinear grid of elements");
  h->nx = nx;
  h->nz = nz;
  h->elem_ex.resize(ne);
  h->elem_ez.resize(ne);
  grid.assign((size_t)nx * nz, -1);
  for (int e = 0; e < ne; ++e) {
    const int ex = int(std::lower_bound(xs.begin(), xs.end(), x0[e]) - xs.begin());
    const int ez = int(std::lower_bound(zs.begin(), zs.end(), z0[e]) - zs.begin());
    if (grid[(size_t)ez * nx + ex] >= 0)
      return set_err(h, SEM2D_E_UNSUPPORTED, "two elements at one lattice position");
    grid[(size_t)ez * nx + ex] = e;
    h->elem_ex[e] = ex;
    h->elem_ez[e] = ez;
  }
  }
  const int nx = h->nx, nz = h->nz;
  // rows: shared (no fault) or split (fault) between consecutive element rows
  h->row0.assign(nz + 1, 0);
  for (int ez = 1; ez < nz; ++ez) {
    int shared = -1;
    for (int ex = 0; ex < nx; ++ex) {
      const int lo = grid[(size_t)(ez - 1) * nx + ex], up = grid[(size_t)ez * nx + ex];
      const int s = ib(0, N - 1, lo) == ib(0, 0, up) ? 1 : 0;
      if (shared < 0) shared = s;
      if (s != shared) return set_err(h, SEM2D_E_UNSUPPORTED, "partially split element row");
    }
    h->row0[ez] = h->row0[ez - 1] + (shared ? N - 1 : N);
  }
  for (int ez = 0; ez < nz; ++ez)
    for (int ex = 1; ex < nx; ++ex)
      if (ib(N - 1, 0, grid[(size_t)ez * nx + ex - 1]) != ib(0, 0, grid[(size_t)ez * nx + ex]))
        return set_err(h, SEM2D_E_UNSUPPORTED, "vertically split element columns are not supported");
  h->LX = nx * (N - 1) + 1;
  h->LZ = h->row0[nz - 1] + N;
  h->row0[nz] = h->LZ;
  h->pitch = (h->LX + 7) / 8 * 8;
  h->plane = (long long)h->pitch * h->LZ;
  if ((long long)h->LX * h->LZ != d->npoin)
    return set_err(h, SEM2D_E_UNSUPPORTED, "node count does not match a structured lattice");
  h->glob2lat.assign(d->npoin, -1);
  for (int e = 0; e < ne; ++e)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        const long long L = (long long)(h->row0[h->elem_ez[e]] + j) * h->pitch + h->elem_ex[e] * (N - 1) + i;
        long long &slot = h->glob2lat[ib(i, j, e)];
        if (slot >= 0 && slot != L) return set_err(h, SEM2D_E_UNSUPPORTED, "inconsistent ibool on the lattice");
        slot = L;
      }
  for (int p = 0; p < d->npoin; ++p)
    if (h->glob2lat[p] < 0) return set_err(h, SEM2D_E_ARG, "global node not referenced by ibool");
  if (d->xjaci) {  // the element geometry is in the general coefficients
    h->general = 1;
    int st;
    if ((st = upload_real(h, &h->geo[0], std::vector<double>(nx, 1.0))) ||
        (st = upload_real(h, &h->geo[1], std::vector<double>(nz, 1.0))) ||
        (st = upload_real(h, &h->geo[2], std::vector<double>(nx, 1.0))) ||
        (st = upload_real(h, &h->geo[3], std::vector<double>(nz, 1.0))))
      return st;
    return SEM2D_OK;
  }
  // rectilinear geometry: one width per column, one height per row
  std::vector<double> dxdxi(nx), dzdeta(nz);
  for (int e = 0; e < ne; ++e) {
    const double ddx = 0.5 * (x1[e] - x0[e]), ddz = 0.5 * (z1[e] - z0[e]);
    if (!(ddx > 0) || !(ddz > 0)) return set_err(h, SEM2D_E_ARG, "degenerate element");
    dxdxi[h->elem_ex[e]] = ddx;
    dzdeta[h->elem_ez[e]] = ddz;
  }
  for (int e = 0; e < ne; ++e)
    if (0.5 * (x1[e] - x0[e]) != dxdxi[h->elem_ex[e]] || 0.5 * (z1[e] - z0[e]) != dzdeta[h->elem_ez[e]])
      return set_err(h, SEM2D_E_UNSUPPORTED, "elements are not rectilinear");
  std::vector<double> xix(nx), etaz(nz);
  for (int i = 0; i < nx; ++i) xix[i] = 1.0 / dxdxi[i];
  for (int j = 0; j < nz; ++j) etaz[j] = 1.0 / dzdeta[j];
  int st;
  if ((st = upload_real(h, &h->geo[0], xix)) || (st = upload_real(h, &h->geo[1], etaz)) ||
      (st = upload_real(h, &h->geo[2], dxdxi)) || (st = upload_real(h, &h->geo[3], dzdeta)))
    return st;
  return SEM2D_OK;
}

int upload_kveta(sem2d_handle *h, const sem2d_problem_desc *d) {
  const int N = d->ngll, NN = N * N, ne = d->nelem;
  if (!d->kv_eta) return SEM2D_OK;
  h->has_kv = 1;
  std::vector<double> el((size_t)NN * ne);
  for (int e = 0; e < ne; ++e) {
    const size_t eo = ((size_t)h->elem_ez[e] * h->nx + h->elem_ex[e]) * NN;
    for (int q = 0; q < NN; ++q) el[eo + q] = d->kv_eta[q + (size_t)NN * e];
  }
  return upload_real(h, &h->kveta, el);
}

// MAT_ELAST_init_a on a grid that is not flat (mat_elastic.f90:290-360):
// a_k = -dvol (moduli x products of the inverse Jacobian), nelast 10 in
// P-SV and 3 in SH, in the lattice element order [k][element][i + N j]
int upload_general(sem2d_handle *h, const sem2d_problem_desc *d) {
  const int N = d->ngll, NN = N * N, ne = d->nelem, na = d->ndof == 1 ? 3 : 10;
  const size_t npt = (size_t)NN * ne;
  if (d->width > 0) return set_err(h, SEM2D_E_UNSUPPORTED, "the 2.5D term on a grid that is not flat");
  if (d->adjoint) return set_err(h, SEM2D_E_UNSUPPORTED, "the gradient workflow on a grid that is not flat");
  std::vector<double> A((size_t)na * npt);
  for (int e = 0; e < ne; ++e) {
    const size_t eo = ((size_t)h->elem_ez[e] * h->nx + h->elem_ex[e]) * NN;
    for (int q = 0; q < NN; ++q) {
      const size_t p = q + (size_t)NN * e;
      const double *X = d->xjaci + 4 * p;
      const double DxiDx = X[0], DetaDx = X[1], DxiDz = X[2], DetaDz = X[3], w = d->dvol[p];
      const double Kx = d->Kx[p], Kz = d->Kz[p], la = d->la[p], mu = d->mu[p], mux = d->mux[p], muz = mu;
      double a[10];
      if (na == 3) {
        a[0] = (mux * DxiDx) * DxiDx + (muz * DxiDz) * DxiDz;
        a[1] = (mux * DetaDx) * DetaDx + (muz * DetaDz) * DetaDz;
        a[2] = (mux * DxiDx) * DetaDx + (muz * DxiDz) * DetaDz;
      } else {
        a[0] = (Kx * DxiDx) * DxiDx + (mu * DxiDz) * DxiDz;
        a[1] = (la * DxiDx) * DetaDz + (mu * DxiDz) * DetaDx;
        a[2] = (Kz * DetaDz) * DetaDz + (mu * DetaDx) * DetaDx;
        a[3] = (Kx * DetaDx) * DetaDx + (mu * DetaDz) * DetaDz;
        a[4] = (la * DxiDz) * DetaDx + (mu * DxiDx) * DetaDz;
        a[5] = (Kz * DxiDz) * DxiDz + (mu * DxiDx) * DxiDx;
        a[6] = (Kx * DxiDx) * DetaDx + (mu * DxiDz) * DetaDz;
        a[7] = ((la + mu) * DxiDx) * DxiDz;
        a[8] = ((la + mu) * DetaDx) * DetaDz;
        a[9] = (Kz * DxiDz) * DetaDz + (mu * DxiDx) * DetaDx;
      }
      for (int k = 0; k < na; ++k) A[(size_t)k * npt + eo + q] = -(w * a[k]);
    }
  }
  h->mat_elem = kMatGeneral;
  h->nmat = 0;
  h->mat_iso = 1;
  int st = upload_real(h, &h->gen, A);
  if (st) return st;
  return upload_kveta(h, d);
}

int upload_material(sem2d_handle *h, const sem2d_problem_desc *d) {
  if (h->general) return upload_general(h, d);
  const int N = d->ngll, NN = N * N, ne = d->nelem;
  const size_t npt = (size_t)NN * ne;
  // isotropic?  Kx = Kz = la + 2 mu and mux = mu everywhere
  bool iso = true;
  for (size_t q = 0; q < npt && iso; ++q)
    iso = d->Kx[q] == d->la[q] + 2.0 * d->mu[q] && d->Kz[q] == d->Kx[q] && d->mux[q] == d->mu[q];
  std::vector<const double *> src;
  if (d->ndof == 2) src = iso ? std::vector<const double *>{d->la, d->mu}
                              : std::vector<const double *>{d->Kx, d->Kz, d->la, d->mu};
  else src = iso ? std::vector<const double *>{d->mu} : std::vector<const double *>{d->mu, d->mux};
  h->nmat = int(src.size());
  h->mat_iso = iso;
  if (d->width > 0 && !iso)
    return set_err(h, SEM2D_E_UNSUPPORTED, "the 2.5D term needs an isotropic material");
  if (d->adjoint) {
    if (!d->rho) return set_err(h, SEM2D_E_ARG, "the gradient workflow needs the density (rho)");
    if (!iso) return set_err(h, SEM2D_E_UNSUPPORTED, "the gradient workflow needs an isotropic material");
  }
  // one value per element when every element is homogeneous (the
  // reference then shares one coefficient set per tag, mat_gen.f90:358-361)
  bool elem_const = !d->adjoint;
  for (int e = 0; e < ne && elem_const; ++e)
    for (size_t m = 0; m < src.size() && elem_const; ++m) {
      const double *v = src[m] + (size_t)NN * e;
      for (int q = 1; q < NN; ++q)
        if (v[q] != v[0]) {
          elem_const = false;
          break;
        }
    }
  if (elem_const) {
    h->mat_elem = kMatElement;
    for (size_t m = 0; m < src.size(); ++m) {
      std::vector<double> el((size_t)ne);
      for (int e = 0; e < ne; ++e) el[(size_t)h->elem_ez[e] * h->nx + h->elem_ex[e]] = src[m][(size_t)NN * e];
      int st = upload_real(h, &h->mat[m], el);
      if (st) return st;
    }
  }
  // node layout when every shared node carries one value
  bool node = !elem_const;
  std::vector<std::vector<double>> planes;
  std::vector<char> seen;
  if (node) {
    planes.assign(src.size(), std::vector<double>(h->plane, 0.0));
    seen.assign(h->plane, 0);
  }
  for (int e = 0; e < ne && node; ++e)
    for (int q = 0; q < NN && node; ++q) {
      const long long L = h->glob2lat[d->ibool[q + (size_t)NN * e] - 1];
      for (size_t m = 0; m < src.size(); ++m) {
        const double v = src[m][q + (size_t)NN * e];
        if (seen[L] && planes[m][L] != v) {
          node = false;
          break;
        }
        planes[m][L] = v;
      }
      seen[L] = 1;
    }
  if (!elem_const) h->mat_elem = node ? kMatNode : kMatPoint;
  if (d->adjoint) {
    if (!node) return set_err(h, SEM2D_E_UNSUPPORTED, "the gradient workflow needs a material continuous at nodes");
    std::vector<double> rp(h->plane, 0.0);
    std::vector<char> seen2(h->plane, 0);
    for (int e = 0; e < ne; ++e)
      for (int q = 0; q < NN; ++q) {
        const long long L = h->glob2lat[d->ibool[q + (size_t)NN * e] - 1];
        const double v = d->rho[q + (size_t)NN * e];
        if (seen2[L] && rp[L] != v) return set_err(h, SEM2D_E_UNSUPPORTED, "density not continuous at nodes");
        rp[L] = v;
        seen2[L] = 1;
      }
    h->adjoint = 1;
    const int st2 = upload_real(h, &h->rho_plane, rp);
    if (st2) return st2;
  }
  int st;
  for (size_t m = 0; m < src.size() && !elem_const; ++m) {
    if (node) {
      st = upload_real(h, &h->mat[m], planes[m]);
    } else {
      std::vector<double> el(npt);
      for (int e = 0; e < ne; ++e) {
        const size_t eo = ((size_t)h->elem_ez[e] * h->nx + h->elem_ex[e]) * NN;
        for (int q = 0; q < NN; ++q) el[eo + q] = src[m][q + (size_t)NN * e];
      }
      st = upload_real(h, &h->mat[m], el);
    }
    if (st) return st;
  }
  return upload_kveta(h, d);
}

// Stacey P3 terms (one per boundary element edge point) grouped by the
// perimeter slot of the node they load, in the order of the descriptor
int upload_stacey(sem2d_handle *h, const sem2d_problem_desc *d) {
  const int nt = d->nstacey, N = h->N, np = d->npoin;
  if (nt <= 0) return SEM2D_OK;
  if (d->ndof != 2) return set_err(h, SEM2D_E_ARG, "Stacey terms need ndof = 2");
  if (!d->stacey_node || !d->stacey_k || !d->stacey_edge || !d->stacey_K)
    return set_err(h, SEM2D_E_ARG, "Stacey arrays missing");
  const int nslot = perimeter_slots(h->LX, h->LZ);
  std::vector<std::vector<int>> by_slot(nslot);
  for (int t = 0; t < nt; ++t) {
    const int p = d->stacey_node[t] - 1;
    if (p < 0 || p >= np || d->stacey_k[t] < 0 || d->stacey_k[t] >= N)
      return set_err(h, SEM2D_E_ARG, "Stacey term out of range");
    const long long L = h->glob2lat[p];
    const int sl = perimeter_slot(int(L % h->pitch), int(L / h->pitch), h->LX, h->LZ);
    if (sl < 0) return set_err(h, SEM2D_E_UNSUPPORTED, "Stacey node inside the domain");
    by_slot[sl].push_back(t);
  }
  // a side that crosses periodic sides: the forces of its two ends, a
  // periodic pair, are summed and shared (KxD, bc_abso.f90:329-332), so
  // each end's slot lists the other's terms too
  if (d->nperio > 0 && d->perio_master && d->perio_slave) {
    std::vector<std::vector<int>> own = by_slot;
    for (int k = 0; k < d->nperio; ++k) {
      const int a = d->perio_master[k] - 1, b = d->perio_slave[k] - 1;
      if (a < 0 || a >= np || b < 0 || b >= np) return set_err(h, SEM2D_E_ARG, "periodic node out of range");
      const long long La = h->glob2lat[a], Lb = h->glob2lat[b];
      const int sa = perimeter_slot(int(La % h->pitch), int(La / h->pitch), h->LX, h->LZ);
      const int sb = perimeter_slot(int(Lb % h->pitch), int(Lb / h->pitch), h->LX, h->LZ);
      if (sa < 0 || sb < 0 || own[sa].empty() || own[sb].empty()) continue;
      // the same list, in the same order, for both ends: equal sums
      std::vector<int> both = own[sa];
      both.insert(both.end(), own[sb].begin(), own[sb].end());
      by_slot[sa] = both;
      by_slot[sb] = both;
    }
  }
  std::vector<int> slot, ptr(1, 0), kk, lat;
  std::vector<double> K0, K1;
  for (int sl = 0; sl < nslot; ++sl) {
    if (by_slot[sl].empty()) continue;
    slot.push_back(sl);
    for (int t : by_slot[sl]) {
      kk.push_back(d->stacey_k[t]);
      for (int l = 0; l < N; ++l) {
        const int q = d->stacey_edge[l + (size_t)N * t] - 1;
        if (q < 0 || q >= np) return set_err(h, SEM2D_E_ARG, "Stacey edge node out of range");
        lat.push_back(int(h->glob2lat[q]));
      }
      K0.push_back(d->stacey_K[t]);
      K1.push_back(d->stacey_K[t + (size_t)nt]);
    }
    ptr.push_back(int(kk.size()));
  }
  K0.insert(K0.end(), K1.begin(), K1.end());
  std::vector<double> H(d->hprime, d->hprime + (size_t)N * N);
  h->st_nslot = int(slot.size());
  h->st_nterm = int(kk.size());
  int st;
  if ((st = dupload(h, &h->d_st_slot, slot)) || (st = dupload(h, &h->d_st_ptr, ptr)) ||
      (st = dupload(h, &h->d_st_k, kk)) || (st = dupload(h, &h->d_st_lat, lat)) ||
      (st = upload_real(h, &h->d_st_K, K0)) || (st = upload_real(h, &h->d_st_H, H)) ||
      (st = upload_real(h, &h->per_kd, std::vector<double>((size_t)2 * nslot, 0.0))))
    return st;
  return SEM2D_OK;
}

// &BC_DIRNEU zero-Dirichlet components by perimeter slot; at a fault node
// the zero that follows the fault in &BC_DEF order is applied by the fault
// update instead
int upload_dirneu(sem2d_handle *h, const sem2d_problem_desc *d) {
  const int n = d->ndir, np = d->npoin;
  if (n <= 0) return SEM2D_OK;
  if (!d->dir_node || !d->dir_comp || !d->dir_after_fault) return set_err(h, SEM2D_E_ARG, "Dirichlet arrays missing");
  const int nslot = perimeter_slots(h->LX, h->LZ);
  std::vector<int> slot(nslot, 0);
  std::vector<unsigned char> fdir(h->nflt ? h->nflt : 1, 0);
  for (int k = 0; k < n; ++k) {
    const int p = d->dir_node[k] - 1, c = d->dir_comp[k];
    if (p < 0 || p >= np || c < 0 || c >= d->ndof) return set_err(h, SEM2D_E_ARG, "Dirichlet entry out of range");
    const long long L = h->glob2lat[p];
    const int I = int(L % h->pitch), J = int(L / h->pitch);
    const int sl = perimeter_slot(I, J, h->LX, h->LZ);
    if (sl < 0) return set_err(h, SEM2D_E_UNSUPPORTED, "Dirichlet node inside the domain");
    const bool on_fault = h->nflt && (J == h->jf1 || (h->two && J == h->jf2));
    if (on_fault && d->dir_after_fault[k])
      fdir[I] |= (unsigned char)(1u << ((J == h->jf1 ? 0 : 1) * 2 + c));
    else
      slot[sl] |= 1 << c;
  }
  h->ndir = n;
  int st;
  if ((st = dupload(h, &h->per_dir, slot)) || (st = dupload(h, &h->d_fdir, fdir))) return st;
  return SEM2D_OK;
}

// periodic node pairs: the lattice columns I = 0 and LX-1 row by row (the
// Cartesian mesher's left and right sides) or the rows J = 0 and LZ-1
// column by column (bottom and top)
int upload_perio(sem2d_handle *h, const sem2d_problem_desc *d) {
  const int n = d->nperio, np = d->npoin;
  if (n <= 0) return SEM2D_OK;
  if (!d->perio_master || !d->perio_slave) return set_err(h, SEM2D_E_ARG, "periodic arrays missing");
  auto ij = [&](int node1, int &I, int &J) {
    const long long L = h->glob2lat[node1 - 1];
    I = int(L % h->pitch);
    J = int(L / h->pitch);
  };
  for (int k = 0; k < n; ++k) {
    const int a = d->perio_master[k] - 1, b = d->perio_slave[k] - 1;
    if (a < 0 || a >= np || b < 0 || b >= np) return set_err(h, SEM2D_E_ARG, "periodic node out of range");
  }
  int I0, J0, I1, J1;
  ij(d->perio_master[0], I0, J0);
  ij(d->perio_slave[0], I1, J1);
  const bool tb = I0 == I1;
  const int len = tb ? h->LX : h->LZ;
  if (n != len) return set_err(h, SEM2D_E_UNSUPPORTED, "periodic sides other than left/right or bottom/top");
  std::vector<int> seen(len, 0);
  for (int k = 0; k < n; ++k) {
    int Ia, Ja, Ib, Jb;
    ij(d->perio_master[k], Ia, Ja);
    ij(d->perio_slave[k], Ib, Jb);
    const bool ok = tb ? (Ia == Ib && ((Ja == 0 && Jb == h->LZ - 1) || (Ja == h->LZ - 1 && Jb == 0)) && !seen[Ia])
                       : (Ja == Jb && ((Ia == 0 && Ib == h->LX - 1) || (Ia == h->LX - 1 && Ib == 0)) && !seen[Ja]);
    if (!ok) return set_err(h, SEM2D_E_UNSUPPORTED, "periodic sides other than left/right or bottom/top");
    seen[tb ? Ia : Ja] = 1;
  }
  if (tb && h->nflt) return set_err(h, SEM2D_E_UNSUPPORTED, "bottom/top periodic sides with a fault");
  h->nperio = n;
  h->perio_tb = tb ? 1 : 0;
  return upload_real(h, &h->perio_f, std::vector<double>((size_t)2 * h->ndof * len, 0.0));
}

// A time function on the device: the TAB rows and their spline second
// derivatives are copied; host_v2 (optional) receives the derivatives for
// an evaluation on the host.
int upload_stf(sem2d_handle *h, const sem2d_stf &s, StfDev *out, std::vector<double> *host_v2 = nullptr) {
  if (const char *m = stf_check(s)) return set_err(h, SEM2D_E_ARG, m);
  StfDev q{};
  q.kind = s.kind;
  q.ntab = s.ntab;
  q.f0 = s.f0;
  q.onset = s.onset;
  q.ampli = s.ampli;
  q.par1 = s.par1;
  q.par2 = s.par2;
  if (s.kind == SEM2D_STF_TAB) {
    const std::vector<double> t(s.tab_t, s.tab_t + s.ntab), v(s.tab_v, s.tab_v + s.ntab);
    const std::vector<double> v2 = stf_spline_d2(s.tab_t, s.tab_v, s.ntab);
    double *dt_ = nullptr, *dv = nullptr, *dv2 = nullptr;
    int st;
    if ((st = dupload(h, &dt_, t)) || (st = dupload(h, &dv, v)) || (st = dupload(h, &dv2, v2))) return st;
    q.t = dt_;
    q.v = dv;
    q.v2 = dv2;
    if (host_v2) *host_v2 = v2;
  }
  *out = q;
  return SEM2D_OK;
}

// The incident plane wave (SRC_WAVE_get_VT src_wave.f90:190-224, phase
// :181-187, SO_WAVE_get_VT src_gen.f90:322-339) and the Neumann tractions
// (bc_DIRNEU_apply bc_dirneu.f90:157-167) as perimeter entries: weight,
// time function and time shift per (slot, entry, component).
int upload_boundary_forces(sem2d_handle *h, const sem2d_problem_desc *d) {
  const bool wave = d->wave_phase != SEM2D_WAVE_NONE && d->nabs > 0 && d->abs_wave;
  if (!wave && d->nneu <= 0) return SEM2D_OK;
  const int nd = h->ndof, np = d->npoin, nslot = perimeter_slots(h->LX, h->LZ);
  std::vector<double> W((size_t)2 * nd * nslot, 0.0), phi((size_t)2 * nslot, 0.0);
  std::vector<signed char> fn((size_t)2 * nd * nslot, -1);
  std::vector<int> used(nslot, 0);
  std::vector<StfDev> stfs;
  auto slot_of = [&](int node1) {
    const int p = node1 - 1;
    if (p < 0 || p >= np) return -2;
    const long long L = h->glob2lat[p];
    return perimeter_slot(int(L % h->pitch), int(L / h->pitch), h->LX, h->LZ);
  };
  if (wave) {
    if (d->wave_phase != SEM2D_WAVE_P && d->wave_phase != SEM2D_WAVE_S)
      return set_err(h, SEM2D_E_ARG, "wave_phase must be SEM2D_WAVE_P or SEM2D_WAVE_S");
    if (!d->wave_stf || !d->abs_B || !d->abs_n) return set_err(h, SEM2D_E_ARG, "incident wave without wave_stf, abs_B or abs_n");
    if (!(d->wave_cp > 0) || !(d->wave_cs > 0)) return set_err(h, SEM2D_E_ARG, "incident wave needs cp > 0 and cs > 0");
    if (!d->coord) return set_err(h, SEM2D_E_ARG, "incident wave without node coordinates");
    StfDev q;
    int st = upload_stf(h, *d->wave_stf, &q);
    if (st) return st;
    h->static_load = h->static_load || d->wave_stf->kind != SEM2D_STF_RICKER;
    const signed char qi = (signed char)stfs.size();
    stfs.push_back(q);
    const double kPi = 3.141592653589793, a = kPi * d->wave_angle / 180.0;
    const double k0 = -std::sin(a), k1 = std::cos(a);  // WAVE_init, src_wave.f90:163-172
    const bool P = d->wave_phase == SEM2D_WAVE_P;
    const double p0 = P ? -std::sin(a) : std::cos(a), p1 = P ? std::cos(a) : std::sin(a);
    const double c = P ? d->wave_cp : d->wave_cs;
    const double s0 = k0 / c, s1 = k1 / c;
    const double mu = d->wave_mu, lam = d->wave_lambda, cp = d->wave_cp, cs = d->wave_cs;
    for (int k = 0; k < d->nabs; ++k) {
      if (!d->abs_wave[k]) continue;
      const int sp = slot_of(d->abs_node[k]);
      if (sp < 0) return set_err(h, SEM2D_E_ARG, "absorbing node out of range");
      if (used[sp] >= 2) return set_err(h, SEM2D_E_UNSUPPORTED, "more than two boundary forces at a node");
      const int e = used[sp]++;
      const double n0 = d->abs_n[k], n1 = d->abs_n[k + d->nabs], B = d->abs_B[k];
      const double KN = k0 * n0 + k1 * n1;
      double V[2], T[2];
      if (nd == 1) {
        V[0] = 1.0;
        T[0] = -mu / cs * KN;
      } else {
        V[0] = p0;
        V[1] = p1;
        if (P) {
          T[0] = -1.0 / cp * (lam * n0 + 2.0 * mu * KN * k0);
          T[1] = -1.0 / cp * (lam * n1 + 2.0 * mu * KN * k1);
        } else {
          const double PN = p0 * n0 + p1 * n1;
          T[0] = -mu / cs * (PN * k0 + KN * p0);
          T[1] = -mu / cs * (PN * k1 + KN * p1);
        }
      }
      for (int cc = 0; cc < nd; ++cc) {
        const size_t ei = ((size_t)e * nd + cc) * nslot + sp;
        W[ei] = d->abs_C[k + (size_t)d->nabs * cc] * V[cc] + B * T[cc];
        fn[ei] = qi;
      }
      const int pn = d->abs_node[k] - 1;
      phi[(size_t)e * nslot + sp] =
          (d->coord[2 * (size_t)pn] - d->wave_ref[0]) * s0 + (d->coord[2 * (size_t)pn + 1] - d->wave_ref[1]) * s1 +
          d->wave_tdelay;
    }
  }
  if (d->nneu > 0) {
    if (!d->neu_node || !d->neu_comp || !d->neu_B || !d->neu_stf || !d->neu_stfs || d->nneu_stf <= 0)
      return set_err(h, SEM2D_E_ARG, "incomplete Neumann traction arrays");
    if (d->nneu_stf > 100) return set_err(h, SEM2D_E_UNSUPPORTED, "too many traction time functions");
    const signed char q0 = (signed char)stfs.size();
    for (int k = 0; k < d->nneu_stf; ++k) {
      StfDev q;
      int st = upload_stf(h, d->neu_stfs[k], &q);
      if (st) return st;
      h->static_load = h->static_load || d->neu_stfs[k].kind != SEM2D_STF_RICKER;
      stfs.push_back(q);
    }
    for (int k = 0; k < d->nneu; ++k) {
      const int sp = slot_of(d->neu_node[k]);
      if (sp == -2) return set_err(h, SEM2D_E_ARG, "traction node out of range");
      if (sp < 0) return set_err(h, SEM2D_E_UNSUPPORTED, "traction node inside the domain");
      const int cc = d->neu_comp[k], qk = d->neu_stf[k];
      if (cc < 0 || cc >= nd) return set_err(h, SEM2D_E_ARG, "traction component out of range");
      if (qk < 0 || qk >= d->nneu_stf) return set_err(h, SEM2D_E_ARG, "traction time function out of range");
      for (int j = 0; j < d->ndir; ++j)
        if (d->dir_node && d->dir_comp && d->dir_node[j] == d->neu_node[k] && d->dir_comp[j] == cc)
          return set_err(h, SEM2D_E_UNSUPPORTED, "a Neumann traction on a zero-Dirichlet component");
      const long long L = h->glob2lat[d->neu_node[k] - 1];
      if (h->nflt && (L / h->pitch == h->jf1 || L / h->pitch == h->jf2))
        return set_err(h, SEM2D_E_UNSUPPORTED, "a Neumann traction on a fault node");
      // an entry of the slot without time shift and free for this component
      int e = -1;
      for (int j = 0; j < used[sp]; ++j)
        if (phi[(size_t)j * nslot + sp] == 0.0 && fn[((size_t)j * nd + cc) * nslot + sp] < 0) e = j;
      if (e < 0) {
        if (used[sp] >= 2) return set_err(h, SEM2D_E_UNSUPPORTED, "more than two boundary forces at a node");
        e = used[sp]++;
      }
      const size_t ei = ((size_t)e * nd + cc) * nslot + sp;
      W[ei] = d->neu_B[k];
      fn[ei] = (signed char)(q0 + qk);
    }
  }
  double *dW = nullptr, *dphi = nullptr;
  signed char *dfn = nullptr;
  StfDev *dstf = nullptr;
  int st;
  if ((st = dupload(h, &dW, W)) || (st = dupload(h, &dphi, phi)) || (st = dupload(h, &dfn, fn)) ||
      (st = dupload(h, &dstf, stfs)))
    return st;
  if ((st = upload_real(h, &h->per_bf, std::vector<double>((size_t)nd * nslot, 0.0)))) return st;
  h->bf.W = dW;
  h->bf.fn = dfn;
  h->bf.phi = dphi;
  h->bf.stf = dstf;
  h->bf.dt = h->dt;
  h->bf.tshift = (h->alpha - 1.0) * h->dt;
  return SEM2D_OK;
}

int upload_mass_and_boundaries(sem2d_handle *h, const sem2d_problem_desc *d) {
  const int nd = d->ndof, np = d->npoin;
  const int nslot = perimeter_slots(h->LX, h->LZ);
  std::vector<double> rm(h->plane, 1.0), prm((size_t)nslot * nd, 0.0), pca((size_t)nslot * nd, 0.0),
      pcb((size_t)nslot * nd, 0.0);
  std::vector<int> used(nslot, 0);
  for (int p = 0; p < np; ++p) {
    const long long L = h->glob2lat[p];
    const int I = int(L % h->pitch), J = int(L / h->pitch);
    const int s = perimeter_slot(I, J, h->LX, h->LZ);
    if (s >= 0) {
      for (int c = 0; c < nd; ++c) prm[(size_t)c * nslot + s] = d->rmass[p + (size_t)np * c];
    } else {
      if (nd == 2 && d->rmass[p] != d->rmass[p + np] &&
          !(h->nflt && (J == h->jf1 || J == h->jf2)))
        return set_err(h, SEM2D_E_UNSUPPORTED, "dof-dependent mass away from the boundary");
    }
    rm[L] = d->rmass[p];
  }
  for (int k = 0; k < d->nabs; ++k) {
    const int p = d->abs_node[k] - 1;
    if (p < 0 || p >= np) return set_err(h, SEM2D_E_ARG, "absorbing node out of range");
    const long long L = h->glob2lat[p];
    const int s = perimeter_slot(int(L % h->pitch), int(L / h->pitch), h->LX, h->LZ);
    if (s < 0) return set_err(h, SEM2D_E_UNSUPPORTED, "absorbing node inside the domain");
    if (used[s] >= 2) return set_err(h, SEM2D_E_UNSUPPORTED, "node on more than two absorbing boundaries");
    std::vector<double> &dst = used[s] == 0 ? pca : pcb;
    for (int c = 0; c < nd; ++c) dst[(size_t)c * nslot + s] = d->abs_C[k + (size_t)d->nabs * c];
    used[s]++;
  }
  int st;
  if ((st = upload_real(h, &h->rmass, rm)) || (st = upload_real(h, &h->per_rm, prm)) ||
      (st = upload_real(h, &h->per_Ca, pca)) || (st = upload_real(h, &h->per_Cb, pcb)))
    return st;
  if ((st = upload_stacey(h, d))) return st;
  if ((st = upload_dirneu(h, d))) return st;
  if ((st = upload_boundary_forces(h, d))) return st;
  return upload_perio(h, d);
}

int upload_fault(sem2d_handle *h, const sem2d_problem_desc *d) {
  const int nf = d->nflt, nd = d->ndof, np = d->npoin;
  h->nflt = nf;
  if (!nf) return SEM2D_OK;
  if (!d->flt_node1 || !d->flt_n1 || !d->flt_B || !d->flt_invM1 || !d->flt_Z || !d->flt_T0)
    return set_err(h, SEM2D_E_ARG, "incomplete fault description");
  h->two = d->flt_node2 != nullptr;
  if (h->two && !d->flt_invM2) return set_err(h, SEM2D_E_ARG, "two-sided fault without invM2");
  if (nf != h->LX) return set_err(h, SEM2D_E_UNSUPPORTED, "fault must span a full lattice row");
  for (int side = 0; side < 1 + h->two; ++side) {
    const int *nodes = side == 0 ? d->flt_node1 : d->flt_node2;
    int J = -1;
    for (int k = 0; k < nf; ++k) {
      const int p = nodes[k] - 1;
      if (p < 0 || p >= np) return set_err(h, SEM2D_E_ARG, "fault node out of range");
      const long long L = h->glob2lat[p];
      const int I = int(L % h->pitch), Jk = int(L / h->pitch);
      if (k == 0) J = Jk;
      if (I != k || Jk != J) return set_err(h, SEM2D_E_UNSUPPORTED, "fault nodes are not a lattice row");
    }
    (side == 0 ? h->jf1 : h->jf2) = J;
  }
  if (d->flt_friction == SEM2D_FRICTION_SWF) {
    if (!d->swf_dc || !d->swf_mus || !d->swf_mud) return set_err(h, SEM2D_E_ARG, "missing SWF parameters");
  } else if (d->flt_friction == SEM2D_FRICTION_RSF) {
    if (!d->rsf_dc || !d->rsf_mus || !d->rsf_a || !d->rsf_b || !d->rsf_vstar)
      return set_err(h, SEM2D_E_ARG, "missing RSF parameters");
    if (d->rsf_kind < 1 || d->rsf_kind > 4) return set_err(h, SEM2D_E_ARG, "rsf_kind out of range");
  } else if (d->flt_friction != SEM2D_FRICTION_TWF) {
    return set_err(h, SEM2D_E_UNSUPPORTED, "fault without SWF, RSF or TWF friction");
  }
  if (d->twf_kind < 0 || d->twf_kind > 3) return set_err(h, SEM2D_E_ARG, "twf_kind out of range");
  if ((d->twf_kind || d->flt_friction == SEM2D_FRICTION_TWF) && (!(d->twf_L > 0) || !(d->twf_V > 0)))
    return set_err(h, SEM2D_E_ARG, "time weakening needs L > 0 and V > 0");
  h->friction = d->flt_friction;
  auto vec = [&](const double *p, size_t n, double fill) {
    std::vector<double> v(n, fill);
    if (p) std::copy(p, p + n, v.begin());
    return v;
  };
  std::vector<double> rmf((size_t)2 * nd * nf, 0.0);
  for (int side = 0; side < 1 + h->two; ++side)
    for (int c = 0; c < nd; ++c)
      for (int k = 0; k < nf; ++k) {
        const int p = (side == 0 ? d->flt_node1 : d->flt_node2)[k] - 1;
        rmf[((size_t)side * nd + c) * nf + k] = d->rmass[p + (size_t)np * c];
      }
  int st;
  auto up = [&](int idx, const std::vector<double> &v) { return dupload(h, &h->fd[idx], v); };
  const size_t nfd = (size_t)nf * nd;
  if ((st = dalloc(h, &h->fd[F_D64], 2 * nfd)) || (st = dalloc(h, &h->fd[F_V64], 2 * nfd)) ||
      (st = dalloc(h, &h->fd[F_A64], 2 * nfd)) || (st = up(F_RM, rmf)) ||
      (st = up(F_N1, vec(d->flt_n1, 2 * (size_t)nf, 0))) || (st = up(F_B, vec(d->flt_B, nf, 0))) ||
      (st = up(F_INVM1, vec(d->flt_invM1, nfd, 0))) || (st = up(F_INVM2, vec(d->flt_invM2, nfd, 0))) ||
      (st = up(F_Z, vec(d->flt_Z, nfd, 0))) || (st = up(F_T0, vec(d->flt_T0, 2 * (size_t)nf, 0))) ||
      (st = up(F_COH, vec(d->flt_cohesion, nf, 0))))
    return st;
  if ((st = up(F_SWF_DC, vec(d->swf_dc, nf, 0.5))) || (st = up(F_SWF_MUS, vec(d->swf_mus, nf, 0.6))) ||
      (st = up(F_SWF_MUD, vec(d->swf_mud, nf, 0.5))) || (st = up(F_SWF_P, vec(d->swf_p, nf, 3.0))) ||
      (st = up(F_SWF_ALPHA, vec(d->swf_alpha, nf, 0.0))))
    return st;
  std::vector<double> rdc = vec(d->rsf_dc, nf, 0.5), rvs = vec(d->rsf_vstar, nf, 1.0);
  std::vector<double> tc(nf), ct(nf);
  for (int k = 0; k < nf; ++k) {
    tc[k] = rdc[k] / rvs[k];
    ct[k] = std::exp(-d->dt / tc[k]);
  }
  if ((st = up(F_RSF_DC, rdc)) || (st = up(F_RSF_MUS, vec(d->rsf_mus, nf, 0.6))) ||
      (st = up(F_RSF_A, vec(d->rsf_a, nf, 0.01))) || (st = up(F_RSF_B, vec(d->rsf_b, nf, 0.02))) ||
      (st = up(F_RSF_VSTAR, rvs)) || (st = up(F_RSF_VC, vec(d->rsf_vc, nf, 1e-6))) ||
      (st = up(F_RSF_TC, tc)) || (st = up(F_RSF_COEFT, ct)))
    return st;
  // state
  std::vector<double> V0(nfd, 0.0), th0(nf, 0.0);
  if (h->friction == SEM2D_FRICTION_RSF) {
    for (int k = 0; k < nf; ++k) {
      V0[k] = d->flt_V0 ? d->flt_V0[k] : 1e-12;
      th0[k] = d->rsf_theta ? d->rsf_theta[k] : 0.0;
    }
  }
  h->h_fault_init = V0;
  h->h_fault_init.insert(h->h_fault_init.end(), th0.begin(), th0.end());
  if ((st = dalloc(h, &h->fd[F_D], nfd)) || (st = up(F_V, V0)) || (st = dalloc(h, &h->fd[F_T], 2 * (size_t)nf)) ||
      (st = dalloc(h, &h->fd[F_TSTICK], 2 * (size_t)nf)) || (st = dalloc(h, &h->fd[F_MU], nf)) ||
      (st = up(F_THETA, th0)) || (st = dalloc(h, &h->fd[F_SIGMA], nf)))
    return st;
  const int oix1 = d->flt_oix1 > 0 ? d->flt_oix1 : 1;
  const int oixn = d->flt_oixn > 0 ? d->flt_oixn : nf;
  const int oixd = d->flt_oixd > 0 ? d->flt_oixd : 1;
  h->onx = (oixn - oix1) / oixd + 1;
  h->fnsamp = std::max(d->flt_nsamp, 0);
  if ((st = dalloc(h, &h->fd[F_SERIES], (size_t)h->onx * 6 * std::max(h->fnsamp, 1)))) return st;
  h->potency = d->flt_potency != 0;
  if (h->potency && ((st = dalloc(h, &h->fd[F_POT], (size_t)6 * nf)) ||
                     (st = dalloc(h, &h->fd[F_POTSERIES], (size_t)6 * (std::max(d->nt, 0) + 1)))))
    return st;
  std::vector<double> xz(2 * (size_t)nf);
  for (int k = 0; k < nf; ++k) {
    const int p = d->flt_node1[k] - 1;
    xz[2 * k] = d->coord[2 * (size_t)p];
    xz[2 * k + 1] = d->coord[2 * (size_t)p + 1];
  }
  if ((st = up(F_XZ, xz))) return st;
  return SEM2D_OK;
}

template <typename real>
FaultParams<real> fault_params(sem2d_handle *h, int cur) {
  const FaultScalars &s = h->fs;
  FaultParams<real> f{};
  f.ndof = h->ndof;
  f.LX = h->LX;
  f.pitch = h->pitch;
  f.plane = h->plane;
  f.nflt = h->nflt;
  f.two = h->two;
  f.jf1 = h->jf1;
  f.jf2 = h->jf2;
  f.f_flt = nullptr;
  f.Dcur = (const real *)h->D[cur];
  f.Dnext = (real *)h->D[1 - cur];
  f.Vnext = (real *)h->V[1 - cur];
  f.Anext = h->keep_accel ? (real *)h->A[1 - cur] : nullptr;
  f.dir_zero = h->ndir ? h->d_fdir : nullptr;
  f.d64 = h->fd[F_D64];
  f.v64 = h->fd[F_V64];
  f.a64 = h->fd[F_A64];
  f.rm = h->fd[F_RM];
  f.n1 = h->fd[F_N1];
  f.B = h->fd[F_B];
  f.invM1 = h->fd[F_INVM1];
  f.invM2 = h->fd[F_INVM2];
  f.Z = h->fd[F_Z];
  f.T0 = h->fd[F_T0];
  f.coh = h->fd[F_COH];
  f.coefA2V = s.coefA2V;
  f.coefA2D = s.coefA2D;
  f.opening = s.opening;
  f.friction = h->friction == SEM2D_FRICTION_RSF ? 2 : h->friction == SEM2D_FRICTION_TWF ? 3 : 1;
  f.twf_kind = s.twf_kind;
  f.twf_mus = s.twf_mus;
  f.twf_mud = s.twf_mud;
  f.twf_mu0 = s.twf_mu0;
  f.twf_X = s.twf_X;
  f.twf_Z = s.twf_Z;
  f.twf_V = s.twf_V;
  f.twf_L = s.twf_L;
  f.twf_T = s.twf_T;
  f.twf_Dc = s.twf_Dc;
  f.fxz = h->fd[F_XZ];
  f.swf_kind = s.swf_kind;
  f.swf_healing = s.swf_healing;
  f.rsf_kind = s.rsf_kind;
  f.normal_kind = s.normal_kind;
  f.normal_V = s.normal_V;
  f.normal_coef = 0;
  if (s.normal_kind == 2) f.normal_coef = std::exp(-h->dt / s.normal_T);
  if (s.normal_kind == 3) f.normal_coef = h->dt / s.normal_L;
  f.swf_dc = h->fd[F_SWF_DC];
  f.swf_mus = h->fd[F_SWF_MUS];
  f.swf_mud = h->fd[F_SWF_MUD];
  f.swf_p = h->fd[F_SWF_P];
  f.swf_alpha = h->fd[F_SWF_ALPHA];
  f.rsf_dc = h->fd[F_RSF_DC];
  f.rsf_mus = h->fd[F_RSF_MUS];
  f.rsf_a = h->fd[F_RSF_A];
  f.rsf_b = h->fd[F_RSF_B];
  f.rsf_vstar = h->fd[F_RSF_VSTAR];
  f.rsf_vc = h->fd[F_RSF_VC];
  f.rsf_Tc = h->fd[F_RSF_TC];
  f.rsf_coeft = h->fd[F_RSF_COEFT];
  f.D = h->fd[F_D];
  f.V = h->fd[F_V];
  f.T = h->fd[F_T];
  f.Tstick = h->fd[F_TSTICK];
  f.MU = h->fd[F_MU];
  f.theta = h->fd[F_THETA];
  f.sigma = h->fd[F_SIGMA];
  f.oit = s.oit;
  f.oitd = s.oitd;
  f.oix1 = s.oix1;
  f.oixd = s.oixd;
  f.onx = h->onx;
  f.nsamp = h->fnsamp;
  f.series = h->fd[F_SERIES];
  f.pot = h->potency ? h->fd[F_POT] : nullptr;
  f.scheme = h->scheme ? 1 : 0;  // the fault node update is the same for HHT-alpha
  f.dt = h->dt;
  f.cv = h->scheme ? h->gamma * h->dt : h->dt;
  f.cpred = (1.0 - h->gamma) * h->dt;
  f.cd2 = (0.5 - h->beta) * h->dt * h->dt;
  f.cb = h->scheme ? h->beta * h->dt * h->dt : 0.0;
  f.tshift = (h->alpha - 1.0) * h->dt;  // HHT-alpha boundary time (solver.f90:118-122)
  f.step = h->d_step;
  f.done = h->d_done;
  f.error = h->d_error;
  f.nr_maxit = h->nr_maxit;
  return f;
}

template <typename real>
int launch_fault_init(sem2d_handle *h) {
  if (!h->nflt) return SEM2D_OK;
  FaultParams<real> f = fault_params<real>(h, h->cur);
  fault_init_kernel<real><<<(h->nflt + 127) / 128, 128, 0, h->stream>>>(f);
  CK(cudaGetLastError());
  h->launches++;
  return SEM2D_OK;
}

// the type-erased description of one step of problem h from buffer parity
// cur; f holds the fault parameters the description points to
template <typename real>
BulkConfig make_config(sem2d_handle *h, int cur, FaultParams<real> &f) {
  BulkConfig bc;
  bc.N = h->N;
  bc.ndof = h->ndof;
  bc.mixed = h->mixed;
  bc.nplanes = h->nplanes;
  bc.nmat = h->nmat;
  bc.has_kv = h->has_kv;
  bc.mat_elem = h->mat_elem;
  bc.mat_iso = h->mat_iso;
  bc.fast = fast_path(h);
  bc.error = h->d_error;
  bc.spin_limit = h->spin_limit;
  bc.march_warps = h->march_warps;
  bc.march_fst = h->march_fst;
  bc.Fcur = h->F[cur];
  bc.Fnext = h->F[1 - cur];
  bc.grid_x = (h->nx + h->TX - 1) / h->TX;
  bc.grid_y = int(h->ztile.size()) - 1;
  bc.LX = h->LX;
  bc.LZ = h->LZ;
  bc.pitch = h->pitch;
  bc.plane = h->plane;
  bc.nx = h->nx;
  bc.nz = h->nz;
  bc.row0 = h->d_row0;
  bc.TX = h->TX;
  bc.ztile = h->d_ztile;
  bc.Dcur = h->D[cur];
  bc.Dnext = h->D[1 - cur];
  bc.Vcur = h->V[cur];
  bc.Vnext = h->V[1 - cur];
  bc.Acur = h->A[cur];
  bc.Anext = h->keep_accel ? h->A[1 - cur] : nullptr;
  for (int m = 0; m < 4; ++m) bc.mat[m] = h->mat[m];
  bc.gen = h->gen;
  bc.gen_stride = (long long)h->N * h->N * h->nx * h->nz;
  bc.kveta = h->kveta;
  bc.rmass = h->rmass;
  for (int g = 0; g < 4; ++g) bc.geo[g] = h->geo[g];
  bc.per_rm = h->per_rm;
  bc.per_Ca = h->per_Ca;
  bc.per_Cb = h->per_Cb;
  bc.per_kd = h->per_kd;
  bc.per_dir = h->ndir ? h->per_dir : nullptr;
  bc.perio_f = h->nperio ? h->perio_f : nullptr;
  bc.perio_tb = h->perio_tb;
  bc.per_bf = h->bf.W ? h->per_bf : nullptr;
  bc.jf1 = h->nflt ? h->jf1 : -1;
  bc.jf2 = h->nflt ? h->jf2 : -1;
  bc.has_fault = h->nflt ? 1 : 0;
  f = FaultParams<real>{};
  if (h->nflt) {
    f = fault_params<real>(h, cur);
    bc.flt = &f;
  }
  bc.nsrc = h->nsrc;
  bc.src_I = h->src_I;
  bc.src_J = h->src_J;
  bc.src_amp = h->src_amp;
  bc.nt = h->nt;
  bc.step = h->d_step;
  bc.done = h->d_done;
  if (h->nrec && !h->rec_separate) {
    bc.rec_nsamp = h->rec_nsamp;
    bc.rec_isamp = h->rec_isamp;
    bc.rec_nrec = h->nrec;
    bc.rec_npts = h->rec_npts;
    bc.rec_field = h->rec_field;
    bc.rec_tile_start = h->rec_tile_start;
    bc.rec_ids = h->rec_ids;
    bc.rec_I = h->rec_I;
    bc.rec_J = h->rec_J;
    bc.rec_w = h->rec_w;
    bc.sis = h->sis;
  }
  bc.scheme = h->scheme;
  bc.dt = h->dt;
  bc.cv = h->scheme ? h->gamma * h->dt : h->dt;
  bc.cpred = (1.0 - h->gamma) * h->dt;
  bc.cd2 = (0.5 - h->beta) * h->dt * h->dt;
  bc.cb = h->scheme ? h->beta * h->dt * h->dt : 0.0;
  bc.cal = 1.0 - h->alpha;
  bc.cpa = h->alpha * ((1.0 - h->gamma) * h->dt);
  bc.kd2 = h->kd2;
  bc.width = h->width;
  bc.chunk_shift = h->fault_chunk;
  bc.fault_force = h->d_fault_force;
  bc.H = h->H.data();
  bc.w = h->w.data();
  bc.stream = h->stream;
  return bc;
}

// Stacey P3 boundary forces of the step's predictor displacement
// (BC_ABSO_apply, bc_abso.f90:321-334), one thread per (perimeter slot,
// component): the sum over the slot's terms t of K(t,c) times the derivative
// of D(:,c) along the element edge, sum_l hprime(l,k_t) D(edge node l, c).
// The step kernel subtracts it at the slot together with the dashpots.
// Under HHT-alpha (cal = 1 - alpha != 0) the displacement is d_alpha =
// d_pred - (1-alpha)(dt v + (1/2-beta) dt^2 a) (displ_alpha, solver.f90:
// 106-113, bc_gen.f90:295).
// The boundary forces of the step about to run (it = completed steps + 1),
// one thread per perimeter slot: per_bf[c*nslot + s] (BoundaryForces).
template <typename real>
__global__ void boundary_force_kernel(const BoundaryForces bf, real *per_bf, int ndof, int nslot, const int *step) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslot) return;
  const int it = *step + 1;
  for (int c = 0; c < ndof; ++c) per_bf[c * nslot + s] = real(boundary_force(bf, ndof, nslot, s, c, it));
}

template <typename real>
__global__ void stacey_kernel(real *per_kd, const real *D, const real *V, const real *A, real cal, real dt, real cd2,
                              int nused, const int *slot, const int *ptr, const int *kk, const int *lat,
                              const real *K, const real *H, int N, int nterm, int nslot, long long plane) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 2 * nused) return;
  const int i = q % nused, c = q / nused;
  const real *Dc = D + c * plane, *Vc = V + c * plane, *Ac = A ? A + c * plane : nullptr;
  auto dval = [&](int l) { return cal != real(0) ? Dc[l] - cal * (dt * Vc[l] + cd2 * Ac[l]) : Dc[l]; };
  real acc = real(0);
  for (int t = ptr[i]; t < ptr[i + 1]; ++t) {
    const int k = kk[t];
    const int *L = lat + (size_t)t * N;
    real dd = H[N * k] * dval(L[0]);
    for (int l = 1; l < N; ++l) dd = dd + H[l + N * k] * dval(L[l]);
    acc = acc + K[t + (size_t)nterm * c] * dd;
  }
  per_kd[(size_t)c * nslot + slot[i]] = acc;
}

// Sum of the potency terms of the fault node pairs of the step just
// completed (step counter `step`) into row `it` of the potency series: one
// block, a fixed summation order (strided partial sums, then a tree).
__global__ void potency_kernel(const double *pot, int nflt, double *series, const int *step, int rows) {
  __shared__ double part[6][256];
  const int t = threadIdx.x;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int k = t; k < nflt; k += 256)
    for (int q = 0; q < 6; ++q) acc[q] += pot[(size_t)q * nflt + k];
  for (int q = 0; q < 6; ++q) part[q][t] = acc[q];
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if (t < w)
      for (int q = 0; q < 6; ++q) part[q][t] += part[q][t + w];
    __syncthreads();
  }
  const int it = *step;
  if (t < 6 && it >= 0 && it < rows) series[(size_t)6 * it + t] = part[t][0];
}

// The progress check of main.f90:73-76: max|v| and max|d| over n values
// of each field into info[0], info[1] (atomic max on the bit patterns,
// which order like the values for non-negative doubles); a value that is
// not finite sets the device error flag to SEM2D_E_NAN.
template <typename real>
__global__ void watch_kernel(const real *V, const real *D, long long n, double *info, int *error) {
  double vm = 0.0, dm = 0.0;
  bool bad = false;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const double v = fabs(double(V[q])), d = fabs(double(D[q]));
    bad = bad || !isfinite(v) || !isfinite(d);
    vm = v > vm ? v : vm;
    dm = d > dm ? d : dm;
  }
  for (int o = 16; o > 0; o >>= 1) {
    vm = fmax(vm, __shfl_xor_sync(0xffffffffu, vm, o));
    dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
  }
  bad = __any_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(reinterpret_cast<unsigned long long *>(info), __double_as_longlong(vm));
    atomicMax(reinterpret_cast<unsigned long long *>(info + 1), __double_as_longlong(dm));
    if (bad) atomicCAS(error, 0, SEM2D_E_NAN);
  }
}

// the fields of one batch member for the check
struct WatchSeg {
  const void *V, *D;
  long long n;
};

// the check over every member of a batch in one launch: blockIdx.y is the
// member, the blocks along x stride over its planes
template <typename real>
__global__ void watch_batch_kernel(const WatchSeg *segs, double *info, int *error) {
  const WatchSeg sg = segs[blockIdx.y];
  const real *V = static_cast<const real *>(sg.V), *D = static_cast<const real *>(sg.D);
  double vm = 0.0, dm = 0.0;
  bool bad = false;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < sg.n; q += (long long)gridDim.x * blockDim.x) {
    const double v = fabs(double(V[q])), d = fabs(double(D[q]));
    bad = bad || !isfinite(v) || !isfinite(d);
    vm = v > vm ? v : vm;
    dm = d > dm ? d : dm;
  }
  for (int o = 16; o > 0; o >>= 1) {
    vm = fmax(vm, __shfl_xor_sync(0xffffffffu, vm, o));
    dm = fmax(dm, __shfl_xor_sync(0xffffffffu, dm, o));
  }
  bad = __any_sync(0xffffffffu, bad);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(reinterpret_cast<unsigned long long *>(info), __double_as_longlong(vm));
    atomicMax(reinterpret_cast<unsigned long long *>(info + 1), __double_as_longlong(dm));
    if (bad) atomicCAS(error, 0, SEM2D_E_NAN);
  }
}

// the check after the step just queued, over the problem or every member
// of a batch (their maxima combined)
int launch_watch(sem2d_handle *h) {
  CK(cudaMemsetAsync(h->d_info, 0, 2 * sizeof(double), h->stream));
  if (!h->subs.empty() && h->steps > 0 && h->subs.size() <= 65535) {
    const int nsim = int(h->subs.size());
    int per = 0;  // blocks per member: about four waves over the batch
    long long nmax = 0;
    for (sem2d_handle *m : h->subs) nmax = std::max(nmax, (long long)m->plane * m->ndof);
    per = int(std::min<long long>((nmax + 255) / 256, std::max(1, 4 * 152 * 4 / nsim)));
    if (!h->d_watch[0]) {
      for (int par = 0; par < 2; ++par) {  // h->cur == par after the step
        std::vector<WatchSeg> segs(nsim);
        for (int i = 0; i < nsim; ++i) {
          sem2d_handle *m = h->subs[i];
          segs[i] = WatchSeg{m->V[par], m->D[1 - par], (long long)m->plane * m->ndof};
        }
        WatchSeg *d = nullptr;
        int st = dupload(h, &d, segs);
        if (st) return st;
        h->d_watch[par] = d;
      }
    }
    const dim3 grid(per, nsim);
    if (h->mixed)
      watch_batch_kernel<float><<<grid, 256, 0, h->stream>>>(static_cast<const WatchSeg *>(h->d_watch[h->cur]),
                                                             h->d_info, h->d_error);
    else
      watch_batch_kernel<double><<<grid, 256, 0, h->stream>>>(static_cast<const WatchSeg *>(h->d_watch[h->cur]),
                                                              h->d_info, h->d_error);
    CK(cudaGetLastError());
    h->launches++;
    h->info_step = h->steps;
    return SEM2D_OK;
  }
  std::vector<sem2d_handle *> probs = h->subs;
  if (probs.empty()) probs.push_back(h);
  for (sem2d_handle *m : probs) {
    // after a step the displacement d^n is the buffer that is not current
    const void *D = h->steps > 0 ? m->D[1 - h->cur] : m->D[h->cur];
    const void *V = m->V[h->cur];
    const long long n = (long long)m->plane * m->ndof;
    const int grid = int(std::min<long long>((n + 255) / 256, 4 * 152));
    if (h->mixed)
      watch_kernel<float><<<grid, 256, 0, h->stream>>>(static_cast<const float *>(V), static_cast<const float *>(D), n,
                                                      h->d_info, h->d_error);
    else
      watch_kernel<double><<<grid, 256, 0, h->stream>>>(static_cast<const double *>(V), static_cast<const double *>(D),
                                                       n, h->d_info, h->d_error);
    CK(cudaGetLastError());
    h->launches++;
  }
  h->info_step = h->steps;
  return SEM2D_OK;
}

int launch_potency(sem2d_handle *h, cudaStream_t s, const int *step) {
  potency_kernel<<<1, 256, 0, s>>>(h->fd[F_POT], h->nflt, h->fd[F_POTSERIES], step, h->nt + 1);
  CK(cudaGetLastError());
  h->launches++;
  return SEM2D_OK;
}

// one step of problem h: the march kernel when it covers the problem, else
// the strip kernel; `receivers` false skips the in-kernel seismograms
int launch_step_kernel(sem2d_handle *h, BulkConfig &bc, bool receivers) {
  if (h->march) {
    bc.rec_ids = receivers ? h->d_march_rec : nullptr;
    MarchLaunch m;
    m.units = h->d_march_units;
    m.nunits = h->march_nunits;
    if (h->march_fault_units) {
      // the fault chunk's units, then the others
      BulkConfig bf = bc;
      bf.step = h->d_step_c;
      bf.done = h->d_done_c;
      MarchLaunch mf = m;
      mf.nunits = h->march_fault_units;
      m.units = static_cast<const int *>(h->d_march_units) + kMarchUnitInts * h->march_fault_units;
      m.nunits = h->march_nunits - h->march_fault_units;
      if (launch_march(bf, mf)) return 1;
    }
    return launch_march(bc, m);
  }
  if (!receivers) bc.rec_tile_start = nullptr;
  return launch_bulk(bc);
}

template <typename real>
int launch_one_step(sem2d_handle *h, int cur, cudaEvent_t *ev = nullptr) {
  FaultParams<real> f;
  BulkConfig bc = make_config<real>(h, cur, f);
  const bool rec = h->nrec && !h->rec_separate;
  if (h->bf.W) {
    const int nslot = perimeter_slots(h->LX, h->LZ);
    boundary_force_kernel<real><<<(nslot + 127) / 128, 128, 0, h->stream>>>(h->bf, (real *)h->per_bf, h->ndof,
                                                                             nslot, h->d_step);
    CK(cudaGetLastError());
    h->launches++;
  }
  if (h->march && h->march_fault_units) {
    // the units reading fault rows, then the others (the timed bulk), then
    // the fault kernel
    bc.rec_ids = rec ? h->d_march_rec : nullptr;
    BulkConfig bf = bc;
    bf.step = h->d_step_c;
    bf.done = h->d_done_c;
    MarchLaunch mf;
    mf.units = h->d_march_units;
    mf.nunits = h->march_fault_units;
    if (h->march_fused) {
      f.step = h->d_step_c;
      if (launch_march_fault_side(bf, mf, h->march_nstrips, h->march_nfch))
        return set_err(h, SEM2D_E_CUDA, std::string("fault side launch: ") + bulk_last_error());
    } else if (launch_march(bf, mf)) {
      return set_err(h, SEM2D_E_CUDA, std::string("bulk launch: ") + bulk_last_error());
    }
    if (ev) CK(cudaEventRecord(ev[0], h->stream));
    MarchLaunch mm;
    mm.units = static_cast<const int *>(h->d_march_units) + kMarchUnitInts * h->march_fault_units;
    mm.nunits = h->march_nunits - h->march_fault_units;
    if (launch_march(bc, mm)) return set_err(h, SEM2D_E_CUDA, std::string("bulk launch: ") + bulk_last_error());
    if (ev) CK(cudaEventRecord(ev[1], h->stream));
    f.step = h->d_step_c;
    if (!h->march_fused && launch_march_fault(bc))
      return set_err(h, SEM2D_E_CUDA, std::string("fault launch: ") + bulk_last_error());
    h->launches += h->march_fused ? 2 : 3;
    if (h->potency && launch_potency(h, h->stream, h->d_step_c)) return SEM2D_E_CUDA;
  } else {
    if (h->st_nslot) {
      const int nthr = 2 * h->st_nslot;
      stacey_kernel<real><<<(nthr + 127) / 128, 128, 0, h->stream>>>(
          (real *)h->per_kd, (const real *)h->D[cur], (const real *)h->V[cur],
          h->scheme == 2 ? (const real *)h->A[cur] : nullptr, real(bc.cal), real(bc.dt), real(bc.cd2), h->st_nslot,
          h->d_st_slot, h->d_st_ptr, h->d_st_k, h->d_st_lat, (const real *)h->d_st_K, (const real *)h->d_st_H,
          h->N, h->st_nterm, perimeter_slots(h->LX, h->LZ), h->plane);
      CK(cudaGetLastError());
      h->launches++;
    }
    if (ev) CK(cudaEventRecord(ev[0], h->stream));
    if (launch_step_kernel(h, bc, rec))
      return set_err(h, SEM2D_E_CUDA, std::string("bulk launch: ") + bulk_last_error());
    h->launches++;
    if (h->nperio) {
      PerioParams<real> pp{};
      pp.LX = h->LX;
      pp.LZ = h->LZ;
      pp.ndof = h->ndof;
      pp.nslot = perimeter_slots(h->LX, h->LZ);
      pp.scheme = h->scheme;
      pp.plane = h->plane;
      pp.pitch = h->pitch;
      pp.pf = (const real *)h->perio_f;
      pp.Dcur = (const real *)h->D[cur];
      pp.Vcur = (const real *)h->V[cur];
      pp.Acur = (const real *)h->A[cur];
      pp.Dnext = (real *)h->D[1 - cur];
      pp.Vnext = (real *)h->V[1 - cur];
      pp.Anext = h->keep_accel ? (real *)h->A[1 - cur] : nullptr;
      pp.per_rm = (const real *)h->per_rm;
      pp.per_Ca = (const real *)h->per_Ca;
      pp.per_Cb = (const real *)h->per_Cb;
      pp.per_dir = h->ndir ? h->per_dir : nullptr;
      pp.per_bf = h->bf.W ? (const real *)h->per_bf : nullptr;
      pp.per_kd = h->st_nslot ? (const real *)h->per_kd : nullptr;
      pp.tb = h->perio_tb;
      pp.dt = real(bc.dt);
      pp.cv = real(bc.cv);
      pp.cpred = real(bc.cpred);
      pp.cpa = real(bc.cpa);
      pp.cd2 = real(bc.cd2);
      pp.cb = real(bc.cb);
      pp.jf1 = h->nflt ? h->jf1 : -1;
      pp.jf2 = h->nflt ? h->jf2 : -1;
      pp.has_fault = h->nflt ? 1 : 0;
      pp.two = h->nflt ? h->two : 0;
      pp.step = h->d_step;
      const int nrow = h->perio_tb ? h->LX : h->LZ;
      perio_kernel<real><<<(nrow + 127) / 128, 128, 0, h->stream>>>(pp, f);
      CK(cudaGetLastError());
      h->launches++;
    }
    if (ev) CK(cudaEventRecord(ev[1], h->stream));
    if (h->nflt && h->potency && launch_potency(h, h->stream, h->d_step)) return SEM2D_E_CUDA;
  }
  if (ev) CK(cudaEventRecord(ev[2], h->stream));
  if (h->nrec && h->rec_separate) {
    RecParams<real> r{};
    r.nrec = h->nrec;
    r.ndof = h->ndof;
    r.nsamp = h->rec_nsamp;
    r.isamp = h->rec_isamp;
    r.npts = h->rec_npts;
    r.plane = h->plane;
    r.lat = h->rec_lat;
    r.w = h->rec_w;
    // after the step: velocity and acceleration are the buffers just written;
    // displacement is the step's predictor plus beta dt^2 times the new
    // acceleration (solver.f90:82)
    r.field = (const real *)(h->rec_field == 'A' ? h->A[1 - cur] : h->rec_field == 'V' ? h->V[1 - cur] : h->D[cur]);
    if (h->rec_field == 'D') {
      r.acc = (const real *)h->A[1 - cur];
      r.cb = real(h->beta * h->dt * h->dt);
    }
    r.sis = h->sis;
    r.step = h->d_step;
    const int nthr = h->nrec * h->ndof;
    receiver_kernel<real><<<(nthr + 127) / 128, 128, 0, h->stream>>>(r);
    CK(cudaGetLastError());
    h->launches++;
  }
  if (ev) CK(cudaEventRecord(ev[3], h->stream));
  return SEM2D_OK;
}

template <typename real>
int launch_batch_step(sem2d_handle *h, cudaEvent_t *ev = nullptr) {
  FaultParams<real> f;
  BulkConfig bc = make_config<real>(h->subs[0], h->cur, f);
  bc.stream = h->stream;
  BatchLaunch b;
  b.params = h->d_params[h->cur];
  b.units = h->d_units;
  b.nunits = h->nunits;
  b.grid = h->batch_grid;
  b.step = h->d_step;
  b.done = h->d_done;
  if (ev) CK(cudaEventRecord(ev[0], h->stream));
  if (h->march) {
    MarchLaunch ml;
    ml.units = h->d_march_units;
    ml.nunits = h->march_nunits;
    ml.sims = h->d_params[h->cur];
    ml.step = h->d_step;
    ml.done = h->d_done;
    if (launch_march_batch(bc, ml))
      return set_err(h, SEM2D_E_CUDA, std::string("batch launch: ") + bulk_last_error());
  } else if (launch_batch(bc, b)) {
    return set_err(h, SEM2D_E_CUDA, std::string("batch launch: ") + bulk_last_error());
  }
  h->launches++;
  if (ev)
    for (int q = 1; q < 4; ++q) CK(cudaEventRecord(ev[q], h->stream));
  return SEM2D_OK;
}

// members follow the batch's step count and buffer parity
void sync_members(sem2d_handle *h) {
  for (sem2d_handle *m : h->subs) {
    m->cur = h->cur;
    m->steps = h->steps;
  }
}

// Steps of a problem with a fault on two streams.  Step k: the fault
// chunk's units (C_k) and then the fault kernel (Q_k) on fstream, the other
// units (M_k) on the main stream.  C_k follows M_{k-1} (it reads the rows
// M_{k-1} wrote) and Q_{k-1} (stream order); M_k follows C_{k-1} but not
// Q_{k-1}: the fault kernel writes only the fault rows, which the chunk
// layout keeps away from every other unit.  So the FP64 fault update of
// step k runs while M_{k+1} computes.
int launch_steps_overlap(sem2d_handle *h, int n) {
  cudaStream_t S = h->stream, F = h->fstream;
  CK(cudaEventRecord(h->ev_m[1], S));
  CK(cudaEventRecord(h->ev_c[1], S));
  for (int k = 0; k < n; ++k) {
    const int q = k & 1;
    FaultParams<float> f;
    BulkConfig bc = make_config<float>(h, h->cur, f);
    const bool rec = h->nrec && !h->rec_separate;
    bc.rec_ids = rec ? h->d_march_rec : nullptr;
    // C_k and Q_k
    CK(cudaStreamWaitEvent(F, h->ev_m[q ^ 1], 0));
    BulkConfig bf = bc;
    bf.step = h->d_step_c;
    bf.done = h->d_done_c;
    bf.stream = F;
    MarchLaunch mf;
    mf.units = h->d_march_units;
    mf.nunits = h->march_fault_units;
    f.step = h->d_step_c;
    if (h->march_fused) {
      if (launch_march_fault_side(bf, mf, h->march_nstrips, h->march_nfch))
        return set_err(h, SEM2D_E_CUDA, std::string("fault side launch: ") + bulk_last_error());
      CK(cudaEventRecord(h->ev_c[q], F));
    } else {
      if (launch_march(bf, mf)) return set_err(h, SEM2D_E_CUDA, std::string("bulk launch: ") + bulk_last_error());
      CK(cudaEventRecord(h->ev_c[q], F));
      if (launch_march_fault(bf)) return set_err(h, SEM2D_E_CUDA, std::string("fault launch: ") + bulk_last_error());
    }
    if (h->potency && launch_potency(h, F, h->d_step_c)) return SEM2D_E_CUDA;
    // M_k
    CK(cudaStreamWaitEvent(S, h->ev_c[q ^ 1], 0));
    MarchLaunch mm;
    mm.units = static_cast<const int *>(h->d_march_units) + kMarchUnitInts * h->march_fault_units;
    mm.nunits = h->march_nunits - h->march_fault_units;
    if (launch_march(bc, mm)) return set_err(h, SEM2D_E_CUDA, std::string("bulk launch: ") + bulk_last_error());
    CK(cudaEventRecord(h->ev_m[q], S));
    h->launches += h->march_fused ? 2 : 3;
    h->cur = 1 - h->cur;
    h->steps++;
  }
  // the main stream ends after the last fault kernel
  CK(cudaEventRecord(h->ev_f, F));
  CK(cudaStreamWaitEvent(S, h->ev_f, 0));
  return SEM2D_OK;
}

int launch_steps(sem2d_handle *h, int n) {
  if (!h->subs.empty()) {
    for (int k = 0; k < n; ++k) {
      const int st = h->mixed ? launch_batch_step<float>(h) : launch_batch_step<double>(h);
      if (st) return st;
      h->cur = 1 - h->cur;
      h->steps++;
    }
    sync_members(h);
    return SEM2D_OK;
  }
  if (h->march_overlap) return launch_steps_overlap(h, n);
  for (int k = 0; k < n; ++k) {
    const int st = h->mixed ? launch_one_step<float>(h, h->cur) : launch_one_step<double>(h, h->cur);
    if (st) return st;
    h->cur = 1 - h->cur;
    h->steps++;
  }
  return SEM2D_OK;
}

int kernels_per_step(const sem2d_handle *h) {
  if (!h->subs.empty()) return 1;
  return 1 + (h->march && h->nflt ? (h->march_fused ? 1 : 2) : 0) + (h->nflt && h->potency ? 1 : 0) +
         (h->nrec && h->rec_separate ? 1 : 0) + (h->st_nslot ? 1 : 0) + (h->nperio ? 1 : 0) + (h->bf.W ? 1 : 0);
}

int ensure_graph(sem2d_handle *h) {
  if (h->graph_exec) return SEM2D_OK;
  const int cur0 = h->cur, steps0 = h->steps;
  const long long l0 = h->launches;
  cudaGraph_t graph;
  CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  int st = launch_steps(h, 2 * kGraphPairs);
  cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
  h->cur = cur0;
  h->steps = steps0;
  h->launches = l0;
  if (st) return st;
  if (e != cudaSuccess) return set_err(h, SEM2D_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&h->graph_exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return set_err(h, SEM2D_E_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return SEM2D_OK;
}

int reset_state(sem2d_handle *h) {
  if (!h->subs.empty()) {
    for (sem2d_handle *m : h->subs) {
      const int st = reset_state(m);
      if (st) return set_err(h, st, m->err);
    }
    CK(cudaMemsetAsync(h->d_step, 0, sizeof(int), h->stream));
    CK(cudaMemsetAsync(h->d_done, 0, sizeof(unsigned), h->stream));
    CK(cudaMemsetAsync(h->d_error, 0, sizeof(int), h->stream));
    CK(cudaMemsetAsync(h->d_info, 0, 2 * sizeof(double), h->stream));
    h->info_step = 0;
    h->cur = 0;
    h->steps = 0;
    sync_members(h);
    return SEM2D_OK;
  }
  const size_t rs = h->mixed ? sizeof(float) : sizeof(double);
  for (int b = 0; b < 2; ++b) {
    CK(cudaMemsetAsync(h->D[b], 0, rs * h->plane * h->ndof, h->stream));
    CK(cudaMemsetAsync(h->V[b], 0, rs * h->plane * h->ndof, h->stream));
    if (h->F[b]) CK(cudaMemsetAsync(h->F[b], 0, rs * h->plane * h->ndof, h->stream));
    if (h->A[b]) CK(cudaMemsetAsync(h->A[b], 0, rs * h->plane * h->ndof, h->stream));
  }
  CK(cudaMemsetAsync(h->d_step, 0, sizeof(int), h->stream));
  CK(cudaMemsetAsync(h->d_done, 0, sizeof(unsigned), h->stream));
  CK(cudaMemsetAsync(h->d_error, 0, sizeof(int), h->stream));
  CK(cudaMemsetAsync(h->d_info, 0, 2 * sizeof(double), h->stream));
  h->info_step = 0;
  if (h->d_step_c) CK(cudaMemsetAsync(h->d_step_c, 0, sizeof(int), h->stream));
  if (h->d_done_c) CK(cudaMemsetAsync(h->d_done_c, 0, sizeof(unsigned), h->stream));
  if (h->sis) CK(cudaMemsetAsync(h->sis, 0, sizeof(double) * (size_t)h->rec_nsamp * h->nrec * h->ndof, h->stream));
  if (h->nflt) {
    const size_t nfd = (size_t)h->nflt * h->ndof;
    for (int a : {F_D64, F_V64, F_A64}) CK(cudaMemsetAsync(h->fd[a], 0, sizeof(double) * 2 * nfd, h->stream));
    for (int a : {F_D}) CK(cudaMemsetAsync(h->fd[a], 0, sizeof(double) * nfd, h->stream));
    for (int a : {F_T, F_TSTICK}) CK(cudaMemsetAsync(h->fd[a], 0, sizeof(double) * 2 * h->nflt, h->stream));
    CK(cudaMemcpyAsync(h->fd[F_V], h->h_fault_init.data(), sizeof(double) * nfd, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemcpyAsync(h->fd[F_THETA], h->h_fault_init.data() + nfd, sizeof(double) * h->nflt,
                       cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->fd[F_SERIES], 0, sizeof(double) * (size_t)h->onx * 6 * std::max(h->fnsamp, 1), h->stream));
    if (h->potency) CK(cudaMemsetAsync(h->fd[F_POTSERIES], 0, sizeof(double) * 6 * ((size_t)h->nt + 1), h->stream));
  }
  h->cur = 0;
  h->steps = 0;
  h->ckpt_saved = -1;
  int st = h->mixed ? launch_fault_init<float>(h) : launch_fault_init<double>(h);
  return st;
}

int check_device_error(sem2d_handle *h) {
  int e = 0;
  CK(cudaStreamSynchronize(h->stream));
  for (sem2d_handle *m : h->subs) {
    const int st = check_device_error(m);
    if (st) return set_err(h, st, m->err);
  }
  CK(cudaMemcpy(&e, h->d_error, sizeof(int), cudaMemcpyDeviceToHost));
  if (e == SEM2D_E_NR) return set_err(h, SEM2D_E_NR, "rate-and-state Newton solver did not converge");
  if (e == SEM2D_E_TIMEOUT) return set_err(h, SEM2D_E_TIMEOUT, "a bounded wait for shared-memory copies expired");
  if (e == SEM2D_E_NAN)
    return set_err(h, SEM2D_E_NAN, "non-finite velocity or displacement found by the check every info_every steps");
  if (e) return set_err(h, e, "device error");
  return SEM2D_OK;
}

// force_tz > 0 sets the chunk height (batch members share one);
// `shared` is a stream owned by a batch
// element row owning lattice row J (lower-left ownership): the highest
// element row starting at or below J
int owner_row(const sem2d_handle *h, int J) {
  const int ez = int(std::upper_bound(h->row0.begin(), h->row0.begin() + h->nz, J) - h->row0.begin()) - 1;
  return std::max(0, std::min(ez, h->nz - 1));
}

// frees a device buffer allocated with dalloc/dupload before destroy
void dfree(sem2d_handle *h, void *p) {
  if (!p) return;
  cudaFree(p);
  h->allocs.erase(std::remove(h->allocs.begin(), h->allocs.end(), p), h->allocs.end());
}

// Work units of the march kernel for chunk height cz (element rows): the
// element rows reading a fault row (those touching one and the row above
// them, which reads the upper fault row as its halo) are chunks of one row
// each and come first, with no chunk boundary inside or right above them,
// so that only the fault chunk reads fault rows; the others are cut every
// cz rows.  Receivers sampled inside the kernel are grouped by unit.
// Replaces the units of an earlier call.
int build_march_units(sem2d_handle *h, int cz) {
  const int nstrips = (h->nx + kMarchColsHost - 1) / kMarchColsHost;
  cz = std::max(1, std::min(cz, h->nz));
  const std::vector<int> &rec_ex = h->march_rec_ex, &rec_ez = h->march_rec_ez;
  // element rows touching a fault row; no chunk boundary inside them or
  // right above them, so that only the fault chunk reads fault rows
  int t0 = h->nz, t1 = -1;
  if (h->nflt)
    for (int z = 0; z < h->nz; ++z) {
      const int a = h->row0[z], b = a + h->N - 1;
      if ((h->jf1 >= a && h->jf1 <= b) || (h->two && h->jf2 >= a && h->jf2 <= b)) {
        t0 = std::min(t0, z);
        t1 = std::max(t1, z);
      }
    }
  // chunks: the element rows reading a fault row (those touching one and
  // the row above them, which reads the upper fault row as its halo) are
  // chunks of one row each and come first; the others are cut every cz rows
  std::vector<int> zb, order;
  int nfch = 0;
  if (t1 >= 0) {
    const int f0 = t0, f1 = std::min(t1 + 2, h->nz);
    for (int z = 0; z < f0; z += cz) zb.push_back(z);
    for (int z = f0; z < f1; ++z) zb.push_back(z);
    for (int z = f1; z < h->nz; z += cz) zb.push_back(z);
    nfch = f1 - f0;
  } else {
    for (int z = 0; z < h->nz; z += cz) zb.push_back(z);
  }
  zb.push_back(h->nz);
  const int nch = int(zb.size()) - 1;
  std::vector<int> pos(nch);
  for (int y = 0; y < nch; ++y)
    if (t1 >= 0 && zb[y] >= t0 && zb[y] < t1 + 2) order.push_back(y);
  for (int y = 0; y < nch; ++y)
    if (!(t1 >= 0 && zb[y] >= t0 && zb[y] < t1 + 2)) order.push_back(y);
  for (int k = 0; k < nch; ++k) pos[order[k]] = k;
  std::vector<int> chunk_of(h->nz);
  for (int y = 0; y < nch; ++y)
    for (int z = zb[y]; z < zb[y + 1]; ++z) chunk_of[z] = y;
  const int nu = nch * nstrips;
  // receivers sampled inside the kernel, grouped by unit
  std::vector<int> cnt(nu + 1, 0), ids;
  std::vector<int> unit_of;
  if (h->nrec && !h->rec_separate) {
    unit_of.resize(h->nrec);
    for (int r = 0; r < h->nrec; ++r) {
      unit_of[r] = pos[chunk_of[rec_ez[r]]] * nstrips + rec_ex[r] / kMarchColsHost;
      cnt[unit_of[r] + 1]++;
    }
  }
  for (int k = 0; k < nu; ++k) cnt[k + 1] += cnt[k];
  ids.resize(std::max(cnt[nu], 1));
  {
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (size_t r = 0; r < unit_of.size(); ++r) ids[fill[unit_of[r]]++] = int(r);
  }
  std::vector<int> units((size_t)nu * kMarchUnitInts);
  for (int k = 0; k < nch; ++k)
    for (int sx = 0; sx < nstrips; ++sx) {
      const int u = k * nstrips + sx, y = order[k];
      int *U = &units[(size_t)u * kMarchUnitInts];
      U[0] = 0;
      U[1] = sx;
      U[2] = zb[y];
      U[3] = zb[y + 1];
      U[4] = cnt[u];
      U[5] = cnt[u + 1];
    }
  dfree(h, h->d_march_units);
  dfree(h, h->d_march_rec);
  h->d_march_units = nullptr;
  h->d_march_rec = nullptr;
  int *du = nullptr, st;
  if ((st = dupload(h, &du, units)) || (st = dupload(h, &h->d_march_rec, ids))) return st;
  h->d_march_units = du;
  h->march_units_host = units;
  h->march_nunits = nu;
  h->march_cz = cz;
  h->march_nstrips = nstrips;
  h->march_nfch = nfch;
  h->march_fault_units = nfch * nstrips;
  return SEM2D_OK;
}


// Work units of the march kernel: strips of 31 element columns by chunks of
// element rows.  The chunk height gives about two units per resident warp
// (SEM2D_MARCH_CZ overrides it); a two-sided fault's rows stay in one chunk,
// whose units come first (their FP64 fault work is the longest).
// SEM2D_MARCH=0 keeps the strip kernel.
int setup_march(sem2d_handle *h, const std::vector<int> &rec_ex, const std::vector<int> &rec_ez,
                const std::vector<int> &rec_jn, int force_cz) {
  h->march = false;
  const char *env = std::getenv("SEM2D_MARCH");
  if (env && std::atoi(env) == 0) return SEM2D_OK;
  // Stacey, Dirichlet or periodic sides, a grid that is not flat: the strip kernel
  if (h->st_nslot || h->ndir || h->nperio || h->general) return SEM2D_OK;
  BulkConfig bc;
  bc.N = h->N;
  bc.ndof = h->ndof;
  bc.mixed = h->mixed;
  bc.fast = fast_path(h);
  bc.mat_iso = h->mat_iso;
  bc.mat_elem = h->mat_elem;
  bc.pitch = h->pitch;
  bc.plane = h->plane;
  if (!march_supported(bc)) return SEM2D_OK;
  if (const char *e = std::getenv("SEM2D_MARCH_WARPS")) h->march_warps = std::atoi(e);
  // with a fault the elastic force is the state: the displacement next to
  // a slipped fault is too large for FP32 to resolve the dynamic stress
  const char *fs = std::getenv("SEM2D_FORCE_STATE");
  h->march_fst = (h->nflt > 0 || h->static_load) && !(fs && std::atoi(fs) == 0);
  bc.march_warps = h->march_warps;
  bc.march_fst = h->march_fst;
  // resident warps per SM
  const int warps_per_sm = march_warps_per_sm(bc);
  if (warps_per_sm <= 0) return set_err(h, SEM2D_E_CUDA, std::string("march kernel: ") + bulk_last_error());
  int st;
  if (h->nflt) {
    // the fault kernel finishes the fault rows after the step: velocity or
    // acceleration receivers there, and displacement ones when the Newmark
    // corrector adds beta dt^2 a, are sampled after it, by the receiver
    // kernel
    const bool corrected = h->scheme == 2 || (h->scheme == 1 && h->beta != 0.0);
    for (size_t r = 0; r < rec_jn.size(); ++r)
      if ((h->rec_field != 'D' || corrected) && (rec_jn[r] == h->jf1 || rec_jn[r] == h->jf2))
        h->rec_separate = true;
    if ((st = dalloc(h, &h->d_fault_force, (size_t)2 * h->ndof * h->nflt))) return st;
  }
  if (h->march_fst)
    for (int b = 0; b < 2; ++b) {
      float *q = nullptr;
      if ((st = dalloc(h, &q, (size_t)h->plane * h->ndof))) return st;
      h->F[b] = q;
    }
  const int nstrips = (h->nx + kMarchColsHost - 1) / kMarchColsHost;
  int cz = 0;
  if (const char *e = std::getenv("SEM2D_MARCH_CZ")) cz = std::atoi(e);
  if (cz <= 0) cz = force_cz;
  if (cz <= 0) {
    int dev = 0, nsm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    const long long target = 2LL * nsm * warps_per_sm;
    cz = int(((long long)nstrips * h->nz + target - 1) / target);
  }
  h->march_rec_ex = rec_ex;
  h->march_rec_ez = rec_ez;
  if ((st = build_march_units(h, cz))) return st;
  h->march = true;
  const int nfch = h->march_nfch;
  if (nfch > 0) {
    const char *fu = std::getenv("SEM2D_FUSED_FAULT");
    h->march_fused = nfch <= kMarchWarpsHost && h->friction != SEM2D_FRICTION_RSF && !(fu && std::atoi(fu) == 0);
    if ((st = dalloc(h, &h->d_step_c, 1)) || (st = dalloc(h, &h->d_done_c, 1))) return st;
    const char *ov = std::getenv("SEM2D_OVERLAP");
    // the boundary-force table of a step is written before the step on the
    // main stream, which the two-stream schedule does not order
    h->march_overlap = !h->rec_separate && !h->bf.W && !(ov && std::atoi(ov) == 0);
    if (h->march_overlap) {
      CK(cudaStreamCreateWithFlags(&h->fstream, cudaStreamNonBlocking));
      for (int q = 0; q < 2; ++q) {
        CK(cudaEventCreateWithFlags(&h->ev_m[q], cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->ev_c[q], cudaEventDisableTiming));
      }
      CK(cudaEventCreateWithFlags(&h->ev_f, cudaEventDisableTiming));
    }
  }
  return SEM2D_OK;
}

int build_batch_tables(sem2d_handle *h);

// ---- the autotuner of the march kernels' launch shape ----------------
// The first handle of a class of problems (dof count, material layout,
// node count and member count to a power of two, SM count) times candidate
// shapes -- chunk height and warps per CTA -- over a few steps with CUDA
// events, keeps the fastest (the analytic
// default unless another is faster by more than 2 %) and records it in the
// tuning cache (autotune.cpp); later handles of the class read it.  The
// shapes give bitwise identical results (the per-node summation order does
// not depend on them), and the state is reset after the trial steps.
// SEM2D_AUTOTUNE=0, or SEM2D_MARCH_CZ / SEM2D_MARCH_WARPS, keeps the
// analytic shape.
struct MarchShape {
  int cz, warps;
};

bool tune_disabled() {
  const char *t = std::getenv("SEM2D_AUTOTUNE");
  if (t && std::atoi(t) == 0) return true;
  for (const char *v : {"SEM2D_MARCH_CZ", "SEM2D_MARCH_WARPS"})
    if (std::getenv(v)) return true;
  return false;
}

int apply_shape(sem2d_handle *h, const MarchShape &s) {
  int st;
  std::vector<sem2d_handle *> probs = h->subs;
  if (probs.empty()) probs.push_back(h);
  for (sem2d_handle *m : probs) {
    if (s.cz != m->march_cz && (st = build_march_units(m, s.cz))) return st;
    m->march_warps = s.warps;
  }
  if (!h->subs.empty() && (st = build_batch_tables(h))) return st;
  h->march_warps = s.warps;
  if (h->graph_exec) {  // a captured graph holds the old units
    cudaGraphExecDestroy(h->graph_exec);
    h->graph_exec = nullptr;
  }
  return SEM2D_OK;
}

// milliseconds per step of n steps after nwarm warm-up steps (direct launches)
int time_shape(sem2d_handle *h, int nwarm, int n, double *ms) {
  int st;
  if ((st = launch_steps(h, nwarm))) return st;
  cudaEvent_t e0, e1;
  CK(cudaEventCreate(&e0));
  CK(cudaEventCreate(&e1));
  CK(cudaEventRecord(e0, h->stream));
  st = launch_steps(h, n);
  CK(cudaEventRecord(e1, h->stream));
  CK(cudaEventSynchronize(e1));
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = double(t) / n;
  return st;
}

// The launch shape of a class of problems: from the tuning cache when it
// holds the class, else timed on the handle's first run of at least
// kTuneSteps steps (tune_on_run).
constexpr int kTuneWarm = 1, kTuneTimed = 16, kTuneShapes = 5;
constexpr int kTuneSteps = kTuneShapes * (kTuneWarm + kTuneTimed);

bool tune_key(const sem2d_handle *h, char *key, size_t n) {
  const sem2d_handle *a = h->subs.empty() ? h : h->subs[0];
  long long nodes = 0;
  if (h->subs.empty()) nodes = h->npoin;
  for (const sem2d_handle *m : h->subs) nodes += m->npoin;
  int dev = 0, nsm = 1;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return false;
  return sem2d_tune_key(a->ndof, a->mat_elem, nodes, int(h->subs.size()), nsm, key, n) == SEM2D_OK;
}

int tune_march(sem2d_handle *h) {
  // a rate-and-state fault keeps the analytic shape: its step time is set as
  // much by the Newton solves on the second stream, and the shape timed on
  // the first steps (the fault at rest) was slower over the run
  if (!h->march || tune_disabled() || (h->nflt > 0 && h->friction == SEM2D_FRICTION_RSF)) return SEM2D_OK;
  char key[160], path[1024];
  if (!tune_key(h, key, sizeof(key))) return SEM2D_OK;
  sem2d_tune_entry e;
  if (sem2d_tune_cache_path(path, sizeof(path)) == SEM2D_OK && sem2d_tune_lookup(path, key, &e) == 1) {
    h->tune_source = 2;
    return apply_shape(h, MarchShape{e.chunk_rows, e.warps_per_cta});
  }
  h->tune_pending = 1;
  return SEM2D_OK;
}

// Times the candidate shapes on the run's own first kTuneSteps steps (every
// shape gives the same bits, so these are steps of the solution), keeps the
// fastest unless the analytic one is within 2 %, and records it in the
// tuning cache.
int tune_on_run(sem2d_handle *h) {
  h->tune_pending = 0;
  const sem2d_handle *a = h->subs.empty() ? h : h->subs[0];
  const int cz0 = a->march_cz;
  const MarchShape cands[kTuneShapes] = {{cz0, a->march_warps}, {cz0, 1}, {2 * cz0, a->march_warps},
                                         {std::max(1, cz0 / 2), a->march_warps}, {4 * cz0, a->march_warps}};
  std::vector<sem2d_tune_entry> res(kTuneShapes);
  int st;
  for (int k = 0; k < kTuneShapes; ++k) {
    double ms = 0;
    if ((st = apply_shape(h, cands[k])) || (st = time_shape(h, kTuneWarm, kTuneTimed, &ms))) return st;
    res[k] = sem2d_tune_entry{std::max(1, std::min(cands[k].cz, a->nz)), cands[k].warps, ms};
  }
  const int best = sem2d_tune_select(res.data(), kTuneShapes, 0.02);
  if ((st = apply_shape(h, cands[best]))) return st;
  h->tune_source = 1;
  char key[160], path[1024];
  if (tune_key(h, key, sizeof(key)) && sem2d_tune_cache_path(path, sizeof(path)) == SEM2D_OK)
    sem2d_tune_record(path, key, &res[best]);  // a cache that cannot be written is not an error
  return SEM2D_OK;
}

int create_impl(sem2d_handle *h, const sem2d_problem_desc *d, cudaStream_t shared = nullptr,
                int force_tz = 0) {
  if (d->ngll != 3 && d->ngll != 5 && d->ngll != 6 && d->ngll != 9)
    return set_err(h, SEM2D_E_UNSUPPORTED, "GPU kernels are compiled for ngll in {3, 5, 6, 9}");
  if (d->ndof != 1 && d->ndof != 2) return set_err(h, SEM2D_E_ARG, "ndof must be 1 or 2");
  if (d->nelem <= 0 || d->npoin <= 0 || !d->ibool || !d->coord || !d->hprime || !d->wgll || !d->rmass ||
      !d->Kx || !d->Kz || !d->la || !d->mu || !d->mux)
    return set_err(h, SEM2D_E_ARG, "incomplete descriptor");
  if (!(d->dt > 0) || d->nt < 0) return set_err(h, SEM2D_E_ARG, "bad time step settings");
  if (d->precision != SEM2D_PRECISION_FP64 && d->precision != SEM2D_PRECISION_MIXED)
    return set_err(h, SEM2D_E_ARG, "unknown precision");
  h->N = d->ngll;
  h->ndof = d->ndof;
  h->nelem = d->nelem;
  h->npoin = d->npoin;
  h->nt = d->nt;
  h->mixed = d->precision == SEM2D_PRECISION_MIXED;
  h->scheme = d->time_scheme == SEM2D_TIME_NEWMARK ? 1 : d->time_scheme == SEM2D_TIME_HHT ? 2 : 0;
  if (d->time_scheme != SEM2D_TIME_LEAPFROG && !h->scheme) return set_err(h, SEM2D_E_ARG, "unknown time scheme");
  h->dt = d->dt;
  h->beta = d->beta;
  h->gamma = h->scheme ? d->gamma : 0.5;
  h->alpha = h->scheme == 2 ? d->alpha : 1.0;
  if (h->scheme == 2 && !(h->alpha >= 0.0 && h->alpha <= 1.0)) return set_err(h, SEM2D_E_ARG, "alpha out of [0,1]");
  h->keep_accel = h->scheme != 0 || d->rec_field == 'A';
  h->nr_maxit = d->flt_nr_maxit > 0 ? d->flt_nr_maxit : 200;
  h->info_every = d->info_every == 0 ? 100 : d->info_every;
  if (const char *e = std::getenv("SEM2D_SPIN_LIMIT")) h->spin_limit = std::max(0, std::atoi(e));
  if (shared) {
    h->stream = shared;
    h->owns_stream = false;
  } else {
    CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  }
  int st;
  if ((st = detect_lattice(h, d))) return st;
  if ((st = upload_fault(h, d))) return st;
  if ((st = upload_material(h, d))) return st;
  if ((st = upload_mass_and_boundaries(h, d))) return st;
  {
    FaultScalars &fs = h->fs;
    fs.coefA2V = d->flt_coefA2V;
    fs.coefA2D = d->flt_coefA2D;
    fs.normal_V = d->normal_V;
    fs.normal_T = d->normal_T;
    fs.normal_L = d->normal_L;
    fs.opening = d->flt_opening;
    fs.swf_kind = d->swf_kind;
    fs.swf_healing = d->swf_healing;
    fs.rsf_kind = d->rsf_kind;
    fs.normal_kind = d->normal_kind;
    fs.oit = d->flt_oit;
    fs.oitd = d->flt_oitd > 0 ? d->flt_oitd : 1;
    fs.oix1 = d->flt_oix1 > 0 ? d->flt_oix1 : 1;
    fs.oixd = d->flt_oixd > 0 ? d->flt_oixd : 1;
    fs.twf_kind = d->twf_kind;
    if (d->nflt > 0 && d->flt_friction == SEM2D_FRICTION_TWF && fs.twf_kind == 0) fs.twf_kind = 1;
    fs.twf_mus = d->twf_mus;
    fs.twf_mud = d->twf_mud;
    fs.twf_mu0 = d->twf_mu0;
    fs.twf_X = d->twf_X;
    fs.twf_Z = d->twf_Z;
    fs.twf_V = d->twf_V;
    fs.twf_L = d->twf_L;
    fs.twf_T = d->twf_T;
    fs.twf_Dc = d->twf_Dc;
  }
  const size_t rs = h->mixed ? sizeof(float) : sizeof(double);
  for (int b = 0; b < 2; ++b) {
    char *p;
    if ((st = dalloc(h, &p, rs * h->plane * h->ndof))) return st;
    h->D[b] = p;
    if ((st = dalloc(h, &p, rs * h->plane * h->ndof))) return st;
    h->V[b] = p;
    if (h->keep_accel) {
      if ((st = dalloc(h, &p, rs * h->plane * h->ndof))) return st;
      h->A[b] = p;
    }
  }
  if ((st = dupload(h, &h->d_row0, h->row0))) return st;
  if ((st = dalloc(h, &h->d_step, 1)) || (st = dalloc(h, &h->d_error, 1)) || (st = dalloc(h, &h->d_done, 1)) ||
      (st = dalloc(h, &h->d_info, 2)))
    return st;
  h->H.assign(d->hprime, d->hprime + h->N * h->N);
  h->w.assign(d->wgll, d->wgll + h->N);
  h->kd2 = d->kd2_form ? 1 : 0;
  h->width = d->width > 0 ? d->width : 0.0;
  // sources: lattice position and per-step amplitude (SO_add, src_gen.f90:290-317)
  h->nsrc = d->nsrc;
  if (h->nsrc > kMaxSrc) return set_err(h, SEM2D_E_UNSUPPORTED, "too many sources");
  if (h->nsrc) {
    std::vector<int> sI(h->nsrc), sJ(h->nsrc);
    std::vector<double> amp((size_t)h->nsrc * h->ndof * (h->nt + 1), 0.0);
    // a time function other than Ricker, evaluated on the host
    StfDev hs{};
    std::vector<double> hv2;
    if (d->src_stf) {
      if (const char *m = stf_check(*d->src_stf)) return set_err(h, SEM2D_E_ARG, m);
      h->static_load = h->static_load || d->src_stf->kind != SEM2D_STF_RICKER;
      const sem2d_stf &q = *d->src_stf;
      hs = StfDev{q.kind, q.ntab, q.f0, q.onset, q.ampli, q.par1, q.par2, q.tab_t, q.tab_v, nullptr};
      if (q.kind == SEM2D_STF_TAB) {
        hv2 = stf_spline_d2(q.tab_t, q.tab_v, q.ntab);
        hs.v2 = hv2.data();
      }
    }
    for (int s = 0; s < h->nsrc; ++s) {
      const int p = d->src_node[s] - 1;
      if (p < 0 || p >= d->npoin) return set_err(h, SEM2D_E_ARG, "source node out of range");
      sI[s] = int(h->glob2lat[p] % h->pitch);
      sJ[s] = int(h->glob2lat[p] / h->pitch);
      const double td = d->src_tdelay ? d->src_tdelay[s] : 0.0, rel = d->src_relamp ? d->src_relamp[s] : 1.0;
      for (int it = 1; it <= h->nt; ++it) {
        // HHT-alpha adds the sources at t + (alpha-1) dt (solver.f90:116-117)
        const double t = it * d->dt + (h->alpha - 1.0) * d->dt;
        double a = d->src_stf ? stf_value(hs, t - td) : ricker(t - td, d->src_f0[s], d->src_t0[s], d->src_ampli[s]);
        a = a * rel;
        for (int c = 0; c < h->ndof; ++c)
          amp[((size_t)s * h->ndof + c) * (h->nt + 1) + it] = h->ndof == 1 ? a : d->src_dir[2 * s + c] * a;
      }
    }
    if ((st = dupload(h, &h->src_I, sI)) || (st = dupload(h, &h->src_J, sJ)) || (st = dupload(h, &h->src_amp, amp)))
      return st;
  }
  // receivers
  h->nrec = d->nrec;
  if (h->nrec) {
    h->rec_isamp = d->rec_isamp > 0 ? d->rec_isamp : 1;
    h->rec_nsamp = d->rec_nsamp;
    h->rec_field = d->rec_field;
    if (h->rec_field != 'D' && h->rec_field != 'V' && h->rec_field != 'A')
      return set_err(h, SEM2D_E_ARG, "rec_field must be D, V or A");
    if (!d->rec_node && (!d->rec_elem || !d->rec_interp))
      return set_err(h, SEM2D_E_ARG, "receivers need nodes or interpolation");
    h->rec_npts = d->rec_node ? 1 : h->N * h->N;
    // interpolated velocity/acceleration (and displacement with the Newmark
    // corrector, which needs the new accelerations) reads nodes owned by
    // several CTAs: sampled by a separate kernel after the step; everything
    // else is sampled inside the bulk kernel by the CTA that owns the receiver
    h->rec_separate = !d->rec_node && (h->rec_field != 'D' || h->scheme == 2 || (h->scheme == 1 && h->beta != 0.0));
  }
  if ((st = dalloc(h, &h->sis, (size_t)std::max(h->rec_nsamp, 1) * std::max(h->nrec, 1) * h->ndof))) return st;
  std::vector<int> rec_ex, rec_ez, rec_jn;  // element owning each receiver (march units), node row
  // strips of TX element columns by chunks of element rows, fault split kept inside a chunk
  h->TX = strip_width(h->N);
  if (h->TX <= 0) return set_err(h, SEM2D_E_UNSUPPORTED, "NGLL not compiled");
  h->nplanes = strip_plane_count(h->ndof, h->nmat, h->mat_elem, h->scheme);
  {
    BulkConfig bc;
    bc.N = h->N;
    bc.ndof = h->ndof;
    bc.mixed = h->mixed;
    bc.nplanes = h->nplanes;
    bc.nmat = h->nmat;
    bc.has_kv = h->has_kv;
    bc.mat_elem = h->mat_elem;
    bc.mat_iso = h->mat_iso;
    bc.fast = fast_path(h);
    bc.nx = h->nx;
    bc.nz = h->nz;
    if (force_tz > 0) h->TZ = std::min(std::min(force_tz, kMaxChunkRows), h->nz);
    else if (choose_tiles(bc, h->row0.data(), &h->TZ))
      return set_err(h, SEM2D_E_UNSUPPORTED, std::string("no strip configuration fits: ") + bulk_last_error());
  }
  h->ztile = tile_rows(h->N, h->nz, h->row0.data(), h->TZ);
  h->fault_chunk = 0;
  if (h->nflt)
    for (size_t y = 0; y + 1 < h->ztile.size(); ++y)
      if (h->row0[h->ztile[y]] <= h->jf1 && h->jf1 < h->row0[h->ztile[y + 1]]) h->fault_chunk = int(y);
  for (size_t y = 0; y + 1 < h->ztile.size(); ++y)
    if (h->ztile[y + 1] - h->ztile[y] + 1 > 2 * kMaxChunkRows + 1)
      return set_err(h, SEM2D_E_UNSUPPORTED, "element-row chunk too tall");
  if ((st = dupload(h, &h->d_ztile, h->ztile))) return st;
  if (h->nrec) {
    // receiver lattice positions; for the fused path, grouped by owning tile
    const int gx = (h->nx + h->TX - 1) / h->TX, gy = int(h->ztile.size()) - 1;
    std::vector<int> tileJ(h->LZ, -1);  // lattice row -> tile row owning it
    for (int y = 0; y < gy; ++y)
      for (int J = h->row0[h->ztile[y]]; J < h->row0[h->ztile[y + 1]]; ++J) tileJ[J] = y;
    std::vector<int> etile(h->nz, -1);
    for (int y = 0; y < gy; ++y)
      for (int z = h->ztile[y]; z < h->ztile[y + 1]; ++z) etile[z] = y;
    std::vector<int> rI, rJ, lat, owner(h->nrec);
    std::vector<double> w;
    rec_ex.assign(h->nrec, 0);
    rec_ez.assign(h->nrec, 0);
    rec_jn.assign(h->nrec, -1);
    const int NN = h->N * h->N;
    for (int r = 0; r < h->nrec; ++r) {
      if (d->rec_node) {
        const int p = d->rec_node[r] - 1;
        if (p < 0 || p >= d->npoin) return set_err(h, SEM2D_E_ARG, "receiver node out of range");
        const long long L = h->glob2lat[p];
        const int I = int(L % h->pitch), J = int(L / h->pitch);
        rI.push_back(I);
        rJ.push_back(J);
        lat.push_back(int(L));
        w.push_back(1.0);
        const int x = std::min(I / (h->TX * (h->N - 1)), gx - 1);
        owner[r] = tileJ[J] * gx + x;
        rec_ex[r] = std::min(I / (h->N - 1), h->nx - 1);
        rec_ez[r] = owner_row(h, J);
        rec_jn[r] = J;
      } else {
        const int e = d->rec_elem[r] - 1;
        if (e < 0 || e >= d->nelem) return set_err(h, SEM2D_E_ARG, "receiver element out of range");
        for (int q = 0; q < NN; ++q) {
          const long long L = h->glob2lat[d->ibool[q + (size_t)NN * e] - 1];
          rI.push_back(int(L % h->pitch));
          rJ.push_back(int(L / h->pitch));
          lat.push_back(int(L));
          w.push_back(d->rec_interp[q + (size_t)NN * r]);
        }
        owner[r] = etile[h->elem_ez[e]] * gx + h->elem_ex[e] / h->TX;
        rec_ex[r] = h->elem_ex[e];
        rec_ez[r] = h->elem_ez[e];
      }
    }
    // node receivers on periodic columns (rows) are sampled after the periodic pass
    if (h->nperio && d->rec_node)
      for (int r = 0; r < h->nrec; ++r)
        if (h->perio_tb ? (rJ[r] == 0 || rJ[r] == h->LZ - 1) : (rI[r] == 0 || rI[r] == h->LX - 1))
          h->rec_separate = true;
    std::vector<int> start(gx * gy + 1, 0), ids(h->nrec);
    for (int r = 0; r < h->nrec; ++r) start[owner[r] + 1]++;
    for (int k = 0; k < gx * gy; ++k) start[k + 1] += start[k];
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int r = 0; r < h->nrec; ++r) ids[fill[owner[r]]++] = r;
    if ((st = dupload(h, &h->rec_lat, lat)) || (st = dupload(h, &h->rec_w, w)) ||
        (st = dupload(h, &h->rec_I, rI)) || (st = dupload(h, &h->rec_J, rJ)) ||
        (st = dupload(h, &h->rec_tile_start, start)) || (st = dupload(h, &h->rec_ids, ids)))
      return st;
  }
  {
    BulkConfig bc;
    bc.N = h->N;
    bc.ndof = h->ndof;
    bc.mixed = h->mixed;
    bc.nplanes = h->nplanes;
    bc.nmat = h->nmat;
    bc.has_kv = h->has_kv;
    bc.mat_elem = h->mat_elem;
    bc.mat_iso = h->mat_iso;
    bc.fast = fast_path(h);
    if (configure_bulk(bc)) return set_err(h, SEM2D_E_CUDA, bulk_last_error());
  }
  if ((st = setup_march(h, rec_ex, rec_ez, rec_jn, force_tz))) return st;
  if (!h->march && !shared && h->mixed && (h->nflt > 0 || h->static_load) && h->scheme == 0 && !h->has_kv &&
      !h->adjoint) {
    const char *fs = std::getenv("SEM2D_FORCE_STATE");
    if (!(fs && std::atoi(fs) == 0)) {
      for (int b = 0; b < 2; ++b) {
        float *q = nullptr;
        if ((st = dalloc(h, &q, (size_t)h->plane * h->ndof))) return st;
        h->F[b] = q;
      }
      h->strip_fst = 1;
    }
  }
  if ((st = reset_state(h))) return st;
  if (!shared && (st = tune_march(h))) return st;  // batch members are tuned with their batch
  CK(cudaStreamSynchronize(h->stream));
  return SEM2D_OK;
}

}  // namespace

namespace {

constexpr int kBatchChunk = 16;  // element rows per chunk of a batch member

int batch_open_impl(sem2d_handle *h) {
  CK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
  h->batch_open = true;
  return SEM2D_OK;
}

int batch_add_impl(sem2d_handle *h, const sem2d_problem_desc *d) {
  auto m = new (std::nothrow) sem2d_handle();
  if (!m) return set_err(h, SEM2D_E_NOMEM, "out of host memory");
  m->owner = h;
  h->subs.push_back(m);
  int st;
  try {
    st = create_impl(m, d, h->stream, kBatchChunk);
  } catch (const std::bad_alloc &) {
    m->err = "out of host memory";
    st = SEM2D_E_NOMEM;
  }
  if (st) {
    const std::string e = m->err;
    h->subs.pop_back();
    m->owner = nullptr;
    sem2d_gpu_destroy(m);
    return set_err(h, st, "problem " + std::to_string(h->subs.size()) + ": " + e);
  }
  // the members' host-side copies of the mesh numbering are not needed again
  std::vector<int>().swap(m->elem_ex);
  std::vector<int>().swap(m->elem_ez);
  return SEM2D_OK;
}

// Members added together: each is set up (lattice recovery, conversion of
// the description's arrays to device planes, uploads) on one of up to
// SEM2D_HOST_THREADS host threads (default: the hardware threads, at most
// 16), all enqueueing on the batch's stream; the members join the batch in
// the order given.  On failure nothing is added and the first failing
// member is named.
int batch_add_parallel(sem2d_handle *h, const sem2d_problem_desc *descs, int n) {
  std::vector<sem2d_handle *> ms(n, nullptr);
  for (int i = 0; i < n; ++i) {
    ms[i] = new (std::nothrow) sem2d_handle();
    if (!ms[i]) {
      for (sem2d_handle *m : ms) delete m;
      return set_err(h, SEM2D_E_NOMEM, "out of host memory");
    }
    ms[i]->owner = h;
  }
  std::vector<int> st(n, SEM2D_OK);
  std::atomic<int> next{0};
  auto work = [&]() {
    for (int i; (i = next.fetch_add(1)) < n;) {
      try {
        st[i] = create_impl(ms[i], &descs[i], h->stream, kBatchChunk);
      } catch (const std::bad_alloc &) {
        ms[i]->err = "out of host memory";
        st[i] = SEM2D_E_NOMEM;
      } catch (...) {  // nothing may leave a worker thread
        ms[i]->err = "host exception while setting the member up";
        st[i] = SEM2D_E_NOMEM;
      }
      if (!st[i]) {
        std::vector<int>().swap(ms[i]->elem_ex);
        std::vector<int>().swap(ms[i]->elem_ez);
      }
    }
  };
  int nthr = int(std::thread::hardware_concurrency());
  if (const char *e = std::getenv("SEM2D_HOST_THREADS"))
    if (std::atoi(e) > 0) nthr = std::atoi(e);
  nthr = std::max(1, std::min({nthr > 0 ? nthr : 1, 16, n}));
  std::vector<std::thread> pool;
  try {
    for (int t = 1; t < nthr; ++t) pool.emplace_back(work);
  } catch (const std::system_error &) {
    // fewer threads than asked: the calling thread does the rest
  }
  work();
  for (std::thread &t : pool) t.join();
  int bad = -1;
  for (int i = 0; i < n && bad < 0; ++i)
    if (st[i]) bad = i;
  if (bad >= 0) {
    const std::string e = ms[bad]->err;
    for (sem2d_handle *m : ms) {
      m->owner = nullptr;
      sem2d_gpu_destroy(m);
    }
    return set_err(h, st[bad], "problem " + std::to_string(h->subs.size() + bad) + ": " + e);
  }
  h->subs.insert(h->subs.end(), ms.begin(), ms.end());
  return SEM2D_OK;
}

// The parameter blocks of every member of a batch for both buffer
// parities and the batch's list of march units (member by member); replaces
// those of an earlier call (the tuner rebuilds them for each shape).
int build_batch_tables(sem2d_handle *h) {
  const int nsim = int(h->subs.size());
  int st;
  const size_t pb = params_bytes(h->N, h->mixed);
  for (int cur = 0; cur < 2; ++cur) {
    std::vector<unsigned char> blk(pb * nsim);
    for (int i = 0; i < nsim; ++i) {
      sem2d_handle *m = h->subs[i];
      if (h->mixed) {
        FaultParams<float> f;
        BulkConfig bc = make_config<float>(m, cur, f);
        if (h->march) bc.rec_ids = m->nrec ? m->d_march_rec : nullptr;
        fill_params_block(bc, blk.data() + pb * i);
      } else {
        FaultParams<double> f;
        BulkConfig bc = make_config<double>(m, cur, f);
        fill_params_block(bc, blk.data() + pb * i);
      }
    }
    dfree(h, h->d_params[cur]);
    h->d_params[cur] = nullptr;
    if ((st = dupload(h, reinterpret_cast<unsigned char **>(&h->d_params[cur]), blk))) return st;
  }
  if (h->march) {
    std::vector<int> mu;
    for (int i = 0; i < nsim; ++i) {
      const std::vector<int> &src = h->subs[i]->march_units_host;
      for (size_t k = 0; k < src.size(); k += kMarchUnitInts) {
        mu.insert(mu.end(), src.begin() + k, src.begin() + k + kMarchUnitInts);
        mu[mu.size() - kMarchUnitInts] = i;
      }
    }
    h->march_nunits = int(mu.size() / kMarchUnitInts);
    dfree(h, h->d_march_units);
    h->d_march_units = nullptr;
    int *du = nullptr;
    if ((st = dupload(h, &du, mu))) return st;
    h->d_march_units = du;
    h->march_cz = h->subs[0]->march_cz;
  }
  return SEM2D_OK;
}

int batch_close_impl(sem2d_handle *h) {
  const int nsim = int(h->subs.size());
  if (nsim <= 0) return set_err(h, SEM2D_E_ARG, "empty batch");
  const sem2d_handle *a = h->subs[0];
  for (const sem2d_handle *m : h->subs) {
    if (m->N != a->N || m->ndof != a->ndof || m->mixed != a->mixed || m->mat_elem != a->mat_elem ||
        m->nplanes != a->nplanes || fast_path(m) != fast_path(a) || m->mat_iso != a->mat_iso ||
        m->has_kv != a->has_kv || m->scheme != a->scheme)
      return set_err(h, SEM2D_E_UNSUPPORTED,
                     "batch members differ in NGLL, dof count, precision, scheme or material layout");
    if (m->nt != a->nt) return set_err(h, SEM2D_E_UNSUPPORTED, "batch members differ in the number of steps");
    if (m->nrec && m->rec_separate)
      return set_err(h, SEM2D_E_UNSUPPORTED, "interpolated velocity/acceleration receivers in a batch");
    if (m->potency) return set_err(h, SEM2D_E_UNSUPPORTED, "fault potency records in a batch");
    if (m->st_nslot) return set_err(h, SEM2D_E_UNSUPPORTED, "Stacey absorbing boundaries in a batch");
    if (m->ndir) return set_err(h, SEM2D_E_UNSUPPORTED, "Dirichlet sides in a batch");
    if (m->nperio) return set_err(h, SEM2D_E_UNSUPPORTED, "periodic sides in a batch");
    if (m->bf.W) return set_err(h, SEM2D_E_UNSUPPORTED, "incident waves or Neumann tractions in a batch");
    if (m->general) return set_err(h, SEM2D_E_UNSUPPORTED, "a grid that is not flat in a batch");
  }
  h->N = a->N;
  h->ndof = a->ndof;
  h->mixed = a->mixed;
  h->nt = a->nt;
  h->scheme = a->scheme;
  h->TX = a->TX;
  h->TZ = a->TZ;
  // the march kernel runs the batch when it covers every member and none
  // has a fault (the fault kernel is per problem)
  h->march = true;
  for (const sem2d_handle *m : h->subs) h->march = h->march && m->march && !m->nflt;
  int st;
  if ((st = dalloc(h, &h->d_step, 1)) || (st = dalloc(h, &h->d_error, 1)) || (st = dalloc(h, &h->d_done, 1)) ||
      (st = dalloc(h, &h->d_info, 2)))
    return st;
  if ((st = build_batch_tables(h))) return st;
  // work units of the strip kernel, member by member
  std::vector<int> units;
  for (int i = 0; i < nsim; ++i) {
    const sem2d_handle *m = h->subs[i];
    const int gx = (m->nx + m->TX - 1) / m->TX, gy = int(m->ztile.size()) - 1;
    for (int yy = 0; yy < gy; ++yy) {
      const int y = (yy + m->fault_chunk) % gy;  // the fault's chunk first
      for (int x = 0; x < gx; ++x) units.insert(units.end(), {i, x, y, gx});
    }
  }
  h->nunits = int(units.size() / 4);
  if ((st = dupload(h, reinterpret_cast<int **>(&h->d_units), units))) return st;
  BulkConfig bc;
  bc.N = h->N;
  bc.ndof = h->ndof;
  bc.mixed = h->mixed;
  bc.nplanes = a->nplanes;
  bc.nmat = a->nmat;
  bc.has_kv = a->has_kv;
  bc.mat_elem = a->mat_elem;
  bc.mat_iso = a->mat_iso;
  bc.fast = fast_path(a);
  const int per_sm = occupancy_bulk(bc);
  if (per_sm <= 0) return set_err(h, SEM2D_E_CUDA, std::string("no resident CTA: ") + bulk_last_error());
  int dev = 0, nsm = 1;
  CK(cudaGetDevice(&dev));
  CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  h->batch_grid = std::min(h->nunits, per_sm * nsm);
  if ((st = reset_state(h))) return st;
  if ((st = tune_march(h))) return st;
  CK(cudaStreamSynchronize(h->stream));
  h->batch_open = false;
  return SEM2D_OK;
}

}  // namespace

namespace sem2d_detail {
// Strain and stress at the element GLL points (MAT_strain_PSV/SH,
// mat_gen.f90:727-774; MAT_ELAST_stress, mat_elastic.f90:804-862) on the
// rectilinear lattice: dxi/dy = deta/dx = 0, so e11 = dUx/dxi dxi/dx,
// e22 = dUz/deta deta/dz, e12 = (dUx/deta deta/dz + dUz/dxi dxi/dx)/2
// (SH: e13 = dU/dxi dxi/dx / 2, e23 = dU/deta deta/dz / 2).  One thread per
// element point; out[((ez*nx + ex)*N*N + i + N*j)*(ndof+1) + c].
template <typename real>
__global__ void strain_stress_kernel(const real *D, int ndof, int N, int nx, int nz, int pitch, long long plane,
                                     const int *row0, const real *xix, const real *etaz, const double *H,
                                     int mat_elem, int iso, const real *m0, const real *m1, const real *m2,
                                     const real *m3, const real *V, const real *kveta, double *eo, double *so) {
  const long long npt = (long long)nx * nz * N * N;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < npt;
       q += (long long)gridDim.x * blockDim.x) {
    const int pt = int(q % (N * N));
    const long long el = q / (N * N);
    const int i = pt % N, j = pt / N, ex = int(el % nx), ez = int(el / nx);
    const long long base = (long long)row0[ez] * pitch + (long long)ex * (N - 1);
    const double dxi = double(xix[ex]), deta = double(etaz[ez]);
    double gx[2] = {0, 0}, ge[2] = {0, 0}, kx[2] = {0, 0}, ke[2] = {0, 0};
    // the stress of a Kelvin-Voigt element is that of d + eta v
    // (MAT_stress_dv, mat_gen.f90:626-641)
    const real *eta = kveta ? kveta + el * N * N : nullptr;
    for (int c = 0; c < ndof; ++c) {
      const real *u = D + c * plane + base;
      double a = H[0 + N * i] * double(u[(long long)j * pitch + 0]);
      for (int k = 1; k < N; ++k) a = a + H[k + N * i] * double(u[(long long)j * pitch + k]);
      double b = double(u[(long long)0 * pitch + i]) * H[0 + N * j];
      for (int k = 1; k < N; ++k) b = b + double(u[(long long)k * pitch + i]) * H[k + N * j];
      gx[c] = a;
      ge[c] = b;
      kx[c] = a;
      ke[c] = b;
      if (eta) {
        const real *w = V + c * plane + base;
        auto uk = [&](int ii, int jj) {
          return double(u[(long long)jj * pitch + ii]) + double(eta[ii + N * jj]) * double(w[(long long)jj * pitch + ii]);
        };
        double ak = H[0 + N * i] * uk(0, j), bk = uk(i, 0) * H[0 + N * j];
        for (int k = 1; k < N; ++k) ak = ak + H[k + N * i] * uk(k, j);
        for (int k = 1; k < N; ++k) bk = bk + uk(i, k) * H[k + N * j];
        kx[c] = ak;
        ke[c] = bk;
      }
    }
    auto mat = [&](const real *m) -> double {
      if (!m) return 0.0;
      if (mat_elem == kMatElement) return double(m[el]);
      if (mat_elem == kMatPoint) return double(m[el * N * N + pt]);
      return double(m[base + (long long)j * pitch + i]);
    };
    double *e = eo + q * (ndof + 1), *s = so + q * (ndof + 1);
    if (ndof == 1) {
      const double mu = mat(m0);  // SH: mu (the reference has no anisotropic SH stress)
      e[0] = 0.5 * (gx[0] * dxi);
      e[1] = 0.5 * (ge[0] * deta);
      s[0] = 2.0 * mu * (0.5 * (kx[0] * dxi));
      s[1] = 2.0 * mu * (0.5 * (ke[0] * deta));
    } else {
      double Kx, Kz, la, mu;
      if (iso) {
        la = mat(m0);
        mu = mat(m1);
        Kx = la + 2.0 * mu;
        Kz = Kx;
      } else {
        Kx = mat(m0);
        Kz = mat(m1);
        la = mat(m2);
        mu = mat(m3);
      }
      e[0] = gx[0] * dxi;
      e[1] = ge[1] * deta;
      e[2] = 0.5 * (ge[0] * deta + gx[1] * dxi);
      const double k0 = kx[0] * dxi, k1 = ke[1] * deta, k2 = 0.5 * (ke[0] * deta + kx[1] * dxi);
      s[0] = Kx * k0 + la * k1;
      s[1] = la * k0 + Kz * k1;
      s[2] = 2.0 * mu * k2;
    }
  }
}

// out = d + cb a over n values: the Newmark corrector of the displacement
// (solver.f90:82) for the outputs read between steps
template <typename real>
__global__ void corrector_kernel(real *out, const real *d, const real *a, real cb, long long n) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
    out[q] = d[q] + cb * a[q];
}
}  // namespace sem2d_detail

extern "C" {

int sem2d_stf_eval(const sem2d_stf *stf, int n, const double *t, double *out) {
  if (!stf || n < 0 || (n > 0 && (!t || !out))) return SEM2D_E_ARG;
  if (const char *m = stf_check(*stf)) {
    sem2d::set_library_error(m);
    return SEM2D_E_ARG;
  }
  StfDev hs{stf->kind, stf->ntab, stf->f0, stf->onset, stf->ampli, stf->par1, stf->par2, stf->tab_t, stf->tab_v,
            nullptr};
  std::vector<double> v2;
  if (stf->kind == SEM2D_STF_TAB) {
    v2 = stf_spline_d2(stf->tab_t, stf->tab_v, stf->ntab);
    hs.v2 = v2.data();
  }
  for (int k = 0; k < n; ++k) out[k] = stf_value(hs, t[k]);
  return SEM2D_OK;
}

int sem2d_gpu_version(void) { return SEM2D_GPU_ABI_VERSION; }

int sem2d_gpu_batch_open(sem2d_handle **out) {
  if (!out) {
    g_create_err = "null argument";
    return SEM2D_E_ARG;
  }
  *out = nullptr;
  auto h = new (std::nothrow) sem2d_handle();
  if (!h) {
    g_create_err = "out of host memory";
    return SEM2D_E_NOMEM;
  }
  const int st = batch_open_impl(h);
  if (st) {
    g_create_err = h->err;
    sem2d_gpu_destroy(h);
    return st;
  }
  *out = h;
  return SEM2D_OK;
}

int sem2d_gpu_batch_add(sem2d_handle *h, const sem2d_problem_desc *desc) {
  if (!h || !desc) return SEM2D_E_ARG;
  if (!h->batch_open) return set_err(h, SEM2D_E_STATE, "not an open batch");
  return batch_add_impl(h, desc);
}

int sem2d_gpu_batch_add_many(sem2d_handle *h, const sem2d_problem_desc *descs, int n) {
  if (!h || (!descs && n > 0) || n < 0) return SEM2D_E_ARG;
  if (!h->batch_open) return set_err(h, SEM2D_E_STATE, "not an open batch");
  if (n == 0) return SEM2D_OK;
  try {
    return batch_add_parallel(h, descs, n);
  } catch (const std::exception &) {
    return set_err(h, SEM2D_E_NOMEM, "out of host resources");
  }
}

int sem2d_gpu_batch_close(sem2d_handle *h) {
  if (!h) return SEM2D_E_ARG;
  if (!h->batch_open) return set_err(h, SEM2D_E_STATE, "not an open batch");
  int st;
  try {
    st = batch_close_impl(h);
  } catch (const std::bad_alloc &) {
    st = set_err(h, SEM2D_E_NOMEM, "out of host memory");
  }
  return st;
}

int sem2d_gpu_create_batch(const sem2d_problem_desc *descs, int nsim, sem2d_handle **out) {
  if (!descs || !out || nsim <= 0) {
    g_create_err = "null argument or empty batch";
    return SEM2D_E_ARG;
  }
  int st = sem2d_gpu_batch_open(out);
  if (st) return st;
  try {
    st = batch_add_parallel(*out, descs, nsim);
  } catch (const std::exception &) {
    st = set_err(*out, SEM2D_E_NOMEM, "out of host resources");
  }
  if (!st) st = sem2d_gpu_batch_close(*out);
  if (st) {
    g_create_err = (*out)->err;
    sem2d_gpu_destroy(*out);
    *out = nullptr;
  }
  return st;
}

int sem2d_gpu_batch_size(sem2d_handle *h) { return h ? int(h->subs.size()) : SEM2D_E_ARG; }

sem2d_handle *sem2d_gpu_batch_member(sem2d_handle *h, int i) {
  if (!h || i < 0 || i >= int(h->subs.size())) return nullptr;
  return h->subs[i];
}

int sem2d_gpu_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return SEM2D_E_CUDA;
  return n;
}

int sem2d_gpu_create(const sem2d_problem_desc *desc, sem2d_handle **out) {
  if (!desc || !out) {
    g_create_err = "null argument";
    return SEM2D_E_ARG;
  }
  *out = nullptr;
  auto h = new (std::nothrow) sem2d_handle();
  if (!h) {
    g_create_err = "out of host memory";
    return SEM2D_E_NOMEM;
  }
  int st;
  try {
    st = create_impl(h, desc);
  } catch (const std::bad_alloc &) {
    h->err = "out of host memory";
    st = SEM2D_E_NOMEM;
  }
  if (st) {
    g_create_err = h->err;
    sem2d_gpu_destroy(h);
    return st;
  }
  *out = h;
  return SEM2D_OK;
}

}  // extern "C"

namespace {

int step_impl(sem2d_handle *h, int nsteps) {
  int st;
  int left = nsteps;
  if (h->tune_pending && left >= kTuneSteps) {
    if ((st = tune_on_run(h))) return st;
    left -= kTuneSteps;
  }
  const char *nog = std::getenv("SEM2D_NO_GRAPH");
  const bool use_graph = !(nog && nog[0] == '1');
  // align to even parity, then replay captured runs
  if (use_graph && left >= 2 * kGraphPairs) {
    if (h->cur != 0) {
      if ((st = launch_steps(h, 1))) return st;
      --left;
    }
    if ((st = ensure_graph(h))) return st;
    while (left >= 2 * kGraphPairs) {
      CK(cudaGraphLaunch(h->graph_exec, h->stream));
      h->steps += 2 * kGraphPairs;
      h->launches += (long long)2 * kGraphPairs * kernels_per_step(h);
      left -= 2 * kGraphPairs;
    }
  }
  if (left && (st = launch_steps(h, left))) return st;
  sync_members(h);
  return SEM2D_OK;
}

// copies the current state (next displacement predictor, velocity) into
// checkpoint slot k
int save_checkpoint(sem2d_handle *h, int k) {
  const size_t n = (h->mixed ? sizeof(float) : sizeof(double)) * (size_t)h->plane * h->ndof;
  char *slot = static_cast<char *>(h->ckpt[k]);
  CK(cudaMemcpyAsync(slot, h->D[h->cur], n, cudaMemcpyDeviceToDevice, h->stream));
  CK(cudaMemcpyAsync(slot + n, h->V[h->cur], n, cudaMemcpyDeviceToDevice, h->stream));
  h->ckpt_saved = k;
  return SEM2D_OK;
}

}  // namespace

extern "C" {

int sem2d_gpu_step(sem2d_handle *h, int nsteps) {
  if (!h) return SEM2D_E_ARG;
  if (h->owner) return set_err(h, SEM2D_E_STATE, "a batch member is stepped through its batch");
  if (h->batch_open) return set_err(h, SEM2D_E_STATE, "the batch is still open");
  if (nsteps < 0) return set_err(h, SEM2D_E_ARG, "negative step count");
  if (h->steps + nsteps > h->nt) return set_err(h, SEM2D_E_ARG, "stepping beyond nt");
  // runs of steps end at every checkpoint (the state of every
  // ckpt_every-th step is kept for the adjoint) and at every check of
  // max|v|, max|d| (every info_every steps)
  const int ie = h->subs.empty() ? h->info_every : h->subs[0]->info_every;
  int st, left = nsteps;
  if (h->ckpt_every > 0 && h->steps == 0 && (st = save_checkpoint(h, 0))) return st;
  while (left > 0) {
    int n = left;
    if (h->ckpt_every > 0) n = std::min(n, h->ckpt_every - h->steps % h->ckpt_every);
    if (ie > 0) n = std::min(n, ie - h->steps % ie);
    if ((st = step_impl(h, n))) return st;
    left -= n;
    if (h->ckpt_every > 0 && h->steps % h->ckpt_every == 0 && (st = save_checkpoint(h, h->steps / h->ckpt_every)))
      return st;
    if (ie > 0 && h->steps % ie == 0 && (st = launch_watch(h))) return st;
  }
  return SEM2D_OK;
}

int sem2d_gpu_get_info(sem2d_handle *h, int *step, double *vmax, double *dmax) {
  if (!h) return SEM2D_E_ARG;
  sem2d_handle *b = h->owner ? h->owner : h;
  double v[2] = {0.0, 0.0};
  CK(cudaStreamSynchronize(b->stream));
  CK(cudaMemcpy(v, b->d_info, sizeof(v), cudaMemcpyDeviceToHost));
  if (step) *step = b->info_step;
  if (vmax) *vmax = v[0];
  if (dmax) *dmax = v[1];
  return SEM2D_OK;
}

int sem2d_gpu_checkpoint_every(sem2d_handle *h, int every) {
  if (!h) return SEM2D_E_ARG;
  if (!h->adjoint) return set_err(h, SEM2D_E_STATE, "the handle was not created for the gradient workflow");
  if (h->steps != 0) return set_err(h, SEM2D_E_STATE, "checkpoints are set before the first step");
  for (void *q : h->ckpt) {
    cudaFree(q);
    h->allocs.erase(std::remove(h->allocs.begin(), h->allocs.end(), q), h->allocs.end());
  }
  h->ckpt.clear();
  h->ckpt_every = every > 0 ? every : 0;
  h->ckpt_saved = -1;
  if (!h->ckpt_every) return SEM2D_OK;
  const size_t n = (h->mixed ? sizeof(float) : sizeof(double)) * (size_t)h->plane * h->ndof;
  for (int k = 0; k <= h->nt / h->ckpt_every; ++k) {
    char *q = nullptr;
    const int st = dalloc(h, &q, 2 * n, false);
    if (st) return st;
    h->ckpt.push_back(q);
  }
  return SEM2D_OK;
}

// out[q * npoin + p] = lat[q * plane + g2l[p]] for the three gradients
static __global__ void gather_nodes_kernel(const double *lat, long long plane, const long long *g2l, int npoin,
                                           double *out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npoin) return;
  const long long L = g2l[p];
  for (int q = 0; q < 3; ++q) out[(size_t)q * npoin + p] = lat[q * plane + L];
}

// The library's pool for per-call device scratch (the adjoint): memory
// freed into it stays reserved for the next call of the process.
static cudaMemPool_t scratch_pool() {
  static std::once_flag once;
  static cudaMemPool_t pool = nullptr;
  std::call_once(once, [] {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return;
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    cudaMemPool_t p = nullptr;
    if (cudaMemPoolCreate(&p, &props) != cudaSuccess) return;
    unsigned long long keep = ~0ull;
    cudaMemPoolSetAttribute(p, cudaMemPoolAttrReleaseThreshold, &keep);
    pool = p;
  });
  return pool;
}

int sem2d_gpu_adjoint(sem2d_handle *h, const double *resid, double *grad_rho, double *grad_vp,
                      double *grad_vs) {
  if (!h || !resid) return SEM2D_E_ARG;
  if (!h->adjoint || !h->rho_plane) return set_err(h, SEM2D_E_STATE, "the handle was not created for the gradient workflow");
  if (h->ckpt_every <= 0 || h->steps != h->nt || h->ckpt_saved != h->nt / h->ckpt_every)
    return set_err(h, SEM2D_E_STATE, "run all nt steps with checkpoints first (sem2d_gpu_checkpoint_every)");
  if (h->N != 5 || h->nflt || h->scheme != 0 || h->has_kv || h->width > 0 || !h->mat_iso ||
      h->mat_elem != kMatNode || h->st_nslot || h->ndir || h->nperio || h->bf.W)
    return set_err(h, SEM2D_E_UNSUPPORTED,
                   "the adjoint covers NGLL=5, isotropic node material, leapfrog, no fault, KV, 2.5D, Stacey "
                   "or Dirichlet sides, incident wave or Neumann traction");
  if (h->nrec && (h->rec_npts != 1 || (h->rec_field != 'V' && h->rec_field != 'D')))
    return set_err(h, SEM2D_E_UNSUPPORTED, "the adjoint needs receivers at nodes recording V or D");
  int st = check_device_error(h);
  if (st) return st;
  const size_t rs = h->mixed ? sizeof(float) : sizeof(double);
  const size_t fbytes = rs * (size_t)h->plane * h->ndof;
  const int k = h->ckpt_every, nd = h->ndof, nslot = perimeter_slots(h->LX, h->LZ);
  // the call's device scratch comes from the library's stream-ordered pool,
  // which keeps its memory between calls (the ring of one shot is several
  // GB: cudaMalloc and cudaFree of it per call cost about a forward step
  // per reverse segment on the 8-shot workload)
  cudaMemPool_t pool = scratch_pool();
  if (!pool) return set_err(h, SEM2D_E_CUDA, "no memory pool for the adjoint");
  std::vector<void *> tmp;
  auto alloc_raw = [&](size_t bytes, bool zero) -> void * {
    void *q = nullptr;
    if (cudaMallocFromPoolAsync(&q, bytes, pool, h->stream) != cudaSuccess) return nullptr;
    tmp.push_back(q);
    if (zero) cudaMemsetAsync(q, 0, bytes, h->stream);
    return q;
  };
  auto alloc = [&](size_t bytes) { return alloc_raw(bytes, true); };
  auto release = [&]() {
    for (void *q : tmp) cudaFreeAsync(q, h->stream);
    cudaStreamSynchronize(h->stream);
    tmp.clear();
  };
  // ring of recomputed forward states: slot j holds (after step n0+j) the
  // displacement predictor, velocity and acceleration (written by the
  // recomputation before any read)
  std::vector<void *> RD(k + 1), RV(k + 1), RA(k + 1);
  for (int j = 1; j <= k; ++j) {
    RD[j] = alloc_raw(fbytes, false);
    RV[j] = alloc_raw(fbytes, false);
    RA[j] = alloc_raw(fbytes, false);
    if (!RD[j] || !RV[j] || !RA[j]) {
      release();
      return set_err(h, SEM2D_E_NOMEM, "no device memory for the recomputed segment");
    }
  }
  void *Dbar[2] = {alloc(fbytes), alloc(fbytes)}, *Vbar[2] = {alloc(fbytes), alloc(fbytes)};
  void *g_la = alloc(rs * h->plane), *g_mu = alloc(rs * h->plane), *g_M = alloc(rs * h->plane);
  void *g_C = alloc(rs * (size_t)nd * nslot);
  double *a_la = (double *)alloc(8 * h->plane), *a_mu = (double *)alloc(8 * h->plane);
  double *a_M = (double *)alloc(8 * h->plane), *a_C = (double *)alloc(8 * (size_t)nd * nslot);
  double *grads = (double *)alloc(8 * 3 * (size_t)h->plane);
  const size_t nres = (size_t)std::max(h->rec_nsamp, 1) * std::max(h->nrec, 1) * nd;
  double *d_resid = (double *)alloc(8 * nres);
  if (!Dbar[0] || !Dbar[1] || !Vbar[0] || !Vbar[1] || !g_la || !g_mu || !g_M || !g_C || !a_la || !a_mu ||
      !a_M || !a_C || !grads || !d_resid) {
    release();
    return set_err(h, SEM2D_E_NOMEM, "no device memory for the adjoint");
  }
  if (h->nrec)
    CK(cudaMemcpyAsync(d_resid, resid, 8 * (size_t)h->rec_nsamp * h->nrec * nd, cudaMemcpyHostToDevice, h->stream));
  AdjConfig ac;
  ac.ndof = nd;
  ac.mixed = h->mixed;
  ac.grid_x = (h->nx + h->TX - 1) / h->TX;
  ac.grid_y = int(h->ztile.size()) - 1;
  ac.LX = h->LX;
  ac.LZ = h->LZ;
  ac.pitch = h->pitch;
  ac.plane = h->plane;
  ac.nx = h->nx;
  ac.nz = h->nz;
  ac.row0 = h->d_row0;
  ac.ztile = h->d_ztile;
  ac.H = h->H.data();
  ac.w = h->w.data();
  for (int q = 0; q < 4; ++q) ac.geo[q] = h->geo[q];
  ac.nmat = h->nmat;
  ac.mat[0] = h->mat[0];
  ac.mat[1] = h->nmat > 1 ? h->mat[1] : nullptr;
  ac.rmass = h->rmass;
  ac.per_rm = h->per_rm;
  ac.per_Ca = h->per_Ca;
  ac.per_Cb = h->per_Cb;
  ac.g_la = g_la;
  ac.g_mu = g_mu;
  ac.g_M = g_M;
  ac.g_C = g_C;
  ac.nrec = h->nrec;
  ac.nsamp = h->rec_nsamp;
  ac.isamp = h->rec_isamp;
  ac.field = h->rec_field;
  ac.rec_I = h->rec_I;
  ac.rec_J = h->rec_J;
  ac.resid = d_resid;
  ac.dt = h->dt;
  ac.kd2 = h->kd2;
  ac.error = h->d_error;
  ac.stream = h->stream;
  if (configure_adjoint(ac)) {
    release();
    return set_err(h, SEM2D_E_CUDA, std::string("adjoint: ") + bulk_last_error());
  }
  // the march passes find the receivers of a lattice row through a CSR index
  MarchAdjConfig mc;
  if (h->march) {
    mc.g_la = g_la;
    mc.g_mu = g_mu;
    mc.g_M = g_M;
    mc.g_C = g_C;
    mc.nrec = h->nrec;
    mc.nsamp = h->rec_nsamp;
    mc.isamp = h->rec_isamp;
    mc.field = h->rec_field;
    mc.rec_I = h->rec_I;
    mc.rec_J = h->rec_J;
    mc.resid = d_resid;
    mc.units = h->d_march_units;
    mc.nunits = h->march_nunits;
  }
  // march path: the adjoint state (lambda, w) in (Dbar, Vbar); the step's
  // configuration is the forward one on those planes, sources and
  // receivers off
  FaultParams<float> f_none;
  auto adj_config = [&](int c) {
    BulkConfig bc = make_config<float>(h, h->cur, f_none);
    bc.Dcur = Dbar[c];
    bc.Vcur = Vbar[c];
    bc.Dnext = Dbar[1 - c];
    bc.Vnext = Vbar[1 - c];
    bc.Acur = bc.Anext = nullptr;
    bc.Fcur = bc.Fnext = nullptr;
    bc.march_fst = 0;
    bc.nsrc = 0;
    bc.rec_nrec = 0;
    bc.rec_ids = nullptr;
    bc.sis = nullptr;
    bc.per_bf = nullptr;
    bc.has_fault = 0;
    bc.flt = nullptr;
    return bc;
  };
  if (h->march) {
    mc.it = h->nt;
    int nl = 0;
    if (launch_march_adjoint_seed(adj_config(0), mc, &nl))
      st = set_err(h, SEM2D_E_CUDA, std::string("adjoint: ") + bulk_last_error());
    h->launches += nl;
  }
  int ca = 0;
  const int nseg = (h->nt + k - 1) / k;
  for (int seg = nseg - 1; seg >= 0 && !st; --seg) {
    const int n0 = seg * k, n1 = std::min(n0 + k, h->nt);
    const size_t half = fbytes;
    RD[0] = h->ckpt[seg];
    RV[0] = static_cast<char *>(h->ckpt[seg]) + half;
    // recompute the forward steps n0+1 .. n1 of the segment
    const int s0 = n0;
    CK(cudaMemcpyAsync(h->d_step, &s0, sizeof(int), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int n = n0 + 1; n <= n1 && !st; ++n) {
      const int j = n - n0;
      if (h->mixed) {
        FaultParams<float> f;
        BulkConfig bc = make_config<float>(h, h->cur, f);
        bc.Dcur = RD[j - 1];
        bc.Vcur = RV[j - 1];
        bc.Dnext = RD[j];
        bc.Vnext = RV[j];
        bc.Anext = RA[j];
        st = launch_step_kernel(h, bc, false) ? set_err(h, SEM2D_E_CUDA, bulk_last_error()) : SEM2D_OK;
      } else {
        FaultParams<double> f;
        BulkConfig bc = make_config<double>(h, h->cur, f);
        bc.Dcur = RD[j - 1];
        bc.Vcur = RV[j - 1];
        bc.Dnext = RD[j];
        bc.Vnext = RV[j];
        bc.Anext = RA[j];
        st = launch_step_kernel(h, bc, false) ? set_err(h, SEM2D_E_CUDA, bulk_last_error()) : SEM2D_OK;
      }
      h->launches++;
    }
    // reverse steps n1 .. n0+1
    for (int n = n1; n > n0 && !st; --n) {
      const int j = n - n0;
      ac.Db = Dbar[ca];
      ac.Vb = Vbar[ca];
      ac.Dbn = Dbar[1 - ca];
      ac.Vbn = Vbar[1 - ca];
      ac.d = RD[j - 1];
      ac.vprev = RV[j - 1];
      ac.a = RA[j];
      ac.it = n;
      if (h->march) {
        mc.d = ac.d;
        mc.vprev = ac.vprev;
        mc.a = ac.a;
        mc.it = n;
        int nl = 0;
        if (launch_march_adjoint(adj_config(ca), mc, &nl))
          st = set_err(h, SEM2D_E_CUDA, std::string("adjoint: ") + bulk_last_error());
        h->launches += nl;
      } else {
        if (launch_adjoint(ac)) st = set_err(h, SEM2D_E_CUDA, std::string("adjoint: ") + bulk_last_error());
        h->launches++;
      }
      ca = 1 - ca;
    }
    if (!st && (launch_fold(g_la, a_la, h->plane, h->mixed, h->stream) ||
                launch_fold(g_mu, a_mu, h->plane, h->mixed, h->stream) ||
                launch_fold(g_M, a_M, h->plane, h->mixed, h->stream) ||
                launch_fold(g_C, a_C, (long long)nd * nslot, h->mixed, h->stream)))
      st = set_err(h, SEM2D_E_CUDA, bulk_last_error());
  }
  if (!st) {
    ChainConfig cc;
    cc.ndof = nd;
    cc.mixed = h->mixed;
    cc.LX = h->LX;
    cc.LZ = h->LZ;
    cc.pitch = h->pitch;
    cc.dt = h->dt;
    cc.rho = h->rho_plane;
    cc.la = nd == 2 ? h->mat[0] : nullptr;
    cc.mu = nd == 2 ? h->mat[1] : h->mat[0];
    cc.rmass = h->rmass;
    cc.per_rm = h->per_rm;
    cc.per_Ca = h->per_Ca;
    cc.per_Cb = h->per_Cb;
    cc.g_la = a_la;
    cc.g_mu = a_mu;
    cc.g_M = a_M;
    cc.g_C = a_C;
    cc.grad_rho = grads;
    cc.grad_vp = grads + h->plane;
    cc.grad_vs = grads + 2 * h->plane;
    cc.stream = h->stream;
    if (launch_chain(cc)) st = set_err(h, SEM2D_E_CUDA, bulk_last_error());
  }
  const int s_now = h->steps;
  if (!st) {
    // the gradients in global node order on the device, copied straight
    // into the caller's arrays
    if (!h->d_glob2lat) {
      if ((st = dupload(h, &h->d_glob2lat, h->glob2lat))) {
        release();
        return st;
      }
    }
    double *nodes = (double *)alloc_raw(8 * 3 * (size_t)h->npoin, false);
    if (!nodes) {
      release();
      return set_err(h, SEM2D_E_NOMEM, "no device memory for the adjoint");
    }
    gather_nodes_kernel<<<(h->npoin + 255) / 256, 256, 0, h->stream>>>(grads, h->plane, h->d_glob2lat, h->npoin,
                                                                       nodes);
    double *out[3] = {grad_rho, grad_vp, grad_vs};
    for (int q = 0; q < 3 && !st; ++q)
      if (out[q] && cudaMemcpyAsync(out[q], nodes + (size_t)q * h->npoin, 8 * (size_t)h->npoin,
                                    cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
        st = set_err(h, SEM2D_E_CUDA, "adjoint: copy back failed");
    if (!st && (cudaMemcpyAsync(h->d_step, &s_now, sizeof(int), cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
                cudaStreamSynchronize(h->stream) != cudaSuccess))
      st = set_err(h, SEM2D_E_CUDA, "adjoint: copy back failed");
  }
  release();
  if (st) return st;
  return check_device_error(h);
}

int sem2d_gpu_step_timed(sem2d_handle *h, int nsteps, double *ms) {
  if (!h || !ms) return SEM2D_E_ARG;
  if (h->owner) return set_err(h, SEM2D_E_STATE, "a batch member is stepped through its batch");
  if (h->batch_open) return set_err(h, SEM2D_E_STATE, "the batch is still open");
  if (nsteps < 0) return set_err(h, SEM2D_E_ARG, "negative step count");
  if (h->steps + nsteps > h->nt) return set_err(h, SEM2D_E_ARG, "stepping beyond nt");
  ms[0] = ms[1] = ms[2] = 0.0;
  constexpr int kBatch = 64;
  std::vector<cudaEvent_t> ev(4 * kBatch);
  for (auto &e : ev) CK(cudaEventCreate(&e));
  // the same max|v|, max|d| checks as sem2d_gpu_step (outside the events)
  const int ie = h->subs.empty() ? h->info_every : h->subs[0]->info_every;
  int st = SEM2D_OK;
  for (int done = 0; done < nsteps && !st;) {
    const int nb = std::min(kBatch, nsteps - done);
    for (int k = 0; k < nb && !st; ++k) {
      if (!h->subs.empty())
        st = h->mixed ? launch_batch_step<float>(h, &ev[4 * k]) : launch_batch_step<double>(h, &ev[4 * k]);
      else
        st = h->mixed ? launch_one_step<float>(h, h->cur, &ev[4 * k])
                      : launch_one_step<double>(h, h->cur, &ev[4 * k]);
      h->cur = 1 - h->cur;
      h->steps++;
      if (!st && ie > 0 && h->steps % ie == 0) {
        sync_members(h);
        st = launch_watch(h);
      }
    }
    sync_members(h);
    if (st) break;
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
      st = set_err(h, SEM2D_E_CUDA, cudaGetErrorString(e));
      break;
    }
    for (int k = 0; k < nb; ++k)
      for (int q = 0; q < 3; ++q) {
        float t = 0.f;
        cudaEventElapsedTime(&t, ev[4 * k + q], ev[4 * k + q + 1]);
        ms[q] += t;
      }
    done += nb;
  }
  for (auto &e : ev) cudaEventDestroy(e);
  if (st) return st;
  return check_device_error(h);
}

void *sem2d_gpu_stream(sem2d_handle *h) { return h ? (void *)h->stream : nullptr; }

int sem2d_gpu_sync(sem2d_handle *h) {
  if (!h) return SEM2D_E_ARG;
  return check_device_error(h);
}

int sem2d_gpu_current_step(sem2d_handle *h) { return h ? h->steps : SEM2D_E_ARG; }

int sem2d_gpu_reset(sem2d_handle *h) {
  if (!h) return SEM2D_E_ARG;
  if (h->owner) return set_err(h, SEM2D_E_STATE, "a batch member is reset through its batch");
  int st = reset_state(h);
  if (st) return st;
  return check_device_error(h);
}

int sem2d_gpu_get_fields(sem2d_handle *h, double *displ, double *veloc, double *accel) {
  if (!h) return SEM2D_E_ARG;
  if (!h->subs.empty()) return set_err(h, SEM2D_E_STATE, "outputs are read from the batch members");
  int st = check_device_error(h);
  if (st) return st;
  if (accel && !h->keep_accel) return set_err(h, SEM2D_E_STATE, "accelerations are not kept (leapfrog without field 'A')");
  const size_t n = (size_t)h->plane * h->ndof;
  // after n >= 1 steps: displacement d^n is the buffer not current; v and a are current
  void *src[3] = {h->steps > 0 ? h->D[1 - h->cur] : h->D[h->cur], h->V[h->cur], h->A[h->cur]};
  double *dst[3] = {displ, veloc, accel};
  std::vector<double> tmp(n);
  std::vector<float> tmpf(h->mixed ? n : 0);
  for (int k = 0; k < 3; ++k) {
    if (!dst[k]) continue;
    if (h->mixed) {
      CK(cudaMemcpy(tmpf.data(), src[k], n * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t q = 0; q < n; ++q) tmp[q] = tmpf[q];
    } else {
      CK(cudaMemcpy(tmp.data(), src[k], n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    for (int c = 0; c < h->ndof; ++c)
      for (int p = 0; p < h->npoin; ++p) dst[k][p + (size_t)h->npoin * c] = tmp[c * h->plane + h->glob2lat[p]];
  }
  if (displ && h->steps > 0 && h->scheme != 0 && h->beta != 0.0) {
    // the buffer holds the step's predictor: add the corrector beta dt^2 a^n
    // (solver.f90:82)
    const double cb = h->beta * h->dt * h->dt;
    if (h->mixed) {
      CK(cudaMemcpy(tmpf.data(), h->A[h->cur], n * sizeof(float), cudaMemcpyDeviceToHost));
      for (size_t q = 0; q < n; ++q) tmp[q] = tmpf[q];
    } else {
      CK(cudaMemcpy(tmp.data(), h->A[h->cur], n * sizeof(double), cudaMemcpyDeviceToHost));
    }
    for (int c = 0; c < h->ndof; ++c)
      for (int p = 0; p < h->npoin; ++p) {
        double &x = displ[p + (size_t)h->npoin * c];
        x = x + cb * tmp[c * h->plane + h->glob2lat[p]];
      }
  }
  return SEM2D_OK;
}


int sem2d_gpu_get_strain_stress(sem2d_handle *h, double *strain, double *stress) {
  if (!h) return SEM2D_E_ARG;
  if (!h->subs.empty()) return set_err(h, SEM2D_E_STATE, "outputs are read from the batch members");
  if (h->elem_ex.empty()) return set_err(h, SEM2D_E_STATE, "element numbering not kept (batch member)");
  if (h->general) return set_err(h, SEM2D_E_UNSUPPORTED, "strain and stress on a grid that is not flat");
  int st = check_device_error(h);
  if (st) return st;
  const int N = h->N, NN = N * N, nc = h->ndof + 1;
  const long long npt = (long long)h->nx * h->nz * NN;
  double *dev = nullptr, *dH = nullptr;
  CK(cudaMalloc(&dev, sizeof(double) * (size_t)npt * nc * 2));
  if (cudaMalloc(&dH, sizeof(double) * NN) != cudaSuccess) {
    cudaFree(dev);
    return set_err(h, SEM2D_E_NOMEM, "cudaMalloc");
  }
  cudaMemcpy(dH, h->H.data(), sizeof(double) * NN, cudaMemcpyHostToDevice);
  const void *D = h->steps > 0 ? h->D[1 - h->cur] : h->D[h->cur];
  void *Dc = nullptr;
  if (h->steps > 0 && h->scheme != 0 && h->beta != 0.0) {
    // displacement d^n = the step's predictor + beta dt^2 a^n (solver.f90:82)
    const long long n = (long long)h->plane * h->ndof;
    const double cb = h->beta * h->dt * h->dt;
    if (cudaMalloc(&Dc, (h->mixed ? sizeof(float) : sizeof(double)) * (size_t)n) != cudaSuccess) {
      cudaFree(dev);
      cudaFree(dH);
      return set_err(h, SEM2D_E_NOMEM, "cudaMalloc");
    }
    const int b = int(std::min<long long>((n + 255) / 256, 4096));
    if (h->mixed)
      sem2d_detail::corrector_kernel<float><<<b, 256, 0, h->stream>>>((float *)Dc, (const float *)D,
                                                                     (const float *)h->A[h->cur], float(cb), n);
    else
      sem2d_detail::corrector_kernel<double><<<b, 256, 0, h->stream>>>((double *)Dc, (const double *)D,
                                                                      (const double *)h->A[h->cur], cb, n);
    D = Dc;
  }
  const int blocks = int(std::min<long long>((npt + 255) / 256, 4096));
  if (h->mixed)
    sem2d_detail::strain_stress_kernel<float><<<blocks, 256, 0, h->stream>>>(
        (const float *)D, h->ndof, N, h->nx, h->nz, h->pitch, h->plane, h->d_row0, (const float *)h->geo[0],
        (const float *)h->geo[1], dH, h->mat_elem, h->mat_iso, (const float *)h->mat[0], (const float *)h->mat[1],
        (const float *)h->mat[2], (const float *)h->mat[3], (const float *)h->V[h->cur],
        h->has_kv ? (const float *)h->kveta : nullptr, dev, dev + npt * nc);
  else
    sem2d_detail::strain_stress_kernel<double><<<blocks, 256, 0, h->stream>>>(
        (const double *)D, h->ndof, N, h->nx, h->nz, h->pitch, h->plane, h->d_row0, (const double *)h->geo[0],
        (const double *)h->geo[1], dH, h->mat_elem, h->mat_iso, (const double *)h->mat[0],
        (const double *)h->mat[1], (const double *)h->mat[2], (const double *)h->mat[3],
        (const double *)h->V[h->cur], h->has_kv ? (const double *)h->kveta : nullptr, dev, dev + npt * nc);
  std::vector<double> host((size_t)npt * nc * 2);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(host.data(), dev, sizeof(double) * host.size(), cudaMemcpyDeviceToHost, h->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  cudaFree(dev);
  cudaFree(dH);
  if (Dc) cudaFree(Dc);
  if (e != cudaSuccess) return set_err(h, SEM2D_E_CUDA, std::string("strain/stress: ") + cudaGetErrorString(e));
  // lattice element (ex, ez) -> the reference's element e
  for (int el = 0; el < h->nelem; ++el) {
    const long long L = (long long)h->elem_ez[el] * h->nx + h->elem_ex[el];
    for (int pt = 0; pt < NN; ++pt)
      for (int c = 0; c < nc; ++c) {
        const size_t src = ((size_t)L * NN + pt) * nc + c, dst = pt + (size_t)NN * (c + (size_t)nc * el);
        if (strain) strain[dst] = host[src];
        if (stress) stress[dst] = host[(size_t)npt * nc + src];
      }
  }
  return SEM2D_OK;
}

int sem2d_gpu_get_seismograms(sem2d_handle *h, double *sis) {
  if (!h || !sis) return SEM2D_E_ARG;
  if (!h->subs.empty()) return set_err(h, SEM2D_E_STATE, "outputs are read from the batch members");
  int st = check_device_error(h);
  if (st) return st;
  if (h->nrec)
    CK(cudaMemcpy(sis, h->sis, sizeof(double) * (size_t)h->rec_nsamp * h->nrec * h->ndof, cudaMemcpyDeviceToHost));
  return SEM2D_OK;
}

int sem2d_gpu_get_fault(sem2d_handle *h, double *out) {
  if (!h || !out) return SEM2D_E_ARG;
  if (!h->subs.empty()) return set_err(h, SEM2D_E_STATE, "outputs are read from the batch members");
  int st = check_device_error(h);
  if (st) return st;
  if (h->nflt && h->fnsamp > 0)
    CK(cudaMemcpy(out, h->fd[F_SERIES], sizeof(double) * (size_t)h->onx * 6 * h->fnsamp, cudaMemcpyDeviceToHost));
  return SEM2D_OK;
}

int sem2d_gpu_get_fault_potency(sem2d_handle *h, double *out) {
  if (!h || !out) return SEM2D_E_ARG;
  if (!h->subs.empty()) return set_err(h, SEM2D_E_STATE, "outputs are read from the batch members");
  if (!h->nflt || !h->potency) return set_err(h, SEM2D_E_STATE, "the handle does not record the fault potency");
  int st = check_device_error(h);
  if (st) return st;
  CK(cudaMemcpy(out, h->fd[F_POTSERIES], sizeof(double) * 6 * ((size_t)h->nt + 1), cudaMemcpyDeviceToHost));
  return SEM2D_OK;
}

int sem2d_gpu_get_fault_state(sem2d_handle *h, double *D, double *V, double *T, double *MU, double *theta) {
  if (!h) return SEM2D_E_ARG;
  if (!h->subs.empty()) return set_err(h, SEM2D_E_STATE, "outputs are read from the batch members");
  int st = check_device_error(h);
  if (st) return st;
  if (!h->nflt) return SEM2D_OK;
  const size_t nfd = (size_t)h->nflt * h->ndof;
  if (D) CK(cudaMemcpy(D, h->fd[F_D], nfd * sizeof(double), cudaMemcpyDeviceToHost));
  if (V) CK(cudaMemcpy(V, h->fd[F_V], nfd * sizeof(double), cudaMemcpyDeviceToHost));
  if (T) CK(cudaMemcpy(T, h->fd[F_T], 2 * h->nflt * sizeof(double), cudaMemcpyDeviceToHost));
  if (MU) CK(cudaMemcpy(MU, h->fd[F_MU], h->nflt * sizeof(double), cudaMemcpyDeviceToHost));
  if (theta) CK(cudaMemcpy(theta, h->fd[F_THETA], h->nflt * sizeof(double), cudaMemcpyDeviceToHost));
  return SEM2D_OK;
}

long long sem2d_gpu_kernel_launches(sem2d_handle *h) { return h ? h->launches : 0; }

int sem2d_gpu_tile_shape(sem2d_handle *h, int *tx, int *tz) {
  if (!h) return SEM2D_E_ARG;
  if (tx) *tx = h->march ? kMarchColsHost : h->TX;
  if (tz) *tz = h->march ? h->march_cz : h->TZ;
  return SEM2D_OK;
}

int sem2d_gpu_destroy(sem2d_handle *h) {
  if (!h) return SEM2D_E_ARG;
  if (h->owner && h->owner->subs.size()) {
    // members are destroyed with their batch
    bool member = false;
    for (sem2d_handle *m : h->owner->subs) member = member || m == h;
    if (member) return set_err(h, SEM2D_E_STATE, "a batch member is destroyed with its batch");
  }
  if (h->stream) cudaStreamSynchronize(h->stream);
  for (sem2d_handle *m : h->subs) {
    m->owner = nullptr;
    sem2d_gpu_destroy(m);
  }
  h->subs.clear();
  if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
  for (void *p : h->allocs) cudaFree(p);
  if (h->stream && h->owns_stream) cudaStreamDestroy(h->stream);
  if (h->fstream) cudaStreamDestroy(h->fstream);
  for (cudaEvent_t e : {h->ev_m[0], h->ev_m[1], h->ev_c[0], h->ev_c[1], h->ev_f})
    if (e) cudaEventDestroy(e);
  delete h;
  return SEM2D_OK;
}

const char *sem2d_gpu_last_error(sem2d_handle *h) { return h ? h->err.c_str() : g_create_err.c_str(); }

}  // extern "C"

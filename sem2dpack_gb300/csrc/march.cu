// march.cu -- instantiation and launch of the march kernels (FP32, NGLL = 5,
// isotropic, leapfrog; material per node or per element).
#include <algorithm>
#include <string>

#include "bulk_inst.cuh"
#include "bulk_launch.h"
#include "march_adjoint.cuh"
#include "march_kernel.cuh"

namespace sem2d {

extern thread_local std::string g_bulk_err;

namespace {

constexpr int kThreads = 32 * kMarchWarps;
static_assert(kMarchWarpsHost == kMarchWarps, "host and device CTA shapes");

// warps per CTA of a launch (1, 2 or 4)
int cta_warps(const BulkConfig &c) { return c.march_warps == 1 || c.march_warps == 2 ? c.march_warps : kMarchWarps; }

// the staged rows of a 4-warp CTA may exceed the default 48 KB of dynamic
// shared memory (P-SV force state: 51 KB); allowed once per kernel
template <int NDOF, int MAT, bool FST>
void allow_stage() {
  static const bool done = [] {
    const int b = kMarchWarps * march_stage_bytes(NDOF, FST);
    cudaFuncSetAttribute(march_step_kernel<NDOF, MAT, FST>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    cudaFuncSetAttribute(march_fault_side_kernel<NDOF, MAT, FST>, cudaFuncAttributeMaxDynamicSharedMemorySize, b);
    return true;
  }();
  (void)done;
}

template <int NDOF, int MAT, bool FST>
int launch_one(const BulkConfig &c, const MarchLaunch &m) {
  allow_stage<NDOF, MAT, FST>();
  BulkParams<float, 5> p;
  fill_params<float, 5>(c, p);
  const int wpc = cta_warps(c);
  const int grid = std::max(1, (m.nunits + wpc - 1) / wpc);  // an empty set still counts the step
  march_step_kernel<NDOF, MAT, FST><<<grid, 32 * wpc, wpc * march_stage_bytes(NDOF, FST), c.stream>>>(
      p, static_cast<const MarchUnit *>(m.units), m.nunits);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <int NDOF, int MAT, bool FST>
int launch_many(const BulkConfig &c, const MarchLaunch &m) {
  MarchBatch b{};
  for (int k = 0; k < 25; ++k) b.H[k] = float(c.H[k]);
  for (int k = 0; k < 5; ++k) b.w[k] = float(c.w[k]);
  b.sims = static_cast<const BulkParams<float, 5> *>(m.sims);
  b.units = static_cast<const MarchUnit *>(m.units);
  b.nunits = m.nunits;
  b.step = m.step;
  b.done = m.done;
  const int wpc = cta_warps(c);
  const int grid = std::max(1, (m.nunits + wpc - 1) / wpc);  // an empty set still counts the step
  march_batch_kernel<NDOF, MAT><<<grid, 32 * wpc, wpc * march_stage_bytes(NDOF, false), c.stream>>>(b);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <int NDOF, int MAT, bool FST>
int launch_side(const BulkConfig &c, const MarchLaunch &m, int nstrips, int nrows) {
  allow_stage<NDOF, MAT, FST>();
  BulkParams<float, 5> p;
  fill_params<float, 5>(c, p);
  march_fault_side_kernel<NDOF, MAT, FST><<<nstrips, kThreads, kMarchWarps * march_stage_bytes(NDOF, FST), c.stream>>>(
      p, static_cast<const MarchUnit *>(m.units), nstrips, nrows);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <int NDOF, int MAT, bool FST>
int occupancy_one(int wpc) {
  allow_stage<NDOF, MAT, FST>();
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_step_kernel<NDOF, MAT, FST>, 32 * wpc,
                                                    wpc * march_stage_bytes(NDOF, FST)) !=
      cudaSuccess)
    return 0;
  return nb * wpc;
}

// the instantiation for (ndof, material layout, state formulation) of c
template <template <int, int, bool> class F, typename... A>
int dispatch(const BulkConfig &c, A &&...a) {
  const bool s = c.march_fst != 0;
  if (c.ndof == 1) {
    if (c.mat_elem == kMatNode) return s ? F<1, kMatNode, true>::run(a...) : F<1, kMatNode, false>::run(a...);
    return s ? F<1, kMatElement, true>::run(a...) : F<1, kMatElement, false>::run(a...);
  }
  if (c.mat_elem == kMatNode) return s ? F<2, kMatNode, true>::run(a...) : F<2, kMatNode, false>::run(a...);
  return s ? F<2, kMatElement, true>::run(a...) : F<2, kMatElement, false>::run(a...);
}
template <int NDOF, int MAT, bool FST>
struct LaunchOne {
  static int run(const BulkConfig &c, const MarchLaunch &m) { return launch_one<NDOF, MAT, FST>(c, m); }
};
template <int NDOF, int MAT, bool FST>
struct LaunchMany {
  static int run(const BulkConfig &c, const MarchLaunch &m) { return launch_many<NDOF, MAT, FST>(c, m); }
};
template <int NDOF, int MAT, bool FST>
struct LaunchSide {
  static int run(const BulkConfig &c, const MarchLaunch &m, int nstrips, int nrows) {
    return launch_side<NDOF, MAT, FST>(c, m, nstrips, nrows);
  }
};
template <int NDOF, int MAT, bool FST>
struct Occupancy {
  static int run(int wpc) { return occupancy_one<NDOF, MAT, FST>(wpc); }
};

}  // namespace

bool march_supported(const BulkConfig &c) {
  return c.N == 5 && c.mixed && c.fast && c.mat_iso && (c.mat_elem == kMatNode || c.mat_elem == kMatElement) &&
         (c.ndof == 1 || c.ndof == 2) && c.pitch % 4 == 0 && c.plane % 4 == 0;
}

int launch_march(const BulkConfig &c, const MarchLaunch &m) { return dispatch<LaunchOne>(c, c, m); }

int launch_march_batch(const BulkConfig &c, const MarchLaunch &m) {
  BulkConfig b = c;
  b.march_fst = 0;  // batches hold no fault: the displacement state
  return dispatch<LaunchMany>(b, b, m);
}

int launch_march_fault_side(const BulkConfig &c, const MarchLaunch &m, int nstrips, int nrows) {
  return dispatch<LaunchSide>(c, c, m, nstrips, nrows);
}

int launch_march_fault(const BulkConfig &c) {
  const FaultParams<float> &f = *static_cast<const FaultParams<float> *>(c.flt);
  // one warp per block: the node pairs spread over the SMs (the FP64 pipe
  // of an SM is shared by its warps)
  march_fault_kernel<<<(f.nflt + 31) / 32, 32, 0, c.stream>>>(f, static_cast<const float *>(c.fault_force));
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

namespace {
// the receivers' misfit derivatives of sample smp (march_adjoint_inject)
int adjoint_inject(const BulkConfig &bc, const MarchAdjConfig &c, void *lam, void *wv, int smp, int disp) {
  const int n = c.nrec * bc.ndof;
  march_adjoint_inject<<<(n + 127) / 128, 128, 0, bc.stream>>>(
      static_cast<float *>(lam), static_cast<float *>(wv), bc.plane, bc.pitch, bc.LX, bc.LZ,
      static_cast<const float *>(bc.rmass), static_cast<const float *>(bc.per_rm), bc.ndof, c.nrec, c.nsamp, smp,
      disp, c.rec_I, c.rec_J, c.resid, float(bc.dt));
  return 1;
}
bool sampled(const MarchAdjConfig &c, int it) {
  const int is = c.isamp > 0 ? c.isamp : 1;
  return c.nrec > 0 && it > 0 && it % is == 0 && it / is < c.nsamp;
}
}  // namespace

int launch_march_adjoint(const BulkConfig &bc, const MarchAdjConfig &c, int *launches) {
  BulkParams<float, 5> p;
  fill_params<float, 5>(bc, p);
  MarchAdj x{};
  x.a = static_cast<const float *>(c.a);
  x.vprev = static_cast<const float *>(c.vprev);
  x.g_M = static_cast<float *>(c.g_M);
  x.g_C = static_cast<float *>(c.g_C);
  MarchAdjParams m{};
  m.LX = bc.LX;
  m.LZ = bc.LZ;
  m.pitch = bc.pitch;
  m.plane = bc.plane;
  m.nx = bc.nx;
  m.nz = bc.nz;
  m.row0 = bc.row0;
  for (int k = 0; k < 25; ++k) m.H[k] = float(bc.H[k]);
  for (int k = 0; k < 5; ++k) m.w[k] = float(bc.w[k]);
  m.xix = static_cast<const float *>(bc.geo[0]);
  m.etaz = static_cast<const float *>(bc.geo[1]);
  m.dxdxi = static_cast<const float *>(bc.geo[2]);
  m.dzdeta = static_cast<const float *>(bc.geo[3]);
  m.lam = static_cast<const float *>(bc.Dcur);
  m.d = static_cast<const float *>(c.d);
  m.g_la = static_cast<float *>(c.g_la);
  m.g_mu = static_cast<float *>(c.g_mu);
  m.kd2 = bc.kd2;
  const MarchUnit *u = static_cast<const MarchUnit *>(c.units);
  const int wpc = cta_warps(bc);
  const int grid = std::max(1, (c.nunits + wpc - 1) / wpc);
  const int mgrid = std::max(1, (c.nunits + kMarchWarps - 1) / kMarchWarps);
  // the misfit derivatives of the step, by an extra CTA of the moduli launch
  const int is = c.isamp > 0 ? c.isamp : 1;
  m.inj = -1;
  if (c.field == 'D' && sampled(c, c.it)) {
    m.inj = 1;
    m.smp = c.it / is;
  } else if (c.field != 'D' && sampled(c, c.it - 1)) {
    m.inj = 0;
    m.smp = (c.it - 1) / is;
  }
  m.ndof = bc.ndof;
  m.nrec = c.nrec;
  m.nsamp = c.nsamp;
  m.lam_next = static_cast<float *>(bc.Dnext);
  m.w_next = static_cast<float *>(bc.Vnext);
  m.rmass = static_cast<const float *>(bc.rmass);
  m.per_rm = static_cast<const float *>(bc.per_rm);
  m.rec_I = c.rec_I;
  m.rec_J = c.rec_J;
  m.resid = c.resid;
  m.dt = float(bc.dt);
  const int mg = mgrid + (m.inj >= 0 ? 1 : 0);
  // the P-SV step stages six planes per node row: 7.5 KB per warp
  const int sb1 = wpc * march_stage_bytes(1, false, true), sb2 = wpc * march_stage_bytes(2, false, true);
  static const bool smem_set = [] {
    cudaFuncSetAttribute(march_adjoint_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kMarchWarps * march_stage_bytes(1, false, true));
    cudaFuncSetAttribute(march_adjoint_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         kMarchWarps * march_stage_bytes(2, false, true));
    return true;
  }();
  (void)smem_set;
  if (bc.ndof == 1) {
    march_adjoint_kernel<1><<<grid, 32 * wpc, sb1, bc.stream>>>(p, x, c.it, u, c.nunits);
    adj_march_moduli<1><<<mg, kThreads, kMarchWarps * adj_moduli_stage_f4(1) * 16, bc.stream>>>(m, u, c.nunits);
  } else {
    march_adjoint_kernel<2><<<grid, 32 * wpc, sb2, bc.stream>>>(p, x, c.it, u, c.nunits);
    adj_march_moduli<2><<<mg, kThreads, kMarchWarps * adj_moduli_stage_f4(2) * 16, bc.stream>>>(m, u, c.nunits);
  }
  *launches = 2;
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

int launch_march_adjoint_seed(const BulkConfig &bc, const MarchAdjConfig &c, int *launches) {
  *launches = 0;
  if (c.field == 'D' || !sampled(c, c.it)) return 0;
  *launches = adjoint_inject(bc, c, bc.Dcur, bc.Vcur, c.it / (c.isamp > 0 ? c.isamp : 1), 0);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

int march_warps_per_sm(const BulkConfig &c) { return dispatch<Occupancy>(c, cta_warps(c)); }

}  // namespace sem2d

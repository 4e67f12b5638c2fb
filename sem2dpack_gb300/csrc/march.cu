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

template <int NDOF, int MAT, bool FST>
int launch_one(const BulkConfig &c, const MarchLaunch &m) {
  BulkParams<float, 5> p;
  fill_params<float, 5>(c, p);
  const int wpc = cta_warps(c);
  const int grid = std::max(1, (m.nunits + wpc - 1) / wpc);  // an empty set still counts the step
  march_step_kernel<NDOF, MAT, FST><<<grid, 32 * wpc, 0, c.stream>>>(p, static_cast<const MarchUnit *>(m.units),
                                                                      m.nunits);
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
  march_batch_kernel<NDOF, MAT><<<grid, 32 * wpc, 0, c.stream>>>(b);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <int NDOF, int MAT, bool FST>
int launch_side(const BulkConfig &c, const MarchLaunch &m, int nstrips, int nrows) {
  BulkParams<float, 5> p;
  fill_params<float, 5>(c, p);
  march_fault_side_kernel<NDOF, MAT, FST><<<nstrips, kThreads, 0, c.stream>>>(
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
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_step_kernel<NDOF, MAT, FST>, 32 * wpc, 0) !=
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

int launch_march_adjoint(const MarchAdjConfig &c) {
  MarchAdjParams p{};
  p.LX = c.LX;
  p.LZ = c.LZ;
  p.pitch = c.pitch;
  p.plane = c.plane;
  p.nx = c.nx;
  p.nz = c.nz;
  p.row0 = c.row0;
  for (int k = 0; k < 25; ++k) p.H[k] = float(c.H[k]);
  for (int k = 0; k < 5; ++k) p.w[k] = float(c.w[k]);
  p.xix = static_cast<const float *>(c.geo[0]);
  p.etaz = static_cast<const float *>(c.geo[1]);
  p.dxdxi = static_cast<const float *>(c.geo[2]);
  p.dzdeta = static_cast<const float *>(c.geo[3]);
  p.mat[0] = static_cast<const float *>(c.mat[0]);
  p.mat[1] = static_cast<const float *>(c.mat[1]);
  p.rmass = static_cast<const float *>(c.rmass);
  p.per_rm = static_cast<const float *>(c.per_rm);
  p.per_Ca = static_cast<const float *>(c.per_Ca);
  p.per_Cb = static_cast<const float *>(c.per_Cb);
  p.Db = static_cast<const float *>(c.Db);
  p.Vb = static_cast<const float *>(c.Vb);
  p.Dbn = static_cast<float *>(c.Dbn);
  p.Vbn = static_cast<float *>(c.Vbn);
  p.d = static_cast<const float *>(c.d);
  p.vprev = static_cast<const float *>(c.vprev);
  p.a = static_cast<const float *>(c.a);
  p.g_la = static_cast<float *>(c.g_la);
  p.g_mu = static_cast<float *>(c.g_mu);
  p.g_M = static_cast<float *>(c.g_M);
  p.g_C = static_cast<float *>(c.g_C);
  p.nrec = c.nrec;
  p.nsamp = c.nsamp;
  p.isamp = c.isamp > 0 ? c.isamp : 1;
  p.field = c.field;
  p.rec_I = c.rec_I;
  p.rec_row = c.rec_row;
  p.rec_ids_row = c.rec_ids_row;
  p.resid = c.resid;
  p.dt = float(c.dt);
  p.kd2 = c.kd2;
  p.it = c.it;
  const MarchUnit *u = static_cast<const MarchUnit *>(c.units);
  const int grid = std::max(1, (c.nunits + kMarchWarps - 1) / kMarchWarps);
  if (c.ndof == 1) {
    adj_march_forces<1><<<grid, kThreads, 0, c.stream>>>(p, u, c.nunits);
    adj_march_moduli<1><<<grid, kThreads, 0, c.stream>>>(p, u, c.nunits);
  } else {
    adj_march_forces<2><<<grid, kThreads, 0, c.stream>>>(p, u, c.nunits);
    adj_march_moduli<2><<<grid, kThreads, 0, c.stream>>>(p, u, c.nunits);
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

int march_warps_per_sm(const BulkConfig &c) { return dispatch<Occupancy>(c, cta_warps(c)); }

}  // namespace sem2d

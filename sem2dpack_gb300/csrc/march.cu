// march.cu -- instantiation and launch of the march kernels (FP32, NGLL = 5,
// isotropic, leapfrog; material per node or per element).
#include <algorithm>
#include <string>

#include "bulk_inst.cuh"
#include "bulk_launch.h"
#include "march_kernel.cuh"

namespace sem2d {

extern thread_local std::string g_bulk_err;

namespace {

constexpr int kThreads = 32 * kMarchWarps;

template <int NDOF, int MAT>
int launch_one(const BulkConfig &c, const MarchLaunch &m) {
  BulkParams<float, 5> p;
  fill_params<float, 5>(c, p);
  const int grid = std::max(1, (m.nunits + kMarchWarps - 1) / kMarchWarps);  // an empty set still counts the step
  march_step_kernel<NDOF, MAT><<<grid, kThreads, 0, c.stream>>>(p, static_cast<const MarchUnit *>(m.units),
                                                                m.nunits);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <int NDOF, int MAT>
int launch_many(const BulkConfig &c, const MarchLaunch &m) {
  MarchBatch b{};
  for (int k = 0; k < 25; ++k) b.H[k] = float(c.H[k]);
  for (int k = 0; k < 5; ++k) b.w[k] = float(c.w[k]);
  b.sims = static_cast<const BulkParams<float, 5> *>(m.sims);
  b.units = static_cast<const MarchUnit *>(m.units);
  b.nunits = m.nunits;
  b.step = m.step;
  b.done = m.done;
  const int grid = std::max(1, (m.nunits + kMarchWarps - 1) / kMarchWarps);  // an empty set still counts the step
  march_batch_kernel<NDOF, MAT><<<grid, kThreads, 0, c.stream>>>(b);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <int NDOF, int MAT>
int occupancy_one() {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, march_step_kernel<NDOF, MAT>, kThreads, 0) != cudaSuccess)
    return 0;
  return nb * kMarchWarps;
}

}  // namespace

bool march_supported(const BulkConfig &c) {
  return c.N == 5 && c.mixed && c.fast && c.mat_iso && (c.mat_elem == kMatNode || c.mat_elem == kMatElement) &&
         (c.ndof == 1 || c.ndof == 2) && c.pitch % 4 == 0 && c.plane % 4 == 0;
}

int launch_march(const BulkConfig &c, const MarchLaunch &m) {
  if (c.ndof == 1)
    return c.mat_elem == kMatNode ? launch_one<1, kMatNode>(c, m) : launch_one<1, kMatElement>(c, m);
  return c.mat_elem == kMatNode ? launch_one<2, kMatNode>(c, m) : launch_one<2, kMatElement>(c, m);
}

int launch_march_batch(const BulkConfig &c, const MarchLaunch &m) {
  if (c.ndof == 1)
    return c.mat_elem == kMatNode ? launch_many<1, kMatNode>(c, m) : launch_many<1, kMatElement>(c, m);
  return c.mat_elem == kMatNode ? launch_many<2, kMatNode>(c, m) : launch_many<2, kMatElement>(c, m);
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

int march_warps_per_sm(const BulkConfig &c) {
  if (c.ndof == 1) return c.mat_elem == kMatNode ? occupancy_one<1, kMatNode>() : occupancy_one<1, kMatElement>();
  return c.mat_elem == kMatNode ? occupancy_one<2, kMatNode>() : occupancy_one<2, kMatElement>();
}

}  // namespace sem2d

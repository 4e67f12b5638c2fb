// bulk_inst.cuh -- instantiation of the bulk kernel for one NGLL.
#pragma once

#include <string>

#include "bulk_kernel.cuh"
#include "bulk_launch.h"

namespace sem2d {

extern thread_local std::string g_bulk_err;

template <typename real, int N, int NDOF, bool MELEM>
int configure_typed(const BulkConfig &c) {
  const size_t smem = bulk_smem_bytes<real, N, NDOF>(c.tile_nodes, c.own_nodes, c.nmat, c.has_kv, c.mat_elem);
  cudaError_t e = cudaFuncSetAttribute(bulk_step_kernel<real, N, NDOF, MELEM>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (e != cudaSuccess) {
    g_bulk_err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <typename real, int N, int NDOF, bool MELEM>
int launch_typed(const BulkConfig &c) {
  BulkParams<real, N> p{};
  p.LX = c.LX;
  p.LZ = c.LZ;
  p.pitch = c.pitch;
  p.plane = c.plane;
  p.nx = c.nx;
  p.nz = c.nz;
  p.row0 = c.row0;
  p.TX = c.TX;
  p.ztile = c.ztile;
  for (int k = 0; k < N * N; ++k) p.H[k] = real(c.H[k]);
  for (int k = 0; k < N; ++k) p.w[k] = real(c.w[k]);
  p.Dcur = static_cast<const real *>(c.Dcur);
  p.Dnext = static_cast<real *>(c.Dnext);
  p.Vcur = static_cast<const real *>(c.Vcur);
  p.Vnext = static_cast<real *>(c.Vnext);
  p.Acur = static_cast<const real *>(c.Acur);
  p.Anext = static_cast<real *>(c.Anext);
  p.mat_iso = c.mat_iso;
  for (int m = 0; m < 4; ++m) p.mat[m] = static_cast<const real *>(c.mat[m]);
  p.mat_elem = c.mat_elem;
  p.kveta = static_cast<const real *>(c.kveta);
  p.rmass = static_cast<const real *>(c.rmass);
  p.xix = static_cast<const real *>(c.geo[0]);
  p.etaz = static_cast<const real *>(c.geo[1]);
  p.dxdxi = static_cast<const real *>(c.geo[2]);
  p.dzdeta = static_cast<const real *>(c.geo[3]);
  p.per_rm = static_cast<const real *>(c.per_rm);
  p.per_Ca = static_cast<const real *>(c.per_Ca);
  p.per_Cb = static_cast<const real *>(c.per_Cb);
  p.jf1 = c.jf1;
  p.jf2 = c.jf2;
  p.has_fault = c.has_fault;
  if (c.has_fault) p.flt = *static_cast<const FaultParams<real> *>(c.flt);
  p.nsrc = c.nsrc;
  p.src_I = c.src_I;
  p.src_J = c.src_J;
  p.src_amp = c.src_amp;
  p.nt = c.nt;
  p.step = c.step;
  p.done = c.done;
  p.rec_nsamp = c.rec_nsamp;
  p.rec_isamp = c.rec_isamp;
  p.rec_nrec = c.rec_nrec;
  p.rec_npts = c.rec_npts;
  p.rec_field = c.rec_field;
  p.rec_tile_start = c.rec_tile_start;
  p.rec_ids = c.rec_ids;
  p.rec_I = c.rec_I;
  p.rec_J = c.rec_J;
  p.rec_w = c.rec_w;
  p.sis = c.sis;
  p.scheme = c.scheme;
  p.dt = real(c.dt);
  p.cv = real(c.cv);
  p.cpred = real(c.cpred);
  p.cd2 = real(c.cd2);
  p.kd2 = c.kd2;
  const size_t smem = bulk_smem_bytes<real, N, NDOF>(c.tile_nodes, c.own_nodes, c.nmat, c.has_kv, c.mat_elem);
  bulk_step_kernel<real, N, NDOF, MELEM><<<dim3(c.grid_x, c.grid_y), kBulkThreads, smem, c.stream>>>(
      p, c.tile_nodes, c.own_nodes, c.nmat, c.has_kv);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <typename real, int N, int NDOF, bool MELEM>
int occupancy_typed(const BulkConfig &c) {
  const size_t smem = bulk_smem_bytes<real, N, NDOF>(c.tile_nodes, c.own_nodes, c.nmat, c.has_kv, c.mat_elem);
  if (configure_typed<real, N, NDOF, MELEM>(c)) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, bulk_step_kernel<real, N, NDOF, MELEM>, kBulkThreads,
                                                    smem) != cudaSuccess)
    return 0;
  return nb;
}

template <typename real, int N, int NDOF>
int occupancy_m(const BulkConfig &c) {
  return c.mat_elem ? occupancy_typed<real, N, NDOF, true>(c) : occupancy_typed<real, N, NDOF, false>(c);
}

template <int N>
int occupancy_for_n(const BulkConfig &c) {
  if (c.ndof == 1) return c.mixed ? occupancy_m<float, N, 1>(c) : occupancy_m<double, N, 1>(c);
  return c.mixed ? occupancy_m<float, N, 2>(c) : occupancy_m<double, N, 2>(c);
}

template <typename real, int N, int NDOF>
int configure_m(const BulkConfig &c) {
  return c.mat_elem ? configure_typed<real, N, NDOF, true>(c) : configure_typed<real, N, NDOF, false>(c);
}
template <typename real, int N, int NDOF>
int launch_m(const BulkConfig &c) {
  return c.mat_elem ? launch_typed<real, N, NDOF, true>(c) : launch_typed<real, N, NDOF, false>(c);
}

template <int N>
int configure_for_n(const BulkConfig &c) {
  if (c.ndof == 1) return c.mixed ? configure_m<float, N, 1>(c) : configure_m<double, N, 1>(c);
  return c.mixed ? configure_m<float, N, 2>(c) : configure_m<double, N, 2>(c);
}

template <int N>
int launch_for_n(const BulkConfig &c) {
  if (c.ndof == 1) return c.mixed ? launch_m<float, N, 1>(c) : launch_m<double, N, 1>(c);
  return c.mixed ? launch_m<float, N, 2>(c) : launch_m<double, N, 2>(c);
}

template <int N>
size_t smem_for_n(int ndof, int mixed, int tn, int on, int nmat, int kv, int me) {
  if (ndof == 1)
    return mixed ? bulk_smem_bytes<float, N, 1>(tn, on, nmat, kv, me) : bulk_smem_bytes<double, N, 1>(tn, on, nmat, kv, me);
  return mixed ? bulk_smem_bytes<float, N, 2>(tn, on, nmat, kv, me) : bulk_smem_bytes<double, N, 2>(tn, on, nmat, kv, me);
}

}  // namespace sem2d

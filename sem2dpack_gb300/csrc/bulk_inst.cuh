// bulk_inst.cuh -- instantiation of the step kernels for one NGLL.
#pragma once

#include <string>

#include "bulk_launch.h"
#include "strip_kernel.cuh"

namespace sem2d {

extern thread_local std::string g_bulk_err;

// the typed parameter block of a problem from its type-erased description
template <typename real, int N>
void fill_params(const BulkConfig &c, BulkParams<real, N> &p) {
  p = BulkParams<real, N>{};
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
  p.Fcur = static_cast<const real *>(c.Fcur);
  p.Fnext = static_cast<real *>(c.Fnext);
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
  p.per_kd = static_cast<const real *>(c.per_kd);
  p.per_dir = c.per_dir;
  p.perio_f = static_cast<real *>(c.perio_f);
  p.gen = static_cast<const real *>(c.gen);
  p.gen_stride = c.gen_stride;
  p.perio_tb = c.perio_tb;
  p.per_bf = static_cast<const real *>(c.per_bf);
  p.jf1 = c.jf1;
  p.jf2 = c.jf2;
  p.has_fault = c.has_fault;
  if (c.has_fault) p.flt = *static_cast<const FaultParams<real> *>(c.flt);
  p.fault_force = static_cast<real *>(c.fault_force);
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
  p.width = real(c.width);
  p.cv = real(c.cv);
  p.cpred = real(c.cpred);
  p.cd2 = real(c.cd2);
  p.cb = real(c.cb);
  p.cal = real(c.cal);
  p.cpa = real(c.cpa);
  p.kd2 = c.kd2;
  p.nmat = c.nmat;
  p.has_kv = c.has_kv;
  p.nplanes = c.nplanes;
  p.error = c.error;
  p.spin_limit = c.spin_limit;
  p.chunk_shift = c.chunk_shift;
}

template <typename real, int N, int NDOF, int MAT, bool FAST>
int configure_typed(const BulkConfig &c) {
  const size_t smem = strip_smem_bytes<real, N, NDOF>(c.nplanes);
  cudaError_t e = cudaFuncSetAttribute(strip_step_kernel<real, N, NDOF, MAT, FAST>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if constexpr (MAT != kMatGeneral) {
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(strip_batch_kernel<real, N, NDOF, MAT, FAST>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  }
  if (e != cudaSuccess) {
    g_bulk_err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <typename real, int N, int NDOF, int MAT, bool FAST>
int launch_typed(const BulkConfig &c) {
  BulkParams<real, N> p;
  fill_params<real, N>(c, p);
  const size_t smem = strip_smem_bytes<real, N, NDOF>(c.nplanes);
  strip_step_kernel<real, N, NDOF, MAT, FAST><<<dim3(c.grid_x, c.grid_y), kStripThreads, smem, c.stream>>>(p);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <typename real, int N, int NDOF, int MAT, bool FAST>
int launch_batch_typed(const BulkConfig &c, const BatchLaunch &b) {
  BatchParams<real, N> bp{};
  for (int k = 0; k < N * N; ++k) bp.H[k] = real(c.H[k]);
  for (int k = 0; k < N; ++k) bp.w[k] = real(c.w[k]);
  bp.sims = static_cast<const BulkParams<real, N> *>(b.params);
  bp.units = static_cast<const int4 *>(b.units);
  bp.nunits = b.nunits;
  bp.step = b.step;
  bp.done = b.done;
  const size_t smem = strip_smem_bytes<real, N, NDOF>(c.nplanes);
  strip_batch_kernel<real, N, NDOF, MAT, FAST><<<b.grid, kStripThreads, smem, c.stream>>>(bp);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

template <typename real, int N, int NDOF, int MAT, bool FAST>
int occupancy_typed(const BulkConfig &c) {
  const size_t smem = strip_smem_bytes<real, N, NDOF>(c.nplanes);
  if (configure_typed<real, N, NDOF, MAT, FAST>(c)) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, strip_step_kernel<real, N, NDOF, MAT, FAST>,
                                                    kStripThreads, smem) != cudaSuccess)
    return 0;
  return nb;
}

// dispatch over the material layout and the fast path (NGLL = 5 only)
template <typename real, int N, int NDOF, typename F>
int dispatch_m(const BulkConfig &c, F &&f) {
  const bool fast = N == 5 && c.fast;
  if (c.mat_elem == kMatGeneral) return f.template operator()<real, N, NDOF, kMatGeneral, false>();
  if (c.mat_elem == kMatPoint)
    return fast ? f.template operator()<real, N, NDOF, kMatPoint, (N == 5)>()
                : f.template operator()<real, N, NDOF, kMatPoint, false>();
  if (c.mat_elem == kMatElement)
    return fast ? f.template operator()<real, N, NDOF, kMatElement, (N == 5)>()
                : f.template operator()<real, N, NDOF, kMatElement, false>();
  return fast ? f.template operator()<real, N, NDOF, kMatNode, (N == 5)>()
              : f.template operator()<real, N, NDOF, kMatNode, false>();
}

template <int N, typename F>
int dispatch_all(const BulkConfig &c, F &&f) {
  if (c.ndof == 1) return c.mixed ? dispatch_m<float, N, 1>(c, f) : dispatch_m<double, N, 1>(c, f);
  return c.mixed ? dispatch_m<float, N, 2>(c, f) : dispatch_m<double, N, 2>(c, f);
}

struct ConfigureOp {
  const BulkConfig &c;
  template <typename real, int N, int NDOF, int MAT, bool FAST>
  int operator()() const { return configure_typed<real, N, NDOF, MAT, FAST>(c); }
};
struct LaunchOp {
  const BulkConfig &c;
  template <typename real, int N, int NDOF, int MAT, bool FAST>
  int operator()() const { return launch_typed<real, N, NDOF, MAT, FAST>(c); }
};
struct OccupancyOp {
  const BulkConfig &c;
  template <typename real, int N, int NDOF, int MAT, bool FAST>
  int operator()() const { return occupancy_typed<real, N, NDOF, MAT, FAST>(c); }
};
struct BatchOp {
  const BulkConfig &c;
  const BatchLaunch &b;
  template <typename real, int N, int NDOF, int MAT, bool FAST>
  int operator()() const {
    if constexpr (MAT == kMatGeneral) {
      g_bulk_err = "batches of grids that are not flat are not supported";
      return 1;
    } else {
      return launch_batch_typed<real, N, NDOF, MAT, FAST>(c, b);
    }
  }
};

template <int N>
int configure_for_n(const BulkConfig &c) { return dispatch_all<N>(c, ConfigureOp{c}); }
template <int N>
int launch_for_n(const BulkConfig &c) { return dispatch_all<N>(c, LaunchOp{c}); }
template <int N>
int occupancy_for_n(const BulkConfig &c) { return dispatch_all<N>(c, OccupancyOp{c}); }
template <int N>
int launch_batch_for_n(const BulkConfig &c, const BatchLaunch &b) { return dispatch_all<N>(c, BatchOp{c, b}); }

template <int N>
size_t smem_for_n(int ndof, int mixed, int nplanes) {
  if (ndof == 1)
    return mixed ? strip_smem_bytes<float, N, 1>(nplanes) : strip_smem_bytes<double, N, 1>(nplanes);
  return mixed ? strip_smem_bytes<float, N, 2>(nplanes) : strip_smem_bytes<double, N, 2>(nplanes);
}

template <int N>
int strip_width_for_n() {
  return StripShape<float, N>::SW1 - 1;
}
template <int N>
int strip_batch_rows_for_n() {
  return StripShape<float, N>::R;
}

// the parameter block of one problem, written to `out` (params_bytes)
template <int N>
size_t params_bytes_for_n(int mixed) {
  return mixed ? sizeof(BulkParams<float, N>) : sizeof(BulkParams<double, N>);
}
template <int N>
void fill_params_for_n(const BulkConfig &c, void *out) {
  if (c.mixed) fill_params<float, N>(c, *static_cast<BulkParams<float, N> *>(out));
  else fill_params<double, N>(c, *static_cast<BulkParams<double, N> *>(out));
}

}  // namespace sem2d

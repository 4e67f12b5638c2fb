// noalloc.cu -- sem2d_gpu_step_noalloc: the bulk step kernel on caller-owned
// device arrays, with its scratch in a file-scope device array.
//
// The handle-based path allocates the partner buffers of its double-buffered
// update and two counters with cudaMalloc.  Here they live in g_scratch:
//   [0, 64)         step counter (int), CTA completion counter (unsigned),
//                   the error flag of calls without a status pointer (int)
//   [64, 16384)     tile-row boundaries, nz+1 ints
//   [16384, ...)    partner displacement plane(s), then partner velocity
// Host code never dereferences g_scratch: its device address is looked up
// once per device with cudaGetSymbolAddress and passed to the kernels.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <mutex>
#include <string>

#include "../../include/sem2d_gpu.h"
#include "bulk_launch.h"

namespace {

constexpr size_t kHeaderBytes = 64;
constexpr size_t kFieldOffset = 16384;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[SEM2D_NOALLOC_SCRATCH_BYTES];

std::mutex g_mutex;
void *g_scratch_addr[kMaxDevices] = {nullptr};

// step counter = step0, completion counter = 0, uniform tile rows of TZ;
// the error flag is left as it is (the caller's status is never cleared)
__global__ void noalloc_setup_kernel(unsigned char *scratch, int step0, int nz, int TZ) {
  int *step = reinterpret_cast<int *>(scratch);
  unsigned *done = reinterpret_cast<unsigned *>(scratch + 4);
  int *ztile = reinterpret_cast<int *>(scratch + kHeaderBytes);
  *step = step0;
  *done = 0u;
  int k = 0;
  for (int z = 0; z < nz; z += TZ) ztile[k++] = z;
  ztile[k] = nz;
}

// the message of a rejected call, returned by sem2d_gpu_last_error(NULL)
int fail(int code, const std::string &msg) {
  sem2d::set_library_error("sem2d_gpu_step_noalloc: " + msg);
  return code;
}

}  // namespace

extern "C" int sem2d_gpu_step_noalloc(const sem2d_lattice_args *a, int nsteps, void *stream) {
  using namespace sem2d;
  if (!a || nsteps < 0) return fail(SEM2D_E_ARG, "null arguments or negative step count");
  if (a->ngll != 3 && a->ngll != 5 && a->ngll != 6 && a->ngll != 9)
    return fail(SEM2D_E_UNSUPPORTED, "ngll must be 3, 5, 6 or 9");
  if (a->ndof != 1 && a->ndof != 2) return fail(SEM2D_E_ARG, "ndof must be 1 or 2");
  if (a->precision != SEM2D_PRECISION_FP64 && a->precision != SEM2D_PRECISION_MIXED)
    return fail(SEM2D_E_ARG, "unknown precision");
  if (a->nx <= 0 || a->nz <= 0 || a->LX != a->nx * (a->ngll - 1) + 1 || a->LZ < a->nz * (a->ngll - 1) + 1 ||
      a->pitch < a->LX)
    return fail(SEM2D_E_ARG, "inconsistent lattice sizes");
  if (!a->d || !a->v || !a->row0 || !a->hprime || !a->wgll || !a->rmass || !a->per_rm || !a->per_Ca ||
      !a->per_Cb || !a->mat[0] || !a->xix || !a->etaz || !a->dxdxi || !a->dzdeta)
    return fail(SEM2D_E_ARG, "missing array");
  {
    // rows are fetched with 16-byte bulk copies: 16-byte aligned planes and
    // a row pitch of a multiple of 16 bytes
    const size_t rs = a->precision == SEM2D_PRECISION_MIXED ? sizeof(float) : sizeof(double);
    const size_t al = 16 / rs;
    if (a->pitch % al != 0) return fail(SEM2D_E_ARG, "the row pitch must be a multiple of 16 bytes");
    const void *ptrs[] = {a->d, a->v, a->rmass, a->mat[0], a->mat[1], a->mat[2], a->mat[3]};
    for (const void *q : ptrs)
      if (reinterpret_cast<uintptr_t>(q) % 16 != 0) return fail(SEM2D_E_ARG, "arrays must be 16-byte aligned");
  }
  if (a->nsrc > 0 && (!a->src_I || !a->src_J || !a->src_amp)) return fail(SEM2D_E_ARG, "missing source arrays");
  if (a->step0 < 0 || a->step0 + nsteps > a->nt) return fail(SEM2D_E_ARG, "steps beyond nt");
  const size_t rs = a->precision == SEM2D_PRECISION_MIXED ? sizeof(float) : sizeof(double);
  const size_t plane = size_t(a->pitch) * a->LZ;
  const size_t field_bytes = (rs * a->ndof * plane + 255) / 256 * 256;
  if (kFieldOffset + 2 * field_bytes > SEM2D_NOALLOC_SCRATCH_BYTES)
    return fail(SEM2D_E_ARG, "problem too large for the no-allocation scratch (SEM2D_NOALLOC_SCRATCH_BYTES)");
  if (kHeaderBytes + 4 * size_t(a->nz + 1) > kFieldOffset)
    return fail(SEM2D_E_ARG, "too many element rows for the no-allocation scratch");
  if (nsteps == 0) return SEM2D_OK;

  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return fail(SEM2D_E_CUDA, "cudaGetDevice");
  unsigned char *scratch;
  {
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
      void *p = nullptr;
      const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess) return fail(SEM2D_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_addr[dev] = p;
    }
    scratch = static_cast<unsigned char *>(g_scratch_addr[dev]);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int N = a->ngll;
  const int TX = strip_width(N), TZ = std::min(16, a->nz);
  if (TX <= 0) return fail(SEM2D_E_UNSUPPORTED, "NGLL not compiled");
  BulkConfig c;
  c.N = N;
  c.ndof = a->ndof;
  c.mixed = a->precision == SEM2D_PRECISION_MIXED;
  c.nmat = a->ndof == 2 ? (a->mat_iso ? 2 : 4) : (a->mat_iso ? 1 : 2);
  for (int m = 0; m < c.nmat; ++m)
    if (!a->mat[m]) return fail(SEM2D_E_ARG, "missing material plane");
  c.has_kv = 0;
  c.mat_elem = 0;
  c.mat_iso = a->mat_iso;
  c.fast = a->mat_iso ? 1 : 0;
  c.nplanes = strip_plane_count(c.ndof, c.nmat, 0, 0);
  if (bulk_smem(N, c.ndof, c.mixed, c.nplanes) > 227 * 1024)
    return fail(SEM2D_E_UNSUPPORTED, "the stage buffers do not fit in shared memory");
  if (configure_bulk(c)) return fail(SEM2D_E_CUDA, std::string("configure: ") + bulk_last_error());
  c.grid_x = (a->nx + TX - 1) / TX;
  c.grid_y = (a->nz + TZ - 1) / TZ;
  c.LX = a->LX;
  c.LZ = a->LZ;
  c.pitch = a->pitch;
  c.plane = (long long)plane;
  c.nx = a->nx;
  c.nz = a->nz;
  c.row0 = a->row0;
  c.TX = TX;
  c.ztile = reinterpret_cast<const int *>(scratch + kHeaderBytes);
  c.H = a->hprime;
  c.w = a->wgll;
  for (int m = 0; m < 4; ++m) c.mat[m] = const_cast<void *>(a->mat[m]);
  c.rmass = const_cast<void *>(a->rmass);
  c.geo[0] = const_cast<void *>(a->xix);
  c.geo[1] = const_cast<void *>(a->etaz);
  c.geo[2] = const_cast<void *>(a->dxdxi);
  c.geo[3] = const_cast<void *>(a->dzdeta);
  c.per_rm = const_cast<void *>(a->per_rm);
  c.per_Ca = const_cast<void *>(a->per_Ca);
  c.per_Cb = const_cast<void *>(a->per_Cb);
  c.nsrc = a->nsrc;
  c.src_I = a->src_I;
  c.src_J = a->src_J;
  c.src_amp = a->src_amp;
  c.nt = a->nt;
  c.step = reinterpret_cast<int *>(scratch);
  c.done = reinterpret_cast<unsigned *>(scratch + 4);
  c.error = a->status ? a->status : reinterpret_cast<int *>(scratch + 8);
  if (const char *e = std::getenv("SEM2D_SPIN_LIMIT")) c.spin_limit = std::max(0, std::atoi(e));
  c.scheme = 0;
  c.dt = a->dt;
  c.cv = a->dt;
  c.kd2 = a->kd2_form ? 1 : 0;
  c.stream = st;
  noalloc_setup_kernel<<<1, 1, 0, st>>>(scratch, a->step0, a->nz, TZ);
  if (const cudaError_t e = cudaGetLastError(); e != cudaSuccess)
    return fail(SEM2D_E_CUDA, std::string("setup launch: ") + cudaGetErrorString(e));
  void *pd = scratch + kFieldOffset, *pv = scratch + kFieldOffset + field_bytes;
  void *bufD[2] = {a->d, pd}, *bufV[2] = {a->v, pv};
  int cur = 0;
  for (int k = 0; k < nsteps; ++k) {
    c.Dcur = bufD[cur];
    c.Dnext = bufD[1 - cur];
    c.Vcur = bufV[cur];
    c.Vnext = bufV[1 - cur];
    if (launch_bulk(c)) return fail(SEM2D_E_CUDA, std::string("launch: ") + bulk_last_error());
    cur = 1 - cur;
  }
  if (cur == 1) {  // the state ended in the scratch: copy it back to the caller
    const size_t n = rs * a->ndof * plane;
    if (cudaMemcpyAsync(a->d, pd, n, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(a->v, pv, n, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return fail(SEM2D_E_CUDA, "copy back failed");
  }
  return SEM2D_OK;
}

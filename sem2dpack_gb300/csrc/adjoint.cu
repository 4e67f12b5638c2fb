// adjoint.cu -- instantiation of the adjoint step kernel (NGLL = 5) and the
// kernels that fold the per-segment gradient sums into FP64 and apply the
// chain rule from (lambda, mu, mass, dashpots) to (rho, vp, vs).
#include <string>

#include "adjoint_kernel.cuh"
#include "bulk_launch.h"

namespace sem2d {

extern thread_local std::string g_bulk_err;

namespace {

template <typename real, int NDOF>
int launch_adj_typed(const AdjConfig &c, bool configure_only) {
  constexpr int N = 5;
  const size_t smem = adj_smem_bytes<real, N, NDOF>(adj_planes(NDOF, c.nmat));
  if (configure_only) {
    const cudaError_t e = cudaFuncSetAttribute(adjoint_step_kernel<real, N, NDOF>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) {
      g_bulk_err = std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e);
      return 1;
    }
    return 0;
  }
  AdjParams<real, N> p{};
  p.LX = c.LX;
  p.LZ = c.LZ;
  p.pitch = c.pitch;
  p.plane = c.plane;
  p.nx = c.nx;
  p.nz = c.nz;
  p.row0 = c.row0;
  p.ztile = c.ztile;
  for (int k = 0; k < N * N; ++k) p.H[k] = real(c.H[k]);
  for (int k = 0; k < N; ++k) p.w[k] = real(c.w[k]);
  p.xix = static_cast<const real *>(c.geo[0]);
  p.etaz = static_cast<const real *>(c.geo[1]);
  p.dxdxi = static_cast<const real *>(c.geo[2]);
  p.dzdeta = static_cast<const real *>(c.geo[3]);
  p.nmat = c.nmat;
  p.mat[0] = static_cast<const real *>(c.mat[0]);
  p.mat[1] = static_cast<const real *>(c.mat[1]);
  p.rmass = static_cast<const real *>(c.rmass);
  p.per_rm = static_cast<const real *>(c.per_rm);
  p.per_Ca = static_cast<const real *>(c.per_Ca);
  p.per_Cb = static_cast<const real *>(c.per_Cb);
  p.Db = static_cast<const real *>(c.Db);
  p.Vb = static_cast<const real *>(c.Vb);
  p.Dbn = static_cast<real *>(c.Dbn);
  p.Vbn = static_cast<real *>(c.Vbn);
  p.d = static_cast<const real *>(c.d);
  p.vprev = static_cast<const real *>(c.vprev);
  p.a = static_cast<const real *>(c.a);
  p.g_la = static_cast<real *>(c.g_la);
  p.g_mu = static_cast<real *>(c.g_mu);
  p.g_M = static_cast<real *>(c.g_M);
  p.g_C = static_cast<real *>(c.g_C);
  p.nrec = c.nrec;
  p.nsamp = c.nsamp;
  p.isamp = c.isamp;
  p.field = c.field;
  p.rec_I = c.rec_I;
  p.rec_J = c.rec_J;
  p.resid = c.resid;
  p.dt = real(c.dt);
  p.kd2 = c.kd2;
  p.it = c.it;
  p.error = c.error;
  adjoint_step_kernel<real, N, NDOF><<<dim3(c.grid_x, c.grid_y), kStripThreads, smem, c.stream>>>(p);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

int dispatch_adj(const AdjConfig &c, bool configure_only) {
  if (c.ndof == 1)
    return c.mixed ? launch_adj_typed<float, 1>(c, configure_only) : launch_adj_typed<double, 1>(c, configure_only);
  return c.mixed ? launch_adj_typed<float, 2>(c, configure_only) : launch_adj_typed<double, 2>(c, configure_only);
}

template <typename real>
__global__ void fold_kernel(real *part, double *acc, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    acc[k] += double(part[k]);
    part[k] = real(0);
  }
}

// Chain rule at every lattice node (I, J):
//   lambda = rho (vp^2 - 2 vs^2), mu = rho vs^2        (mat_elastic.f90:189-321)
//   M0 = sum_e rho W  ->  dM/drho = M0 / rho             (mat_mass.f90:29-61)
//   C  = rho c w |J1D| per side, c = vp on the side's normal dof and vs on the
//        tangential one (bc_abso.f90:195-207): dC/drho = C/rho, dC/dc = C/c
// The normal dof of a dashpot is the one with the larger coefficient (vp > vs).
template <typename real>
__global__ void chain_kernel(ChainConfig c) {
  const long long n = (long long)c.LX * c.LZ;
  const int nslot = perimeter_slots(c.LX, c.LZ);
  const long long plane = (long long)c.pitch * c.LZ;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int I = int(k % c.LX), J = int(k / c.LX);
    const long long g = (long long)J * c.pitch + I;
    const double rho = double(static_cast<const real *>(c.rho)[g]);
    const double mu = double(static_cast<const real *>(c.mu)[g]);
    const double la = c.ndof == 2 ? double(static_cast<const real *>(c.la)[g]) : 0.0;
    const double vs2 = mu / rho, vp2 = (la + 2.0 * mu) / rho;
    const double vs = sqrt(vs2), vp = sqrt(vp2);
    const double gla = c.ndof == 2 ? c.g_la[g] : 0.0, gmu = c.g_mu[g];
    double grho = gla * (vp2 - 2.0 * vs2) + gmu * vs2;
    double gvp = c.ndof == 2 ? gla * (2.0 * rho * vp) : 0.0;
    double gvs = gla * (-4.0 * rho * vs) + gmu * (2.0 * rho * vs);
    const int sp = (J == 0 || J == c.LZ - 1 || I == 0 || I == c.LX - 1) ? perimeter_slot(I, J, c.LX, c.LZ) : -1;
    double m0;
    if (sp >= 0) {
      const double ca0 = double(static_cast<const real *>(c.per_Ca)[sp]);
      const double cb0 = double(static_cast<const real *>(c.per_Cb)[sp]);
      m0 = 1.0 / double(static_cast<const real *>(c.per_rm)[sp]) - 0.5 * c.dt * (ca0 + cb0);
      for (int dash = 0; dash < 2; ++dash) {
        const real *tab = static_cast<const real *>(dash == 0 ? c.per_Ca : c.per_Cb);
        double C[2] = {0, 0};
        for (int q = 0; q < c.ndof; ++q) C[q] = double(tab[q * nslot + sp]);
        const int nrm = c.ndof == 2 ? (C[0] > C[1] ? 0 : 1) : -1;
        for (int q = 0; q < c.ndof; ++q) {
          if (C[q] == 0.0) continue;
          const double gC = c.g_C[q * nslot + sp];
          grho += gC * (C[q] / rho);
          if (q == nrm) gvp += gC * (C[q] / vp);
          else gvs += gC * (C[q] / vs);
        }
      }
    } else {
      m0 = 1.0 / double(static_cast<const real *>(c.rmass)[g]);
    }
    grho += c.g_M[g] * (m0 / rho);
    c.grad_rho[g] = grho;
    c.grad_vp[g] = gvp;
    c.grad_vs[g] = gvs;
  }
  (void)plane;
}

}  // namespace

int configure_adjoint(const AdjConfig &c) { return dispatch_adj(c, true); }
int launch_adjoint(const AdjConfig &c) { return dispatch_adj(c, false); }

int launch_fold(void *part, double *acc64, long long n, int mixed, cudaStream_t s) {
  if (n <= 0) return 0;
  const int blocks = int((n + 255) / 256 > 4096 ? 4096 : (n + 255) / 256);
  if (mixed) fold_kernel<float><<<blocks, 256, 0, s>>>(static_cast<float *>(part), acc64, n);
  else fold_kernel<double><<<blocks, 256, 0, s>>>(static_cast<double *>(part), acc64, n);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

int launch_chain(const ChainConfig &c) {
  const long long n = (long long)c.LX * c.LZ;
  const int blocks = int((n + 255) / 256 > 4096 ? 4096 : (n + 255) / 256);
  if (c.mixed) chain_kernel<float><<<blocks, 256, 0, c.stream>>>(c);
  else chain_kernel<double><<<blocks, 256, 0, c.stream>>>(c);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_bulk_err = cudaGetErrorString(e);
    return 1;
  }
  return 0;
}

}  // namespace sem2d

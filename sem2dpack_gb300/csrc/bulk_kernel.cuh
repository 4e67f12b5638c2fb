// bulk_kernel.cuh -- the fused spectral-element step for one tile of
// elements per CTA.
//
// One launch performs, for every lattice node a CTA owns, what the
// reference does in one pass of solve_leapfrog / solve_Newmark
// (solver.f90:42-83, 140-161):
//   f = -K d            compute_Fint (solver.f90:273-316) with MAT_Fint ->
//                       ELAST_KD1/KD2 (mat_elastic.f90:464-775) and the
//                       Kelvin-Voigt term (mat_kelvin_voigt.f90:137-151)
//   f += sources        SO_add (src_gen.f90:290-317)
//   f -= C v            BC_ABSO_apply (bc_abso.f90:286-319)
//   a = rmass f, v += c a, next displacement predictor
// Fault-row nodes only get f; the fault kernel finishes them.
//
// Work decomposition.  A CTA owns the lattice nodes of a TX x TZ tile of
// elements (lower-left convention).  Nodes on its left/bottom edges also
// receive forces from the neighbouring element column/row, so those
// elements are recomputed (a one-element halo).  Displacements of the tile
// (with halo) are staged in shared memory once; elements are processed in
// the four parity colours of the element lattice, so elements of one
// colour never share a node and add into the shared force tile without
// atomics; the per-node sum is therefore in a fixed order.
//
// Element operator.  For an N x N element the gradients dU/dxi = H^T U and
// dU/deta = U H and the divergence H tmp + tmp H^T are computed with N
// threads per element: thread t owns column t for the xi-contractions and
// row t for the eta-contractions, keeping each N-vector in registers (N
// shared loads per contraction instead of N^2).  The P-SV cross terms are
// exchanged through a per-warp scratch area.
#pragma once

#include "sem2d_common.cuh"

namespace sem2d {

template <int N, int NDOF>
struct BulkShape {
  static constexpr int kSlots = 32 / N;             // elements per warp
  static constexpr int kScr = (NDOF == 2 ? 4 : 1);  // scratch planes per element
};

// shared-memory footprint (bytes) of one CTA, same arithmetic as the kernel
template <typename real, int N, int NDOF>
__host__ __device__ inline size_t bulk_smem_bytes(int tile_nodes, int nmat_planes, int has_kv,
                                                  int mat_elem) {
  const int nwarps = kBulkThreads / 32;
  size_t n = size_t(tile_nodes) * NDOF * 2;                 // D, F
  if (!mat_elem) n += size_t(tile_nodes) * nmat_planes;     // material
  if (has_kv) n += size_t(tile_nodes) * NDOF;               // V for Kelvin-Voigt
  n += size_t(nwarps) * BulkShape<N, NDOF>::kSlots * BulkShape<N, NDOF>::kScr * N * N;
  return n * sizeof(real);
}

template <typename real, int N, int NDOF>
__global__ void __launch_bounds__(kBulkThreads)
    bulk_step_kernel(const BulkParams<real, N> p, const int tile_nodes, const int nmat,
                     const int has_kv) {
  constexpr int NN = N * N;
  constexpr int SLOTS = BulkShape<N, NDOF>::kSlots;
  constexpr int NSCR = BulkShape<N, NDOF>::kScr;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  real *sD = reinterpret_cast<real *>(smem_raw);
  real *sF = sD + size_t(tile_nodes) * NDOF;
  real *sM = sF + size_t(tile_nodes) * NDOF;
  real *sV = sM + (p.mat_elem ? 0 : size_t(tile_nodes) * nmat);
  real *sS = sV + (has_kv ? size_t(tile_nodes) * NDOF : 0);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const int ex0 = blockIdx.x * p.TX, ez0 = blockIdx.y * p.TZ;
  const int ex1 = min(ex0 + p.TX, p.nx), ez1 = min(ez0 + p.TZ, p.nz);
  const int hx = ex0 > 0 ? 1 : 0;
  const int hz = (ez0 > 0 && p.row0[ez0] == p.row0[ez0 - 1] + (N - 1)) ? 1 : 0;
  const int exa = ex0 - hx, eza = ez0 - hz;
  const int Ia = exa * (N - 1), Ib = (ex1 - 1) * (N - 1) + N;
  const int Ja = p.row0[eza], Jb = p.row0[ez1 - 1] + N;
  const int TW = Ib - Ia, TH = Jb - Ja;
  const int I0 = ex0 * (N - 1), I1 = (ex1 == p.nx) ? p.LX : ex1 * (N - 1);
  const int J0 = p.row0[ez0], J1 = p.row0[ez1];  // row0[nz] == LZ

  // ---- 1. stage the tile: displacement (+velocity for KV), material ----
  for (int idx = tid; idx < TW * TH; idx += blockDim.x) {
    const int I = Ia + idx % TW, J = Ja + idx / TW;
    const long long g = (long long)J * p.pitch + I;
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      sD[c * tile_nodes + idx] = p.Dcur[c * p.plane + g];
      sF[c * tile_nodes + idx] = real(0);
      if (has_kv) {
        real v = p.Vcur[c * p.plane + g];
        if (p.scheme == 1) v = v + p.cpred * p.Acur[c * p.plane + g];
        sV[c * tile_nodes + idx] = v;
      }
    }
    if (!p.mat_elem)
      for (int m = 0; m < nmat; ++m) sM[m * tile_nodes + idx] = p.mat[m][g];
  }
  __syncthreads();

  // ---- 2. element forces, four parity colours ----
  const int nEx = ex1 - exa, nEz = ez1 - eza;
  const int slot = lane / N, t = lane - slot * N;
  const bool lane_ok = slot < SLOTS;
  real *scr = sS + (size_t(warp) * SLOTS + (lane_ok ? slot : 0)) * NSCR * NN;

  for (int colour = 0; colour < 4; ++colour) {
    const int px = colour & 1, pz = colour >> 1;
    const int fx = ((exa & 1) == px) ? 0 : 1;  // first local column of this parity
    const int fz = ((eza & 1) == pz) ? 0 : 1;
    const int nxc = nEx > fx ? (nEx - fx + 1) / 2 : 0;
    const int nzc = nEz > fz ? (nEz - fz + 1) / 2 : 0;
    const int ncol = nxc * nzc;
    for (int base = warp * SLOTS; base < ncol; base += nwarps * SLOTS) {
      const int k = base + slot;
      const bool act = lane_ok && k < ncol;
      int ex = 0, ez = 0, eb = 0;
      if (act) {
        const int lx = fx + 2 * (k % nxc), lz = fz + 2 * (k / nxc);
        ex = exa + lx;
        ez = eza + lz;
        eb = (p.row0[ez] - Ja) * TW + (ex * (N - 1) - Ia);
      }
      // material / geometry of this element
      real xix = 0, etaz = 0, det = 0;
      const real *kve = nullptr;
      if (act) {
        xix = p.xix[ex];
        etaz = p.etaz[ez];
        det = p.dxdxi[ex] * p.dzdeta[ez];
        if (has_kv) kve = p.kveta + ((long long)ez * p.nx + ex) * NN;
      }
      const long long eoff = ((long long)ez * p.nx + ex) * NN;
      auto matv = [&](int m, int i, int j) -> real {
        return p.mat_elem ? p.mat[m][eoff + i + N * j] : sM[m * tile_nodes + eb + j * TW + i];
      };
      auto uval = [&](int c, int i, int j) -> real {
        real u = sD[c * tile_nodes + eb + j * TW + i];
        if (has_kv) u = u + kve[i + N * j] * sV[c * tile_nodes + eb + j * TW + i];
        return u;
      };

      if (NDOF == 1) {
        real col[N], row[N], gxi[N], geta[N];
        if (act) {
#pragma unroll
          for (int q = 0; q < N; ++q) {
            col[q] = uval(0, q, t);
            row[q] = uval(0, t, q);
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[0 + N * i] * col[0];
#pragma unroll
            for (int q = 1; q < N; ++q) a = a + p.H[q + N * i] * col[q];
            gxi[i] = a;
          }
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = row[0] * p.H[0 + N * j];
#pragma unroll
            for (int q = 1; q < N; ++q) a = a + row[q] * p.H[q + N * j];
            geta[j] = a;
          }
          // column part: points (q,t); row part: points (t,q)
#pragma unroll
          for (int q = 0; q < N; ++q) {
            const real mux = p.mat_iso ? matv(0, q, t) : matv(1, q, t);
            const real W1 = det * (p.w[q] * p.w[t]);
            col[q] = -(W1 * ((mux * xix) * xix)) * gxi[q];
            const real mu = matv(0, t, q);
            const real W2 = det * (p.w[t] * p.w[q]);
            row[q] = -(W2 * ((mu * etaz) * etaz)) * geta[q];
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[i + N * 0] * col[0];
#pragma unroll
            for (int q = 1; q < N; ++q) a = a + p.H[i + N * q] * col[q];
            scr[i + N * t] = a;  // column part at (i,t)
          }
        }
        __syncwarp();
        if (act) {
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = row[0] * p.H[j + N * 0];
#pragma unroll
            for (int q = 1; q < N; ++q) a = a + row[q] * p.H[j + N * q];
            const real fl = scr[t + N * j] + a;
            sF[eb + j * TW + t] += fl;
          }
        }
        __syncwarp();
      } else {
        real cx[N], cz[N], rx[N], rz[N];  // loads, then reused
        real gxx[N], gxz[N], gex[N], gez[N];
        real *SXX = scr, *SXZ = scr + NN, *SEX = scr + 2 * NN, *SEZ = scr + 3 * NN;
        if (act) {
#pragma unroll
          for (int q = 0; q < N; ++q) {
            cx[q] = uval(0, q, t);
            cz[q] = uval(1, q, t);
            rx[q] = uval(0, t, q);
            rz[q] = uval(1, t, q);
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[0 + N * i] * cx[0], b = p.H[0 + N * i] * cz[0];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + p.H[q + N * i] * cx[q];
              b = b + p.H[q + N * i] * cz[q];
            }
            gxx[i] = a;  // dUx/dxi at (i,t)
            gxz[i] = b;  // dUz/dxi at (i,t)
          }
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = rx[0] * p.H[0 + N * j], b = rz[0] * p.H[0 + N * j];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + rx[q] * p.H[q + N * j];
              b = b + rz[q] * p.H[q + N * j];
            }
            gex[j] = a;  // dUx/deta at (t,j)
            gez[j] = b;  // dUz/deta at (t,j)
          }
#pragma unroll
          for (int q = 0; q < N; ++q) {
            SXX[q + N * t] = gxx[q];
            SXZ[q + N * t] = gxz[q];
            SEX[t + N * q] = gex[q];
            SEZ[t + N * q] = gez[q];
          }
        }
        __syncwarp();
        if (act) {
          // column part at points (q,t) and row part at points (t,q)
#pragma unroll
          for (int q = 0; q < N; ++q) {
            real la, mu, Kx, Kz;
            if (p.mat_iso) {
              la = matv(0, q, t);
              mu = matv(1, q, t);
              Kx = la + real(2) * mu;
            } else {
              Kx = matv(0, q, t);
              la = matv(2, q, t);
              mu = matv(3, q, t);
            }
            const real W = det * (p.w[q] * p.w[t]);
            const real a1 = -(W * ((Kx * xix) * xix));
            const real a2 = -(W * ((la * xix) * etaz));
            const real a5 = -(W * ((mu * xix) * etaz));
            const real a6 = -(W * ((mu * xix) * xix));
            cx[q] = a1 * gxx[q] + a2 * SEZ[q + N * t];
            cz[q] = a5 * SEX[q + N * t] + a6 * gxz[q];
          }
#pragma unroll
          for (int q = 0; q < N; ++q) {
            real la, mu, Kz;
            if (p.mat_iso) {
              la = matv(0, t, q);
              mu = matv(1, t, q);
              Kz = la + real(2) * mu;
            } else {
              Kz = matv(1, t, q);
              la = matv(2, t, q);
              mu = matv(3, t, q);
            }
            const real W = det * (p.w[t] * p.w[q]);
            const real a2 = -(W * ((la * xix) * etaz));
            const real a3 = -(W * ((Kz * etaz) * etaz));
            const real a4 = -(W * ((mu * etaz) * etaz));
            const real a5 = -(W * ((mu * xix) * etaz));
            const real gzx = SXZ[t + N * q], gxx_r = SXX[t + N * q];
            rx[q] = p.kd2 ? a4 * (gex[q] + gzx) : a4 * gex[q] + a5 * gzx;
            rz[q] = a2 * gxx_r + a3 * gez[q];
          }
        }
        __syncwarp();
        if (act) {
          // divergence: column part -> scratch, row part summed by row owner
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[i + N * 0] * cx[0], b = p.H[i + N * 0] * cz[0];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + p.H[i + N * q] * cx[q];
              b = b + p.H[i + N * q] * cz[q];
            }
            SXX[i + N * t] = a;
            SXZ[i + N * t] = b;
          }
        }
        __syncwarp();
        if (act) {
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = rx[0] * p.H[j + N * 0], b = rz[0] * p.H[j + N * 0];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + rx[q] * p.H[j + N * q];
              b = b + rz[q] * p.H[j + N * q];
            }
            const int ti = eb + j * TW + t;
            sF[ti] += SXX[t + N * j] + a;
            sF[tile_nodes + ti] += SXZ[t + N * j] + b;
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();
  }

  // ---- 3. point sources at owned nodes (in source order) ----
  const int it = *p.step + 1;
  if (tid == 0 && p.nsrc > 0) {
    for (int s = 0; s < p.nsrc; ++s) {
      const int I = p.src_I[s], J = p.src_J[s];
      if (I >= I0 && I < I1 && J >= J0 && J < J1 && it <= p.nt) {
        const int ti = (J - Ja) * TW + (I - Ia);
        for (int c = 0; c < NDOF; ++c)
          sF[c * tile_nodes + ti] += real(p.src_amp[((long long)s * NDOF + c) * (p.nt + 1) + it]);
      }
    }
  }
  __syncthreads();

  // ---- 4. absorbing dashpots, inverse mass, time update of owned nodes ----
  const int OW = I1 - I0, OH = J1 - J0;
  for (int idx = tid; idx < OW * OH; idx += blockDim.x) {
    const int I = I0 + idx % OW, J = J0 + idx / OW;
    const int ti = (J - Ja) * TW + (I - Ia);
    const long long g = (long long)J * p.pitch + I;
    const int slot_p = perimeter_slot(I, J, p.LX, p.LZ);
    const int nslot = perimeter_slots(p.LX, p.LZ);
    const bool fault_row = (J == p.jf1 || J == p.jf2);
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      real f = sF[c * tile_nodes + ti];
      const real vold = p.Vcur[c * p.plane + g];
      real vpred = vold;
      if (p.scheme == 1) vpred = vold + p.cpred * p.Acur[c * p.plane + g];
      real rm;
      if (slot_p >= 0) {
        const int so = c * nslot + slot_p;
        f = f - p.per_Ca[so] * vpred;
        f = f - p.per_Cb[so] * vpred;
        rm = p.per_rm[so];
      } else {
        rm = p.rmass[g];
      }
      if (fault_row) {
        const int side = (J == p.jf1) ? 0 : 1;
        p.f_flt[(side * NDOF + c) * p.LX + I] = f;
        continue;
      }
      const real a = rm * f;
      const real vnew = vpred + p.cv * a;
      const real dcur = sD[c * tile_nodes + ti];
      real dnext;
      if (p.scheme == 1)
        dnext = (dcur + p.dt * vnew) + p.cd2 * a;
      else
        dnext = dcur + p.dt * vnew;
      p.Vnext[c * p.plane + g] = vnew;
      p.Dnext[c * p.plane + g] = dnext;
      if (p.Anext) p.Anext[c * p.plane + g] = a;
    }
  }
}

}  // namespace sem2d

// bulk_kernel.cuh -- one fused launch per time step.
//
// For every lattice node a CTA owns, one launch performs what the reference
// does in one pass of solve_leapfrog / solve_Newmark (solver.f90:42-83,
// 140-161):
//   f = -K d            compute_Fint (solver.f90:273-316) with MAT_Fint ->
//                       ELAST_KD1/KD2 (mat_elastic.f90:464-775) and the
//                       Kelvin-Voigt term (mat_kelvin_voigt.f90:137-151)
//   f += sources        SO_add (src_gen.f90:290-317)
//   f -= C v            BC_ABSO_apply (bc_abso.f90:286-319)
//   dynamic fault       BC_DYNFLT_apply (bc_dynflt.f90:569-739), FP64
//   a = rmass f, v += c a, next displacement predictor
//   seismograms         REC_store (receivers.f90:309-344) for the receivers
//                       the CTA owns
// and the last CTA to finish advances the device step counter, so a time
// step is a single kernel node in the captured CUDA graph.
//
// Work decomposition.  A CTA owns the lattice nodes of a tile of TX element
// columns by ztile[y]..ztile[y+1] element rows (lower-left convention).
// Nodes on its left/bottom edges also receive forces from the neighbouring
// element column/row, so those elements are recomputed (a one-element
// halo).  The host places tile-row boundaries away from a fault split, so
// both split rows of a fault belong to the same CTA.  Displacement (and the
// material when it is stored per node) of the tile with its halo, and the
// velocity and inverse mass of the owned nodes, are staged in shared memory
// up front; elements are processed in the four parity colours of the
// element lattice, so elements of one colour never share a node and add
// into the shared force tile without atomics, in a fixed order per node.
//
// Element operator.  For an N x N element the gradients dU/dxi = H^T U and
// dU/deta = U H and the divergence H tmp + tmp H^T are computed with N
// threads per element: thread t owns column t for the xi-contractions and
// row t for the eta-contractions, keeping each N-vector in registers (N
// shared loads per contraction instead of N^2).  The P-SV cross terms are
// exchanged through a per-warp scratch area.
#pragma once

#include "fault_kernel.cuh"
#include "sem2d_common.cuh"

namespace sem2d {

template <int N, int NDOF>
struct BulkShape {
  static constexpr int kSlots = 32 / N;             // elements per warp
  static constexpr int kScr = (NDOF == 2 ? 4 : 1);  // scratch planes per element
};

// shared-memory footprint (bytes) of one CTA, same arithmetic as the kernel
template <typename real, int N, int NDOF>
__host__ __device__ inline size_t bulk_smem_bytes(int tile_nodes, int own_nodes, int nmat_planes,
                                                  int has_kv, int mat_elem) {
  const int nwarps = kBulkThreads / 32;
  size_t n = size_t(tile_nodes) * NDOF * 2;                 // D, F
  if (!mat_elem) n += size_t(tile_nodes) * nmat_planes;     // material
  if (has_kv) n += size_t(tile_nodes) * NDOF;               // V of the tile (Kelvin-Voigt)
  n += size_t(own_nodes) * (NDOF + 1);                      // owned V, rmass
  n += size_t(nwarps) * BulkShape<N, NDOF>::kSlots * BulkShape<N, NDOF>::kScr * N * N;
  return n * sizeof(real);
}

// minimum resident CTAs per SM the register allocation is sized for
template <typename real>
struct BulkOccupancy {
  static constexpr int kMinBlocks = sizeof(real) == 4 ? 4 : 2;
};

template <typename real, int N, int NDOF, bool MELEM>
__global__ void __launch_bounds__(kBulkThreads, BulkOccupancy<real>::kMinBlocks)
    bulk_step_kernel(const BulkParams<real, N> p, const int tile_nodes, const int own_nodes,
                     const int nmat, const int has_kv) {
  constexpr int NN = N * N;
  constexpr int SLOTS = BulkShape<N, NDOF>::kSlots;
  constexpr int NSCR = BulkShape<N, NDOF>::kScr;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  real *sD = reinterpret_cast<real *>(smem_raw);
  real *sF = sD + size_t(tile_nodes) * NDOF;
  real *sM = sF + size_t(tile_nodes) * NDOF;
  real *sV = sM + (MELEM ? 0 : size_t(tile_nodes) * nmat);
  real *sVo = sV + (has_kv ? size_t(tile_nodes) * NDOF : 0);
  real *sRm = sVo + size_t(own_nodes) * NDOF;
  real *sS = sRm + own_nodes;

  const int it = *p.step + 1;  // the step this launch computes
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = blockDim.x >> 5;
  const int ex0 = blockIdx.x * p.TX, ex1 = min(ex0 + p.TX, p.nx);
  const int ez0 = p.ztile[blockIdx.y], ez1 = p.ztile[blockIdx.y + 1];
  const int hx = ex0 > 0 ? 1 : 0;
  const int hz = (ez0 > 0 && p.row0[ez0] == p.row0[ez0 - 1] + (N - 1)) ? 1 : 0;
  const int exa = ex0 - hx, eza = ez0 - hz;
  const int Ia = exa * (N - 1), Ib = (ex1 - 1) * (N - 1) + N;
  const int Ja = p.row0[eza], Jb = p.row0[ez1 - 1] + N;
  const int TW = Ib - Ia, TH = Jb - Ja;
  const int I0 = ex0 * (N - 1), I1 = (ex1 == p.nx) ? p.LX : ex1 * (N - 1);
  const int J0 = p.row0[ez0], J1 = p.row0[ez1];  // row0[nz] == LZ
  const int OW = I1 - I0, OH = J1 - J0;

  // ---- 1. stage the tile (with halo) and the owned nodes ----
  for (int j = warp; j < TH; j += nwarps) {
    const long long rowg = (long long)(Ja + j) * p.pitch + Ia;
    for (int i = lane; i < TW; i += 32) {
      const int idx = j * TW + i;
      const long long g = rowg + i;
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
      if (!MELEM)
        for (int m = 0; m < nmat; ++m) sM[m * tile_nodes + idx] = p.mat[m][g];
    }
  }
  for (int j = warp; j < OH; j += nwarps) {
    const long long rowg = (long long)(J0 + j) * p.pitch + I0;
    for (int i = lane; i < OW; i += 32) {
      const int o = j * OW + i;
      const long long g = rowg + i;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        real v = p.Vcur[c * p.plane + g];
        if (p.scheme == 1) v = v + p.cpred * p.Acur[c * p.plane + g];
        sVo[c * own_nodes + o] = v;  // velocity predictor
      }
      sRm[o] = p.rmass[g];
    }
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
      real xix = 0, etaz = 0, det = 0;
      if (act) {
        const int kz = k / nxc;
        ex = exa + fx + 2 * (k - kz * nxc);
        ez = eza + fz + 2 * kz;
        eb = (p.row0[ez] - Ja) * TW + (ex * (N - 1) - Ia);
        xix = p.xix[ex];
        etaz = p.etaz[ez];
        det = p.dxdxi[ex] * p.dzdeta[ez];
      }
      const long long eoff = ((long long)ez * p.nx + ex) * NN;
      const real *kve = has_kv ? p.kveta + eoff : nullptr;
      auto matv = [&](int m, int i, int j) -> real {
        if (MELEM) return p.mat[m][eoff + i + N * j];
        return sM[m * tile_nodes + eb + j * TW + i];
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
          // column part at points (q,t), row part at points (t,q)
          if (p.mat_iso) {
#pragma unroll
            for (int q = 0; q < N; ++q) {
              const real mux = matv(0, q, t), mu = matv(0, t, q);
              col[q] = -((det * (p.w[q] * p.w[t])) * ((mux * xix) * xix)) * gxi[q];
              row[q] = -((det * (p.w[t] * p.w[q])) * ((mu * etaz) * etaz)) * geta[q];
            }
          } else {
#pragma unroll
            for (int q = 0; q < N; ++q) {
              const real mux = matv(1, q, t), mu = matv(0, t, q);
              col[q] = -((det * (p.w[q] * p.w[t])) * ((mux * xix) * xix)) * gxi[q];
              row[q] = -((det * (p.w[t] * p.w[q])) * ((mu * etaz) * etaz)) * geta[q];
            }
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
            sF[eb + j * TW + t] += scr[t + N * j] + a;
          }
        }
        __syncwarp();
      } else {
        real cx[N], cz[N], rx[N], rz[N];
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
#pragma unroll
          for (int q = 0; q < N; ++q) {
            // column part at point (q,t)
            real la, mu, Kx;
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
            // row part at point (t,q)
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
  if (tid == 0 && p.nsrc > 0 && it <= p.nt) {
    for (int s = 0; s < p.nsrc; ++s) {
      const int I = p.src_I[s], J = p.src_J[s];
      if (I >= I0 && I < I1 && J >= J0 && J < J1) {
        const int ti = (J - Ja) * TW + (I - Ia);
        for (int c = 0; c < NDOF; ++c)
          sF[c * tile_nodes + ti] += real(p.src_amp[((long long)s * NDOF + c) * (p.nt + 1) + it]);
      }
    }
  }
  __syncthreads();

  // ---- 4. absorbing dashpots, inverse mass, time update of owned nodes ----
  const int nslot = perimeter_slots(p.LX, p.LZ);
  for (int j = warp; j < OH; j += nwarps) {
    const int J = J0 + j;
    const bool fault_row = (J == p.jf1 || J == p.jf2);
    const bool edge_row = (J == 0 || J == p.LZ - 1);
    for (int i = lane; i < OW; i += 32) {
      const int I = I0 + i;
      const int o = j * OW + i;
      const int ti = (J - Ja) * TW + (I - Ia);
      const long long g = (long long)J * p.pitch + I;
      const int sp = (edge_row || I == 0 || I == p.LX - 1) ? perimeter_slot(I, J, p.LX, p.LZ) : -1;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        real f = sF[c * tile_nodes + ti];
        const real vpred = sVo[c * own_nodes + o];
        real rm;
        if (sp >= 0) {
          const int so = c * nslot + sp;
          f = f - p.per_Ca[so] * vpred;
          f = f - p.per_Cb[so] * vpred;
          rm = p.per_rm[so];
        } else {
          rm = sRm[o];
        }
        if (fault_row) {  // finished by the fault phase below
          sF[c * tile_nodes + ti] = f;
          continue;
        }
        const real a = rm * f;
        const real vnew = vpred + p.cv * a;
        const real dcur = sD[c * tile_nodes + ti];
        const real dnext = p.scheme == 1 ? (dcur + p.dt * vnew) + p.cd2 * a : dcur + p.dt * vnew;
        p.Vnext[c * p.plane + g] = vnew;
        p.Dnext[c * p.plane + g] = dnext;
        if (p.Anext) p.Anext[c * p.plane + g] = a;
      }
    }
  }

  // ---- 5. fault nodes of this tile (FP64) ----
  const bool fault_here = p.has_fault && p.jf1 >= J0 && p.jf1 < J1;
  const int nrec_here = p.rec_tile_start ? p.rec_tile_start[blockIdx.y * gridDim.x + blockIdx.x + 1] -
                                               p.rec_tile_start[blockIdx.y * gridDim.x + blockIdx.x]
                                         : 0;
  if (fault_here || nrec_here) __syncthreads();
  if (fault_here) {
    for (int I = I0 + tid; I < I1; I += blockDim.x) {
      double f1[2] = {0, 0}, f2[2] = {0, 0};
      for (int c = 0; c < NDOF; ++c) {
        f1[c] = double(sF[c * tile_nodes + (p.jf1 - Ja) * TW + (I - Ia)]);
        if (p.flt.two) f2[c] = double(sF[c * tile_nodes + (p.jf2 - Ja) * TW + (I - Ia)]);
      }
      fault_node_update(p.flt, I, it, f1, f2);
    }
  }

  // ---- 6. seismograms of the receivers owned by this tile ----
  if (nrec_here) {
    if (fault_here) __syncthreads();
    const int s = it / p.rec_isamp;
    if (it % p.rec_isamp == 0 && s < p.rec_nsamp) {
      const int r0 = p.rec_tile_start[blockIdx.y * gridDim.x + blockIdx.x];
      for (int q = tid; q < nrec_here * NDOF; q += blockDim.x) {
        const int r = p.rec_ids[r0 + q % nrec_here], c = q / nrec_here;
        double val;
        if (p.rec_npts == 1) {  // receiver at a node: D, V or A
          const int I = p.rec_I[r], J = p.rec_J[r];
          val = p.rec_field == 'D' ? double(sD[c * tile_nodes + (J - Ja) * TW + (I - Ia)])
                : p.rec_field == 'V' ? double(p.Vnext[c * p.plane + (long long)J * p.pitch + I])
                                     : double(p.Anext[c * p.plane + (long long)J * p.pitch + I]);
        } else {  // interpolated displacement; the element lies in this tile
          const int *RI = p.rec_I + (size_t)r * p.rec_npts, *RJ = p.rec_J + (size_t)r * p.rec_npts;
          const double *W = p.rec_w + (size_t)r * p.rec_npts;
          val = W[0] * double(sD[c * tile_nodes + (RJ[0] - Ja) * TW + (RI[0] - Ia)]);
          for (int k = 1; k < p.rec_npts; ++k)
            val = val + W[k] * double(sD[c * tile_nodes + (RJ[k] - Ja) * TW + (RI[k] - Ia)]);
        }
        p.sis[s + (size_t)p.rec_nsamp * (r + (size_t)p.rec_nrec * c)] = val;
      }
    }
  }

  // ---- 7. the last CTA to finish advances the step counter ----
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(p.done, 1u);
    if (prev == gridDim.x * gridDim.y - 1) {
      *p.done = 0u;
      __threadfence();
      *p.step = it;
    }
  }
}

}  // namespace sem2d

// adjoint_kernel.cuh -- one reverse time step of the discrete adjoint of the
// leapfrog scheme and the material-gradient accumulation, in the same
// strip/batch/TMA structure as the forward step kernel.
//
// Forward step n (solve_leapfrog, solver.f90:140-161; the state read at step
// n is d^n and v^{n-1}):
//   v^n = v^{n-1} + dt M^{-1} ( F(theta) d^n - C v^{n-1} + s^n ),
//   d^{n+1} = d^n + dt v^n,
// with F = -K the element-force operator (compute_Fint), M the inverse-mass
// diagonal with the absorbing fold M0 + dt/2 C (bc_abso.f90:243) and C the
// absorbing dashpots.  With Db = dJ/dd^{n+1}, Vb = dJ/dv^{n+1} (total
// derivatives of the misfit J through every later step), one reverse step is
//   Vb^n     = g_v^n + dt Db^{n+1} + (I - dt M^{-1} C) Vb^{n+1}
//   lambda^n = dt M^{-1} Vb^n
//   Db^n     = g_d^n + Db^{n+1} + F(theta) lambda^n      (K is symmetric)
// where g_v, g_d are the misfit derivatives with respect to the recorded
// velocity or displacement (the adjoint sources at the receivers).  The
// gradient with respect to the parameters theta collects, for every step,
//   lambda^n . dF/dtheta d^n              (moduli at every element point)
//   - lambda^n . a^n dM/dtheta            (mass, and the dt/2 C fold)
//   - lambda^n . v^{n-1} dC/dtheta        (dashpots)
// The moduli part at an element point q of weight W is, for the element
// force of the stress form used by the forward kernel,
//   d/dla = -W div(lambda) div(d)
//   d/dmu = -W [2 xix^2 dxi lx dxi dx + 2 etaz^2 deta lz deta dz
//               + xix dxi lz (etaz deta dx + xix dxi dz)
//               + etaz deta lx (etaz deta dx + s dxi dz)]
// (s = etaz for the NGLL=5 KD2 form, xix otherwise), summed over the
// elements around each node.  The kernel accumulates those per node in the
// precision of the fields; the host folds them into FP64 every segment.
//
// This kernel covers the problems of the gradient workflow: NGLL = 5,
// isotropic material continuous at nodes (node planes lambda, mu),
// leapfrog, no Kelvin-Voigt, no 2.5D term, no fault, receivers at nodes.
#pragma once

#include <type_traits>

#include "sem2d_common.cuh"
#include "strip_kernel.cuh"
#include "tma.cuh"

namespace sem2d {

template <typename real, int N>
struct AdjParams {
  int LX, LZ, pitch;
  long long plane;
  int nx, nz;
  const int *row0;
  const int *ztile;
  real H[N * N], w[N];
  const real *xix, *etaz, *dxdxi, *dzdeta;
  int nmat;                    // 2 (lambda, mu) for P-SV, 1 (mu) for SH
  const real *mat[2];
  const real *rmass;           // plane
  const real *per_rm, *per_Ca, *per_Cb;  // perimeter tables [c*nslot + slot]
  const real *Db, *Vb;         // adjoint state of step n+1
  real *Dbn, *Vbn;             // adjoint state of step n (written)
  const real *d;               // forward d^n
  const real *vprev;           // forward v^{n-1}
  const real *a;               // forward a^n
  real *g_la, *g_mu, *g_M;     // per-node partial sums (planes)
  real *g_C;                   // per perimeter slot and dof [c*nslot + slot]
  // misfit derivatives at the receivers, laid out like the seismograms
  int nrec, nsamp, isamp;
  char field;                  // 'V' or 'D'
  const int *rec_I, *rec_J;
  const double *resid;         // [s + nsamp*(r + nrec*c)]
  real dt;
  int kd2;
  int it;                      // the forward step n being reversed
  int *error;
};

// planes of an adjoint stage: Db, Vb, d (ndof each), moduli, inverse mass
__host__ __device__ inline int adj_planes(int ndof, int nmat) { return 3 * ndof + nmat + 1; }

template <typename real, int N, int NDOF>
__host__ __device__ inline size_t adj_smem_bytes(int nplanes) {
  using S = StripShape<real, N>;
  constexpr int tw = strip_row_stride<real, N>();
  size_t n = 2 * size_t(nplanes) * S::HR * tw;  // two stages
  n += 2 * size_t(NDOF) * S::HR * tw;          // lambda and the misfit derivative over the stage
  n += size_t(S::kNSlot) * 4 * N * N;          // element scratch: gradients, forces, moduli terms
  n += 2 * size_t(NDOF + 2) * tw;              // carry rows (forces, two moduli terms), double-buffered
  return n * sizeof(real);
}

template <typename real, int N, int NDOF>
__global__ void __launch_bounds__(kStripThreads, sizeof(real) == 4 ? 2 : 1) adjoint_step_kernel(const __grid_constant__ AdjParams<real, N> p) {
  using S = StripShape<real, N>;
  constexpr int NN = N * N, SL = S::kSlots, SW1 = S::SW1, R = S::R, HR = S::HR, AL = S::AL;
  constexpr int TWp = strip_row_stride<real, N>();
  constexpr int PS = HR * TWp;
  constexpr int NW = kStripThreads / 32;
  constexpr int NSC = 4;  // scratch planes per element
  constexpr int NC = NDOF + 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ signed char s_r[2][HR], s_j[2][HR], s_stat[HR];
  __shared__ int s_err;
  __shared__ int s_row0[kMaxChunk + 2];
  __shared__ real s_etaz[kMaxChunk + 1], s_dzdeta[kMaxChunk + 1];
  __shared__ real s_xix[SW1], s_dxdxi[SW1];

  const int NP = adj_planes(NDOF, p.nmat);
  const size_t stage_sz = size_t(NP) * PS;
  real *stg = reinterpret_cast<real *>(smem_raw);
  real *sL = stg + 2 * stage_sz;       // lambda^n over the stage
  real *sG = sL + NDOF * PS;           // misfit derivative (velocity or displacement)
  real *scr = sG + NDOF * PS;
  real *carry = scr + size_t(S::kNSlot) * NSC * NN;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int SW = SW1 - 1;
  const int ex0 = blockIdx.x * SW, ex1 = min(ex0 + SW, p.nx);
  const int hx = ex0 > 0 ? 1 : 0;
  const int exa = ex0 - hx, ncol = ex1 - exa;
  const int Ia = exa * (N - 1), Ib = (ex1 - 1) * (N - 1) + N;
  const int Ial = Ia & ~(AL - 1), xo = Ia - Ial;
  const int cw = ((Ib + AL - 1) & ~(AL - 1)) - Ial;
  const int I0 = ex0 * (N - 1), I1 = (ex1 == p.nx) ? p.LX : ex1 * (N - 1);
  const int OWc = I1 - I0, ii0 = I0 - Ia;
  const int ez0 = p.ztile[blockIdx.y], ez1 = p.ztile[blockIdx.y + 1];
  const int hz = (ez0 > 0 && p.row0[ez0] == p.row0[ez0 - 1] + (N - 1)) ? 1 : 0;
  const int eza = ez0 - hz;
  const int nb = (ez1 - eza + R - 1) / R;
  const int it = p.it;
  const int nslot = perimeter_slots(p.LX, p.LZ);
  const bool sampled = it % p.isamp == 0 && it / p.isamp < p.nsamp;
  const int samp = it / p.isamp;

  for (int k = tid; k <= ez1 - eza; k += kStripThreads) {
    s_row0[k] = p.row0[eza + k];
    if (k < ez1 - eza) {
      s_etaz[k] = p.etaz[eza + k];
      s_dzdeta[k] = p.dzdeta[eza + k];
    }
  }
  for (int k = tid; k < ncol; k += kStripThreads) {
    s_xix[k] = p.xix[exa + k];
    s_dxdxi[k] = p.dxdxi[exa + k];
  }
  if (tid == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
    s_err = 0;
  }
  __syncthreads();
  auto rw = [&](int ez) { return s_row0[ez - eza]; };
  const int J0own = rw(ez0), J1own = rw(ez1);

  auto plane_src = [&](int pl) -> const real * {
    if (pl < NDOF) return p.Db + pl * p.plane;
    if (pl < 2 * NDOF) return p.Vb + (pl - NDOF) * p.plane;
    if (pl < 3 * NDOF) return p.d + (pl - 2 * NDOF) * p.plane;
    if (pl < 3 * NDOF + p.nmat) return p.mat[pl - 3 * NDOF];
    return p.rmass;
  };
  auto issue = [&](int bb) {
    const int st = bb & 1;
    const int eb0 = eza + bb * R, eb1 = min(eb0 + R, ez1);
    const int Jlo = rw(eb0), nr = rw(eb1 - 1) + N - Jlo;
    const uint32_t rowbytes = uint32_t(cw) * sizeof(real);
    if (tid == 0) mbar_arrive_expect_tx(&bar[st], rowbytes * uint32_t(nr * NP));
    real *base = stg + st * stage_sz;
    for (int q = tid; q < nr * NP; q += kStripThreads) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      const int pl = q / nr, row = q - pl * nr;
      bulk_g2s(base + size_t(pl) * PS + size_t(row) * TWp,
               plane_src(pl) + (long long)(Jlo + row) * p.pitch + Ial, rowbytes, &bar[st]);
    }
  };
  issue(0);
  if (nb > 1) issue(1);
  uint32_t ph[2] = {0u, 0u};

  const int slot = lane / N, t = lane - slot * N;
  const bool lane_ok = slot < SL;
  const int e_slot = warp * SL + (lane_ok ? slot : 0);
  const int r_slot = e_slot / SW1, c_slot = e_slot - r_slot * SW1;
  real *sc = scr + size_t(e_slot) * NSC * NN;
  const real xix = lane_ok && c_slot < ncol ? s_xix[c_slot] : real(0);
  const real dxdxi = lane_ok && c_slot < ncol ? s_dxdxi[c_slot] : real(0);
  const real wt = p.w[t < N ? t : 0];
  const real dt = p.dt;

  for (int b = 0; b < nb; ++b) {
    const int st = b & 1;
    const int eb0 = eza + b * R, eb1 = min(eb0 + R, ez1), nre = eb1 - eb0;
    const int Jlo = rw(eb0), nr = rw(eb1 - 1) + N - Jlo;
    const bool from_carry = b > 0 && rw(eb0) == rw(eb0 - 1) + (N - 1);
    if (tid < HR) {
      const int jj = tid;
      int r0 = -1, j0 = 0, r1 = -1, j1 = 0;
      for (int r = 0; r < nre; ++r) {
        const int j = jj - (rw(eb0 + r) - Jlo);
        if (j >= 0 && j < N) {
          if (r0 < 0) {
            r0 = r;
            j0 = j;
          } else {
            r1 = r;
            j1 = j;
          }
        }
      }
      s_r[0][jj] = r0;
      s_j[0][jj] = j0;
      s_r[1][jj] = r1;
      s_j[1][jj] = j1;
      const int J = Jlo + jj;
      int fate = 1;
      if (jj >= nr || J < J0own || J >= J1own) fate = 0;
      else if (eb1 < ez1 && rw(eb1) == J) fate = 2;
      s_stat[jj] = fate;
    }
    // misfit derivatives of this step at the stage nodes
    for (int q = tid; q < NDOF * nr * TWp; q += kStripThreads) sG[q % (nr * TWp) + (q / (nr * TWp)) * PS] = real(0);
    if (!mbar_wait(&bar[st], ph[st])) atomicOr(&s_err, 1);
    ph[st] ^= 1u;
    __syncthreads();
    if (s_err) {
      if (tid == 0) {
        if (p.error) atomicExch(p.error, kErrTimeout);
        mbar_wait(&bar[st], ph[st] ^ 1u);
        if (b + 1 < nb) mbar_wait(&bar[st ^ 1], ph[st ^ 1]);
      }
      __syncthreads();
      return;
    }
    if (sampled)
      for (int q = tid; q < p.nrec * NDOF; q += kStripThreads) {
        const int r = q % p.nrec, c = q / p.nrec;
        const int I = p.rec_I[r], J = p.rec_J[r];
        const int col = I - Ial, jj = J - Jlo;
        if (col < 0 || col >= cw || jj < 0 || jj >= nr) continue;
        const real g = real(p.resid[samp + (size_t)p.nsamp * (r + (size_t)p.nrec * c)]);
        sG[c * PS + jj * TWp + col] += g;
      }
    __syncthreads();

    real *sg = stg + st * stage_sz;
    const real *sDb = sg, *sd = sg + 2 * NDOF * PS;
    real *sVb = sg + NDOF * PS;  // Vb^{n+1}, replaced by Vb^n
    const real *sM = sg + 3 * NDOF * PS, *sRm = sg + size_t(3 * NDOF + p.nmat) * PS;

    // ---- Vb^n and lambda^n at every stage node ----
    for (int q = tid; q < nr * cw; q += kStripThreads) {
      const int jj = q / cw, col = q - jj * cw;
      const int I = Ial + col, J = Jlo + jj;
      const int si = jj * TWp + col;
      const bool edge = (J == 0 || J == p.LZ - 1 || I == 0 || I == p.LX - 1) && I < p.LX;
      const int sp = edge ? perimeter_slot(I, J, p.LX, p.LZ) : -1;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        const real vb = sVb[c * PS + si];
        real rm = sRm[si], cv = real(0);
        if (sp >= 0) {
          const int so = c * nslot + sp;
          rm = p.per_rm[so];
          cv = p.per_Ca[so] + p.per_Cb[so];
        }
        const real gv = p.field == 'D' ? real(0) : sG[c * PS + si];
        const real vn = (gv + dt * sDb[c * PS + si]) + (vb - (dt * rm) * (cv * vb));
        sVb[c * PS + si] = vn;
        sL[c * PS + si] = (dt * rm) * vn;
      }
    }
    __syncthreads();

    // ---- element phase: F(lambda) and the moduli terms lambda . dF/dtheta d ----
    {
      const int r = r_slot, c = c_slot;
      const bool act = lane_ok && r < nre && c < ncol;
      const int ez = eb0 + r;
      const int eb = act ? (rw(ez) - Jlo) * TWp + xo + c * (N - 1) : 0;
      const real etaz = act ? s_etaz[ez - eza] : real(0);
      const real det = dxdxi * (act ? s_dzdeta[ez - eza] : real(0));
      const real wdt = det * wt;
      auto at = [&](const real *pl, int i, int j) -> real { return pl[eb + j * TWp + i]; };
      if constexpr (NDOF == 1) {
        // planes: 0 dlambda/dxi then F, 1 dlambda/deta, 2 dd/dxi then the
        // column part, 3 dd/deta then d/dmu
        real *SX = sc, *SE = sc + NN, *DX = sc + 2 * NN, *DE = sc + 3 * NN;
        real cl[N], rl[N];
        if (act) {
          real lx[N], lr[N], ux[N], ur[N];
#pragma unroll
          for (int q = 0; q < N; ++q) {
            lx[q] = at(sL, q, t);
            lr[q] = at(sL, t, q);
            ux[q] = at(sd, q, t);
            ur[q] = at(sd, t, q);
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[0 + N * i] * lx[0], b2 = p.H[0 + N * i] * ux[0];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + p.H[q + N * i] * lx[q];
              b2 = b2 + p.H[q + N * i] * ux[q];
            }
            SX[i + N * t] = a;   // dlambda/dxi at (i,t)
            DX[i + N * t] = b2;  // dd/dxi at (i,t)
          }
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = lr[0] * p.H[0 + N * j], b2 = ur[0] * p.H[0 + N * j];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + lr[q] * p.H[q + N * j];
              b2 = b2 + ur[q] * p.H[q + N * j];
            }
            SE[t + N * j] = a;   // dlambda/deta at (t,j)
            DE[t + N * j] = b2;  // dd/deta at (t,j)
          }
        }
        __syncwarp();
        if (act) {
          const real cxx = -(wdt * xix) * xix, czz = -(wdt * etaz) * etaz;
#pragma unroll
          for (int q = 0; q < N; ++q) {
            const int kc = q + N * t, kr = t + N * q;
            const real mu_c = at(sM, q, t), mu_r = at(sM, t, q);
            cl[q] = (cxx * p.w[q]) * (mu_c * SX[kc]);
            rl[q] = (czz * p.w[q]) * (mu_r * SE[kr]);
            // d/dmu at point (q,t): -W (xix^2 dxi l dxi d + etaz^2 deta l deta d)
            DE[kc] = (cxx * p.w[q]) * (SX[kc] * DX[kc]) + (czz * p.w[q]) * (SE[kc] * DE[kc]);
          }
        }
        __syncwarp();
        if (act) {
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[i + N * 0] * cl[0];
#pragma unroll
            for (int q = 1; q < N; ++q) a = a + p.H[i + N * q] * cl[q];
            DX[i + N * t] = a;  // column part at (i,t)
          }
        }
        __syncwarp();
        if (act) {
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = rl[0] * p.H[j + N * 0];
#pragma unroll
            for (int q = 1; q < N; ++q) a = a + rl[q] * p.H[j + N * q];
            SX[t + N * j] = DX[t + N * j] + a;  // F(lambda) at (t,j)
          }
        }
        __syncwarp();
      } else {
        // planes: 0-1 dlambda/dxi then F, 2-3 dlambda/deta, then dd/deta,
        // then the moduli terms d/dla, d/dmu
        real *SXX = sc, *SXZ = sc + NN, *SEX = sc + 2 * NN, *SEZ = sc + 3 * NN;
        real dxx[N], dxz[N], dex[N], dez[N];
        if (act) {
          real lx[N], lz[N];
#pragma unroll
          for (int q = 0; q < N; ++q) {
            lx[q] = at(sL, q, t);
            lz[q] = at(sL + PS, q, t);
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[0 + N * i] * lx[0], b2 = p.H[0 + N * i] * lz[0];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + p.H[q + N * i] * lx[q];
              b2 = b2 + p.H[q + N * i] * lz[q];
            }
            SXX[i + N * t] = a;
            SXZ[i + N * t] = b2;
          }
#pragma unroll
          for (int q = 0; q < N; ++q) {
            lx[q] = at(sL, t, q);
            lz[q] = at(sL + PS, t, q);
          }
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = lx[0] * p.H[0 + N * j], b2 = lz[0] * p.H[0 + N * j];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + lx[q] * p.H[q + N * j];
              b2 = b2 + lz[q] * p.H[q + N * j];
            }
            SEX[t + N * j] = a;
            SEZ[t + N * j] = b2;
          }
          real ux[N], uz[N];
#pragma unroll
          for (int q = 0; q < N; ++q) {
            ux[q] = at(sd, q, t);
            uz[q] = at(sd + PS, q, t);
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[0 + N * i] * ux[0], b2 = p.H[0 + N * i] * uz[0];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + p.H[q + N * i] * ux[q];
              b2 = b2 + p.H[q + N * i] * uz[q];
            }
            dxx[i] = a;  // dd_x/dxi at (i,t)
            dxz[i] = b2;
          }
#pragma unroll
          for (int q = 0; q < N; ++q) {
            ux[q] = at(sd, t, q);
            uz[q] = at(sd + PS, t, q);
          }
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = ux[0] * p.H[0 + N * j], b2 = uz[0] * p.H[0 + N * j];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + ux[q] * p.H[q + N * j];
              b2 = b2 + uz[q] * p.H[q + N * j];
            }
            dex[j] = a;  // dd_x/deta at (t,j)
            dez[j] = b2;
          }
        }
        __syncwarp();
        real cx[N], cz[N], rx[N], rz[N], lzx[N], lzz[N];
        const real sxz = p.kd2 ? etaz : xix;
        if (act) {
          const real wcx = -(wdt * xix), wrz = -(wdt * etaz);
#pragma unroll
          for (int q = 0; q < N; ++q) {
            // column part at (q,t)
            const int k = q + N * t;
            const real la = at(sM, q, t), mu = at(sM + PS, q, t);
            const real Kx = la + real(2) * mu;
            const real lxx = xix * SXX[k], lxz = xix * SXZ[k];
            lzx[q] = etaz * SEX[k];
            lzz[q] = etaz * SEZ[k];
            const real wq = wcx * p.w[q];
            cx[q] = wq * (Kx * lxx + la * lzz[q]);
            cz[q] = wq * (mu * (lzx[q] + lxz));
          }
#pragma unroll
          for (int q = 0; q < N; ++q) {
            // row part at (t,q)
            const int k = t + N * q;
            const real la = at(sM, t, q), mu = at(sM + PS, t, q);
            const real Kz = la + real(2) * mu;
            const real wq = wrz * p.w[q];
            rx[q] = wq * (mu * (etaz * SEX[k] + sxz * SXZ[k]));
            rz[q] = wq * (la * (xix * SXX[k]) + Kz * (etaz * SEZ[k]));
          }
        }
        __syncwarp();
        if (act) {
#pragma unroll
          for (int q = 0; q < N; ++q) {
            SEX[t + N * q] = dex[q];  // dd_x/deta at (t,q)
            SEZ[t + N * q] = dez[q];
          }
        }
        __syncwarp();
        if (act) {
#pragma unroll
          for (int q = 0; q < N; ++q) {
            // moduli terms at (q,t)
            const int k = q + N * t;
            const real lxx = xix * SXX[k], lxz = xix * SXZ[k];
            const real uxx = xix * dxx[q], uxz = xix * dxz[q], uzx = etaz * SEX[k], uzz = etaz * SEZ[k];
            const real W = wdt * p.w[q];
            SEX[k] = -W * ((lxx + lzz[q]) * (uxx + uzz));
            SEZ[k] = -W * (real(2) * (lxx * uxx) + real(2) * (lzz[q] * uzz) + lxz * (uzx + uxz) +
                           lzx[q] * (uzx + sxz * dxz[q]));
          }
        }
        __syncwarp();
        if (act) {
#pragma unroll
          for (int i = 0; i < N; ++i) {
            real a = p.H[i + N * 0] * cx[0], b2 = p.H[i + N * 0] * cz[0];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + p.H[i + N * q] * cx[q];
              b2 = b2 + p.H[i + N * q] * cz[q];
            }
            SXX[i + N * t] = a;
            SXZ[i + N * t] = b2;
          }
        }
        __syncwarp();
        if (act) {
#pragma unroll
          for (int j = 0; j < N; ++j) {
            real a = rx[0] * p.H[j + N * 0], b2 = rz[0] * p.H[j + N * 0];
#pragma unroll
            for (int q = 1; q < N; ++q) {
              a = a + rx[q] * p.H[j + N * q];
              b2 = b2 + rz[q] * p.H[j + N * q];
            }
            SXX[t + N * j] = SXX[t + N * j] + a;  // F(lambda) at (t,j)
            SXZ[t + N * j] = SXZ[t + N * j] + b2;
          }
        }
        __syncwarp();
      }
    }
    __syncthreads();

    // ---- assembly and the per-node updates ----
    // quantities per node: F(lambda) (NDOF), d/dla, d/dmu (P-SV) or d/dmu (SH)
    constexpr int NQ = NDOF == 2 ? 4 : 2;
    auto qplane = [&](int k) -> int {  // scratch plane of quantity k
      if (NDOF == 2) return k;           // F_x, F_z, d/dla, d/dmu
      return k == 0 ? 0 : 3;             // F, d/dmu
    };
    real *cin = carry + (st ^ 1) * NC * TWp, *cout = carry + st * NC * TWp;
    // A thread's nodes: the global reads of all of them (forward
    // acceleration, gradient partial sums) are issued first, so that their
    // latencies overlap, then the nodes are assembled and updated in turn.
    constexpr int OWS = SW * (N - 1) + 1;  // >= OWc
    constexpr int NQI = (HR * OWS + kStripThreads - 1) / kStripThreads;
    constexpr int NG = NDOF + 1 + (NDOF == 2 ? 2 : 1);  // a (NDOF), g_M, g_la, g_mu
    real pre[NQI][NG];
#pragma unroll
    for (int k = 0; k < NQI; ++k) {
      const int q = tid + k * kStripThreads;
      const int jj = q / OWc, io = q - jj * OWc;
      const bool upd = q < nr * OWc && s_stat[jj < HR ? jj : 0] == 1;
      const long long g = (long long)(Jlo + jj) * p.pitch + I0 + io;
#pragma unroll
      for (int c = 0; c < NDOF; ++c) pre[k][c] = upd ? p.a[c * p.plane + g] : real(0);
      pre[k][NDOF] = upd ? p.g_M[g] : real(0);
      if (NDOF == 2) {
        pre[k][NDOF + 1] = upd ? p.g_la[g] : real(0);
        pre[k][NDOF + 2] = upd ? p.g_mu[g] : real(0);
      } else {
        pre[k][NDOF + 1] = upd ? p.g_mu[g] : real(0);
      }
    }
#pragma unroll
    for (int k = 0; k < NQI; ++k) {
      const int q = tid + k * kStripThreads;
      if (q >= nr * OWc) break;
      const int jj = q / OWc, io = q - jj * OWc;
      const int fate = s_stat[jj];
      if (fate == 0) continue;
      const int ii = ii0 + io;
      real f[NQ];
#pragma unroll
      for (int k2 = 0; k2 < NQ; ++k2) f[k2] = (jj == 0 && from_carry) ? cin[k2 * TWp + io] : real(0);
      const int ce = ii / (N - 1), il0 = ii - ce * (N - 1);
#pragma unroll
      for (int kk = 0; kk < 2; ++kk) {
        const int rr = s_r[kk][jj], jl = s_j[kk][jj];
        if (rr < 0) continue;
        if (il0 == 0 && ce > 0) {
          const real *sl = scr + size_t(rr * SW1 + ce - 1) * NSC * NN + (N - 1) + N * jl;
#pragma unroll
          for (int k2 = 0; k2 < NQ; ++k2) f[k2] = f[k2] + sl[qplane(k2) * NN];
        }
        if (ce < ncol) {
          const real *sl = scr + size_t(rr * SW1 + ce) * NSC * NN + il0 + N * jl;
#pragma unroll
          for (int k2 = 0; k2 < NQ; ++k2) f[k2] = f[k2] + sl[qplane(k2) * NN];
        }
      }
      if (fate == 2) {
#pragma unroll
        for (int k2 = 0; k2 < NQ; ++k2) cout[k2 * TWp + io] = f[k2];
        continue;
      }
      const int I = I0 + io, J = Jlo + jj;
      const int si = jj * TWp + xo + ii;
      const long long g = (long long)J * p.pitch + I;
      const bool edge = (J == 0 || J == p.LZ - 1 || I == 0 || I == p.LX - 1);
      const int sp = edge ? perimeter_slot(I, J, p.LX, p.LZ) : -1;
      real gm = real(0);
#pragma unroll
      for (int c = 0; c < NDOF; ++c) {
        const real lam = sL[c * PS + si];
        const real an = pre[k][c];
        const real gd = p.field == 'D' ? sG[c * PS + si] : real(0);
        p.Vbn[c * p.plane + g] = sVb[c * PS + si];
        p.Dbn[c * p.plane + g] = (gd + sDb[c * PS + si]) + f[c];
        gm = gm - lam * an;
        if (sp >= 0) {
          const real vp = p.vprev[c * p.plane + g];
          p.g_C[c * nslot + sp] += -lam * (vp + (real(0.5) * dt) * an);
        }
      }
      p.g_M[g] = pre[k][NDOF] + gm;
      if (NDOF == 2) {
        p.g_la[g] = pre[k][NDOF + 1] + f[2];
        p.g_mu[g] = pre[k][NDOF + 2] + f[3];
      } else {
        p.g_mu[g] = pre[k][NDOF + 1] + f[1];
      }
    }
    __syncthreads();
    if (b + 2 < nb) issue(b + 2);
  }
}

}  // namespace sem2d

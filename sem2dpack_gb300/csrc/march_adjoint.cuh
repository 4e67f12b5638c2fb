// march_adjoint.cuh -- one reverse step of the discrete adjoint (the
// recursion of adjoint_kernel.cuh) with one element per thread, for FP32
// fields, NGLL = 5, isotropic material continuous at nodes.
//
// The adjoint state of adjoint_kernel.cuh (Db, Vb) is carried here as
//   lambda^n = dt M^-1 Vb^n,   w^n = dt M^-1 Db^n,
// with which the recursion
//   Vb^n = g_v^n + dt Db^{n+1} + (I - dt M^-1 C) Vb^{n+1},
//   Db^n = g_d^n + Db^{n+1} + F lambda^n
// becomes (M and C are diagonal)
//   w^n          = w^{n+1} + dt M^-1 (F lambda^n + g_d^n)
//   lambda^{n-1} = (I - dt M^-1 C) lambda^n + dt w^n + dt M^-1 g_v^{n-1}:
// the leapfrog step of the forward march kernel with (lambda, w) in place
// of (d, v) and the dashpots acting on the lambda update instead of the
// force; the misfit derivatives are node-local additions at the receivers
// (adjoint_inject_one, by an extra CTA of the second launch).  Reverse step n reads (lambda^n, w^{n+1}) and
// writes (lambda^{n-1}, w^n); it starts from lambda^{nt} = dt M^-1 g_v^{nt},
// w^{nt+1} = 0.
//
// Two launches per reverse step, both walking the forward's march units:
//   march_adjoint_kernel: march_unit<..., ADJ> (march_kernel.cuh): the
//     step above, plus the mass term g_M += -lambda^n . a^n at every owned
//     node and the dashpot term g_C += -lambda^n . (v^{n-1} + dt/2 a^n) on
//     the perimeter;
//   adj_march_moduli: the gradients of lambda^n and d^n at every element
//     point (row by row) and the moduli products
//       d/dla = -W div(lambda) div(d)
//       d/dmu = -W [2 lxx uxx + 2 lzz uzz + lxz (uzx + uxz) + lzx (uzx + s dxz)]
//     (SH: (cxx w_i) dxi l dxi d + (czz w_i) deta l deta d), assembled like
//     forces and added to the per-node sums g_la, g_mu.
#pragma once

#include "march_kernel.cuh"
#include "sem2d_common.cuh"

namespace sem2d {

struct MarchAdjParams {
  int LX, LZ, pitch;
  long long plane;
  int nx, nz;
  const int *row0;
  float H[25], w[5];
  const float *xix, *etaz, *dxdxi, *dzdeta;
  const float *lam;  // lambda^n
  const float *d;    // forward d^n
  float *g_la, *g_mu;
  int kd2;
  // the misfit derivatives of the step (march_adjoint_inject), added by the
  // launch's last CTA when inj >= 0 (0: velocity, 1: displacement)
  int inj, ndof, nrec, nsamp, smp;
  float *lam_next, *w_next;  // lambda^{n-1}, w^n
  const float *rmass, *per_rm;
  const int *rec_I, *rec_J;
  const double *resid;
  float dt;
};

// one reverse step of lambda, w and the mass and dashpot sums
template <int NDOF>
__global__ void __launch_bounds__(32 * kMarchWarps, NDOF == 1 ? 4 : 3)
    march_adjoint_kernel(const __grid_constant__ BulkParams<float, 5> p, const __grid_constant__ MarchAdj x, int it,
                         const MarchUnit *units, int nunits) {
  const int warp = threadIdx.x >> 5;
  const int uid = blockIdx.x * (blockDim.x >> 5) + warp;
  extern __shared__ float4 march_stage[];
  if (uid < nunits)
    march_unit<NDOF, kMatNode, false, true>(p, p.H, p.w, units[uid], it,
                                            march_stage + warp * march_stage_f4(NDOF, false, true), &x);
}

// The misfit derivatives g of sample smp at the receivers' nodes, thread k
// for receiver k % nrec and dof k / nrec (several receivers at one node add
// up), after a reverse step's main launch:
//   velocity (disp = 0): lambda += dt M^-1 g  (g_v^{n-1} into lambda^{n-1};
//     at the start, g_v^{nt} into lambda^{nt});
//   displacement (disp = 1): w += dt M^-1 g and lambda += dt (dt M^-1 g)
//     (g_d^n into w^n, and through it into lambda^{n-1} = ... + dt w^n).
__device__ __forceinline__ void adjoint_inject_one(int k, float *lam, float *wv, long long plane, int pitch, int LX,
                                                   int LZ, const float *rmass, const float *per_rm, int nrec,
                                                   int nsamp, int smp, int disp, const int *rec_I, const int *rec_J,
                                                   const double *resid, float dt) {
  const int r = k % nrec, c = k / nrec;
  const int I = rec_I[r], J = rec_J[r];
  float rm = rmass[(long long)J * pitch + I];
  if (J == 0 || J == LZ - 1 || I == 0 || I == LX - 1)
    rm = per_rm[c * perimeter_slots(LX, LZ) + perimeter_slot(I, J, LX, LZ)];
  const float g = float(resid[smp + (size_t)nsamp * (r + (size_t)nrec * c)]);
  const long long o = c * plane + (long long)J * pitch + I;
  const float q = (dt * rm) * g;
  if (disp) {
    atomicAdd(wv + o, q);
    atomicAdd(lam + o, dt * q);
  } else {
    atomicAdd(lam + o, q);
  }
}

__global__ void march_adjoint_inject(float *lam, float *wv, long long plane, int pitch, int LX, int LZ,
                                     const float *rmass, const float *per_rm, int ndof, int nrec, int nsamp, int smp,
                                     int disp, const int *rec_I, const int *rec_J, const double *resid, float dt) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nrec * ndof)
    adjoint_inject_one(k, lam, wv, plane, pitch, LX, LZ, rmass, per_rm, nrec, nsamp, smp, disp, rec_I, rec_J, resid,
                       dt);
}

// ---------------------------------------------------------------------
// the moduli products lambda^n . dF/dtheta d^n
// the gradient sums' rows of an element row, staged by cp.async when the
// row starts (per warp: node rows j = 0..4, NQ planes, 16 bytes per lane)
__host__ __device__ constexpr int adj_moduli_stage_f4(int ndof) { return 5 * (ndof == 2 ? 2 : 1) * 32; }

template <int NDOF>
__device__ __forceinline__ void adj_moduli_unit(const MarchAdjParams &p, const MarchUnit &u, float4 *stage) {
  constexpr int N = 5;
  constexpr int NQ = NDOF == 2 ? 2 : 1;  // d/dla, d/dmu (P-SV) or d/dmu (SH)
  const int lane = threadIdx.x & 31;
  const int ex = kMarchCols * u.strip - 1 + lane;
  const bool act = ex >= 0 && ex < p.nx;
  const bool ld = ex >= 0 && ex <= p.nx;
  const bool own = act && lane > 0;
  const bool last_col = act && ex == p.nx - 1;
  const int I0 = 4 * (ex < 0 ? 0 : ex);
  const long long pl = p.plane;
  const float xix = act ? p.xix[ex] : 0.f, dxdxi = act ? p.dxdxi[ex] : 0.f;
  const float *H = p.H, *w = p.w;

  int zs = u.z0;
  if (u.z0 > 0 && p.row0[u.z0] == p.row0[u.z0 - 1] + (N - 1)) zs = u.z0 - 1;
  float carry[NQ][N];
#pragma unroll
  for (int c = 0; c < NQ; ++c)
#pragma unroll
    for (int i = 0; i < N; ++i) carry[c][i] = 0.f;
  bool have_carry = false;

  // the 5x5 values of a plane at the lane's element (element row at J0)
  auto rows = [&](const float *src, int J0, float (&V)[NDOF][N][N]) {
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      float4 q[N];
      float v5[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const float *b = src + c * pl + (long long)(J0 + j) * p.pitch + I0;
        q[j] = ld ? ldg4(b) : make_float4(0.f, 0.f, 0.f, 0.f);
        v5[j] = (lane == 31 && act) ? __ldg(b + 4) : 0.f;
      }
#pragma unroll
      for (int j = 0; j < N; ++j) {
        V[c][j][0] = q[j].x;
        V[c][j][1] = q[j].y;
        V[c][j][2] = q[j].z;
        V[c][j][3] = q[j].w;
        const float nx4 = __shfl_down_sync(0xffffffffu, q[j].x, 1);
        V[c][j][4] = lane < 31 ? nx4 : v5[j];
      }
    }
  };

  for (int ez = zs; ez < u.z1; ++ez) {
    const bool halo = ez < u.z0;
    const int J0 = p.row0[ez];
    const float etaz = act ? p.etaz[ez] : 0.f;
    const float det = dxdxi * (act ? p.dzdeta[ez] : 0.f);
    const float sxz = p.kd2 ? etaz : xix;
    const bool top_last = ez == p.nz - 1;
    if (!halo && own) {
      const int nrow = top_last ? N : N - 1;
#pragma unroll
      for (int j = 0; j < N; ++j)
        if (j < nrow) {
          const long long g = (long long)(J0 + j) * p.pitch + I0;
#pragma unroll
          for (int c = 0; c < NQ; ++c)
            cp_async16(stage + (j * NQ + c) * 32 + lane, ((NDOF == 2 && c == 0) ? p.g_la : p.g_mu) + g);
        }
      cp_async_commit();
    }
    float Lm[NDOF][N][N], Dm[NDOF][N][N];
    rows(p.lam, J0, Lm);
    rows(p.d, J0, Dm);
    const bool top_shared = !top_last && p.row0[ez + 1] == J0 + N - 1;
    const bool bottom_carry = have_carry;
#pragma unroll
    for (int j = 0; j < N; ++j) {
      // products at the points (i, j) of this row
      float P[NQ][N];
      const float wdt = det * w[j];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        float gl[NDOF][2], gd[NDOF][2];  // [c][0] d/dxi, [c][1] d/deta
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          float a = H[0 + N * i] * Lm[c][j][0], b = H[0 + N * i] * Dm[c][j][0];
#pragma unroll
          for (int q = 1; q < N; ++q) {
            a = a + H[q + N * i] * Lm[c][j][q];
            b = b + H[q + N * i] * Dm[c][j][q];
          }
          // d/deta at (i,j): sum_q u(i,q) H[q + N j], u(i,q) = row q, column i
          float e = Lm[c][0][i] * H[0 + N * j], f = Dm[c][0][i] * H[0 + N * j];
#pragma unroll
          for (int q = 1; q < N; ++q) {
            e = e + Lm[c][q][i] * H[q + N * j];
            f = f + Dm[c][q][i] * H[q + N * j];
          }
          gl[c][0] = a;
          gd[c][0] = b;
          gl[c][1] = e;
          gd[c][1] = f;
        }
        if (NDOF == 1) {
          const float cxx = -(wdt * xix) * xix, czz = -(wdt * etaz) * etaz;
          P[0][i] = (cxx * w[i]) * (gl[0][0] * gd[0][0]) + (czz * w[i]) * (gl[0][1] * gd[0][1]);
        } else {
          const float lxx = xix * gl[0][0], lxz = xix * gl[1][0];
          const float lzx = etaz * gl[0][1], lzz = etaz * gl[1][1];
          const float uxx = xix * gd[0][0], uxz = xix * gd[1][0], uzx = etaz * gd[0][1], uzz = etaz * gd[1][1];
          const float W = wdt * w[i];
          P[0][i] = -W * ((lxx + lzz) * (uxx + uzz));
          P[NQ - 1][i] = -W * (2.f * (lxx * uxx) + 2.f * (lzz * uzz) + lxz * (uzx + uxz) +
                               lzx * (uzx + sxz * gd[1][0]));
        }
      }
      // assemble: the left element's column 4, the carried bottom row
      float Lq[NQ];
#pragma unroll
      for (int c = 0; c < NQ; ++c) Lq[c] = __shfl_up_sync(0xffffffffu, P[c][N - 1], 1);
      const int J = J0 + j;
      if (j == N - 1 && !top_last) {
        if (top_shared) {
#pragma unroll
          for (int c = 0; c < NQ; ++c)
#pragma unroll
            for (int i = 0; i < N; ++i) carry[c][i] = (i == 0 ? Lq[c] : 0.f) + P[c][i];
        }
        continue;
      }
      if (halo || !own) continue;
      if (j == 0) cp_async_wait_all();
      const long long g = (long long)J * p.pitch + I0;
      float sum[NQ][N];
#pragma unroll
      for (int c = 0; c < NQ; ++c)
#pragma unroll
        for (int i = 0; i < N; ++i) {
          float f = (j == 0 && bottom_carry) ? carry[c][i] : 0.f;
          if (i == 0) f = f + Lq[c];
          sum[c][i] = f + P[c][i];
        }
#pragma unroll
      for (int c = 0; c < NQ; ++c) {
        float *G = (NDOF == 2 && c == 0) ? p.g_la : p.g_mu;
        float4 q = stage[(j * NQ + c) * 32 + lane];
        q.x = q.x + sum[c][0];
        q.y = q.y + sum[c][1];
        q.z = q.z + sum[c][2];
        q.w = q.w + sum[c][3];
        *reinterpret_cast<float4 *>(G + g) = q;
        if (last_col) G[g + 4] = G[g + 4] + sum[c][4];
      }
    }
    have_carry = top_shared;
  }
}

template <int NDOF>
__global__ void __launch_bounds__(32 * kMarchWarps, NDOF == 1 ? 4 : 3)
    adj_march_moduli(const __grid_constant__ MarchAdjParams p, const MarchUnit *units, int nunits) {
  if (p.inj >= 0 && blockIdx.x == gridDim.x - 1) {
    // the extra CTA: the misfit derivatives (lambda^{n-1} and w^n, which
    // this launch does not read)
    for (int k = threadIdx.x; k < p.nrec * p.ndof; k += blockDim.x)
      adjoint_inject_one(k, p.lam_next, p.w_next, p.plane, p.pitch, p.LX, p.LZ, p.rmass, p.per_rm, p.nrec, p.nsamp,
                         p.smp, p.inj, p.rec_I, p.rec_J, p.resid, p.dt);
    return;
  }
  const int warp = threadIdx.x >> 5;
  const int uid = blockIdx.x * (blockDim.x >> 5) + warp;
  extern __shared__ float4 moduli_stage[];
  if (uid < nunits) adj_moduli_unit<NDOF>(p, units[uid], moduli_stage + warp * adj_moduli_stage_f4(NDOF));
}

}  // namespace sem2d

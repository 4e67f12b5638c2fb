// march_adjoint.cuh -- one reverse step of the discrete adjoint (the same
// step as adjoint_kernel.cuh) with one element per thread, for FP32 fields,
// NGLL = 5, isotropic material continuous at nodes.
//
// Two launches per reverse step n, both walking the march units (a warp per
// strip of 31 element columns and chunk of element rows, a halo row below
// the chunk, lane 0 the column left of the strip):
//   adj_march_forces: at every node of an element row the node-local update
//       Vb^n = g_v + dt Db + (I - dt M^-1 C) Vb,  lambda = dt M^-1 Vb^n
//     (recomputed by every element that touches the node), then the element
//     forces F(lambda) exactly as the forward march kernel assembles them,
//     and at the owned nodes Db^n = g_d + Db + F(lambda), Vb^n, the mass term
//     g_M += -lambda . a^n and the dashpot term
//     g_C += -lambda . (v^{n-1} + dt/2 a^n) on the perimeter;
//   adj_march_moduli: lambda again from Vb^n (bitwise the same value), the
//     gradients of lambda and d^n at every element point (on the fly, row by
//     row), the moduli products
//       d/dla = -W div(lambda) div(d)
//       d/dmu = -W [2 lxx uxx + 2 lzz uzz + lxz (uzx + uxz) + lzx (uzx + s dxz)]
//     (SH: (cxx w_i) dxi l dxi d + (czz w_i) deta l deta d), assembled like
//     forces and added to the per-node sums g_la, g_mu.
// Receivers of the misfit derivative are found through a per-lattice-row
// index (rec_row: CSR of receiver numbers by row).
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
  const float *mat[2];  // node planes: (lambda, mu) for P-SV, (mu) for SH
  const float *rmass, *per_rm, *per_Ca, *per_Cb;
  const float *Db, *Vb;  // adjoint state of step n+1
  float *Dbn, *Vbn;      // adjoint state of step n (Vbn read by the moduli pass)
  const float *d, *vprev, *a;  // forward d^n, v^{n-1}, a^n
  float *g_la, *g_mu, *g_M, *g_C;
  int nrec, nsamp, isamp;
  char field;  // 'V' or 'D'
  const int *rec_I;
  const int *rec_row;  // [LZ+1] into rec_ids_row
  const int *rec_ids_row;
  const double *resid;  // [s + nsamp*(r + nrec*c)]
  float dt;
  int kd2;
  int it;  // the forward step being reversed
};

// Misfit derivatives of this step at the five node columns I0..I0+4 of
// every lane for lattice row J: the warp reads the row's receivers
// together (receiver k by lane k mod 32) into its shared table, indexed by
// (lane, column); has[i]: a receiver at the lane's column i.  Called by all
// lanes of the warp (the row is the same for the warp).
struct AdjRowTable {
  float g[2][32][5];
  int has[32][5];
};

__device__ __forceinline__ void adj_row_resid(const MarchAdjParams &p, int J, int I0, int lane, int strip, int samp,
                                              int ndof, AdjRowTable &t, float (&g)[2][5], bool (&has)[5]) {
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    t.has[lane][i] = 0;
    t.g[0][lane][i] = 0.f;
    t.g[1][lane][i] = 0.f;
  }
  __syncwarp();
  const int ex0 = kMarchCols * strip - 1;  // element column of lane 0
  for (int k = p.rec_row[J] + lane; k < p.rec_row[J + 1]; k += 32) {
    const int r = p.rec_ids_row[k];
    const int I = p.rec_I[r];
    // lane owning column I (column I % 4 of element I / 4) and, for the
    // first column of an element, the lane to its left (its fifth column)
    const int e = min(I / 4, p.nx - 1), col = I - 4 * e;
    const int la = e - ex0;
    for (int c = 0; c < ndof; ++c) {
      const float v = float(p.resid[samp + (size_t)p.nsamp * (r + (size_t)p.nrec * c)]);
      if (la >= 0 && la < 32) {
        atomicAdd(&t.g[c][la][col], v);
        if (c == 0) atomicOr(&t.has[la][col], 1);
      }
      if (col == 0 && la - 1 >= 0 && la - 1 < 32) {
        atomicAdd(&t.g[c][la - 1][4], v);
        if (c == 0) atomicOr(&t.has[la - 1][4], 1);
      }
    }
  }
  __syncwarp();
#pragma unroll
  for (int i = 0; i < 5; ++i) {
    has[i] = t.has[lane][i] != 0;
    g[0][i] = t.g[0][lane][i];
    g[1][i] = t.g[1][lane][i];
  }
  __syncwarp();
  (void)I0;
}

// Vb^n and lambda at node (I, J) from the step's inputs.  The general form
// (perimeter dashpots and inverse mass, misfit derivative gv) is out of
// line: inlined at every node of an element it made the kernel larger than
// the instruction cache.  `special` (a perimeter node or one with a
// receiver) depends on the node alone, so every element touching a node
// computes the same lambda.
__device__ __noinline__ float2 adj_lambda_general(const MarchAdjParams &p, int I, int J, float db, float vb, float rmi,
                                                  int c, int nslot, float gv) {
  float rm = rmi, cv = 0.f;
  if (J == 0 || J == p.LZ - 1 || I == 0 || I == p.LX - 1) {
    const int so = c * nslot + perimeter_slot(I, J, p.LX, p.LZ);
    rm = p.per_rm[so];
    cv = p.per_Ca[so] + p.per_Cb[so];
  }
  const float vn = (gv + p.dt * db) + (vb - (p.dt * rm) * (cv * vb));
  return make_float2(vn, (p.dt * rm) * vn);
}

struct AdjLambda {
  __device__ __forceinline__ static void at(const MarchAdjParams &p, int I, int J, float db, float vb, float rmi,
                                            int c, int nslot, bool special, float gv, float &vn, float &lam) {
    if (special || J == 0 || J == p.LZ - 1 || I == 0 || I == p.LX - 1) {
      const float2 r = adj_lambda_general(p, I, J, db, vb, rmi, c, nslot, gv);
      vn = r.x;
      lam = r.y;
      return;
    }
    vn = p.dt * db + vb;  // interior node without receiver
    lam = (p.dt * rmi) * vn;
  }
};

// inverse mass of node (I, J) for dof c (perimeter table on the boundary)
__device__ __noinline__ float adj_rm_edge(const MarchAdjParams &p, int I, int J, int c, int nslot) {
  return p.per_rm[c * nslot + perimeter_slot(I, J, p.LX, p.LZ)];
}

// dashpot gradient terms of a perimeter node
template <int NDOF>
__device__ __noinline__ void adj_dashpot_terms(const MarchAdjParams &p, int I, int J, int nslot, float l0, float l1,
                                               float a0, float a1) {
  const int sp = perimeter_slot(I, J, p.LX, p.LZ);
  const float lam[2] = {l0, l1}, an[2] = {a0, a1};
  for (int c = 0; c < NDOF; ++c) {
    const float vp = p.vprev[c * p.plane + (long long)J * p.pitch + I];
    p.g_C[c * nslot + sp] += -lam[c] * (vp + (0.5f * p.dt) * an[c]);
  }
}

// lambda at the 5x5 nodes of the lane's element (element row starting at
// lattice row J0), from Db/Vb (forces pass) or from Vb^n (moduli pass);
// `sampled`: this step is sampled and one of the element row's node rows
// holds receivers (uniform across the warp)
template <int NDOF, bool FROM_VBN>
__device__ __forceinline__ void adj_lambda_rows(const MarchAdjParams &p, int J0, int I0, int lane, bool ld, bool act,
                                                int nslot, bool sampled, int samp, float (&L)[NDOF][5][5],
                                                AdjRowTable *tab, int strip) {
  constexpr int N = 5;
  const bool l31 = lane == 31 && act;  // lane 31 computes its element's fifth column itself
#pragma unroll
  for (int j = 0; j < N; ++j) {
    const int J = J0 + j;
    const long long g = (long long)J * p.pitch + I0;
    // every input of the row is requested before any is used
    const float4 rq = ld ? ldg4(p.rmass + g) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float r5 = l31 ? __ldg(p.rmass + g + 4) : 0.f;
    float4 vq[NDOF], dq[NDOF];
    float v5[NDOF], d5[NDOF];
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      const float *vsrc = (FROM_VBN ? p.Vbn : p.Vb) + c * p.plane + g;
      vq[c] = ld ? ldg4(vsrc) : make_float4(0.f, 0.f, 0.f, 0.f);
      v5[c] = l31 ? __ldg(vsrc + 4) : 0.f;
      if (!FROM_VBN) {
        const float *dsrc = p.Db + c * p.plane + g;
        dq[c] = ld ? ldg4(dsrc) : make_float4(0.f, 0.f, 0.f, 0.f);
        d5[c] = l31 ? __ldg(dsrc + 4) : 0.f;
      } else {
        dq[c] = make_float4(0.f, 0.f, 0.f, 0.f);
        d5[c] = 0.f;
      }
    }
    const float rmv[N] = {rq.x, rq.y, rq.z, rq.w, r5};
    // receivers of this row (velocity misfit: enters lambda)
    float gres[2][5] = {{0.f, 0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f, 0.f}};
    bool has[5] = {false, false, false, false, false};
    if (!FROM_VBN && sampled && p.field != 'D' && p.rec_row[J + 1] > p.rec_row[J])
      adj_row_resid(p, J, I0, lane, strip, samp, NDOF, *tab, gres, has);
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      const float vv[N] = {vq[c].x, vq[c].y, vq[c].z, vq[c].w, v5[c]};
      const float dd[N] = {dq[c].x, dq[c].y, dq[c].z, dq[c].w, d5[c]};
      float lam4[N];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const int I = I0 + i;
        float lam = 0.f;
        const bool here = i < N - 1 ? (ld && I < p.LX) : l31;
        if (here) {
          if (FROM_VBN) {
            float rm = rmv[i];
            if (J == 0 || J == p.LZ - 1 || I == 0 || I == p.LX - 1) rm = adj_rm_edge(p, I, J, c, nslot);
            lam = (p.dt * rm) * vv[i];
          } else {
            float vn;
            AdjLambda::at(p, I, J, dd[i], vv[i], rmv[i], c, nslot, has[i], gres[c][i], vn, lam);
          }
        }
        lam4[i] = lam;
      }
#pragma unroll
      for (int i = 0; i < N - 1; ++i) L[c][j][i] = lam4[i];
      // fifth column: the next lane's first (lane 31: its own)
      const float nx4 = __shfl_down_sync(0xffffffffu, lam4[0], 1);
      L[c][j][4] = lane < 31 ? nx4 : lam4[4];
    }
  }
}

// ---------------------------------------------------------------------
// pass 1: F(lambda), Db^n, Vb^n, mass and dashpot terms
template <int NDOF>
__device__ __forceinline__ void adj_forces_unit(const MarchAdjParams &p, const MarchUnit &u, AdjRowTable *tab) {
  constexpr int N = 5;
  const int lane = threadIdx.x & 31;
  const int ex = kMarchCols * u.strip - 1 + lane;
  const bool act = ex >= 0 && ex < p.nx;
  const bool ld = ex >= 0 && ex <= p.nx;
  const bool own = act && lane > 0;
  const bool last_col = act && ex == p.nx - 1;
  const int I0 = 4 * (ex < 0 ? 0 : ex);
  const long long pl = p.plane;
  const float xix = act ? p.xix[ex] : 0.f, dxdxi = act ? p.dxdxi[ex] : 0.f;
  const int nslot = perimeter_slots(p.LX, p.LZ);
  const bool sampled = p.nrec > 0 && p.it % p.isamp == 0 && p.it / p.isamp < p.nsamp;
  const int samp = p.it / p.isamp;
  const float *H = p.H, *w = p.w;

  int zs = u.z0;
  if (u.z0 > 0 && p.row0[u.z0] == p.row0[u.z0 - 1] + (N - 1)) zs = u.z0 - 1;
  float carry[NDOF][N];
#pragma unroll
  for (int c = 0; c < NDOF; ++c)
#pragma unroll
    for (int i = 0; i < N; ++i) carry[c][i] = 0.f;
  bool have_carry = false;

  for (int ez = zs; ez < u.z1; ++ez) {
    const bool halo = ez < u.z0;
    const int J0 = p.row0[ez];
    const float etaz = act ? p.etaz[ez] : 0.f;
    const float det = dxdxi * (act ? p.dzdeta[ez] : 0.f);
    // receivers in the element row's node rows (the lookups are skipped
    // for the others)
    const bool rec = sampled && p.rec_row[min(J0 + N, p.LZ)] > p.rec_row[J0];
    float A[NDOF][N][N], B[NDOF][N][N];
    adj_lambda_rows<NDOF, false>(p, J0, I0, lane, ld, act, nslot, rec, samp, A, tab, u.strip);
    // F(lambda): the forward march kernel's element operator
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
#pragma unroll
      for (int j = 0; j < N; ++j)
#pragma unroll
        for (int i = 0; i < N; ++i) {
          float a = H[0 + N * i] * A[c][j][0];
#pragma unroll
          for (int q = 1; q < N; ++q) a = a + H[q + N * i] * A[c][j][q];
          B[c][j][i] = a;
        }
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
#pragma unroll
      for (int i = 0; i < N; ++i) {
        float t[N];
#pragma unroll
        for (int j = 0; j < N; ++j) {
          float a = A[c][0][i] * H[0 + N * j];
#pragma unroll
          for (int q = 1; q < N; ++q) a = a + A[c][q][i] * H[q + N * j];
          t[j] = a;
        }
#pragma unroll
        for (int j = 0; j < N; ++j) A[c][j][i] = t[j];
      }
#pragma unroll
    for (int j = 0; j < N; ++j) {
      float m0[N], m1[N];
#pragma unroll
      for (int m = 0; m < NDOF; ++m) {
        const float *b = p.mat[m] + (long long)(J0 + j) * p.pitch + I0;
        const float4 q = ld ? ldg4(b) : make_float4(0.f, 0.f, 0.f, 0.f);
        const float m5 = (lane == 31 && act) ? __ldg(b + 4) : 0.f;
        float *v = m == 0 ? m0 : m1;
        v[0] = q.x;
        v[1] = q.y;
        v[2] = q.z;
        v[3] = q.w;
        const float nx4 = __shfl_down_sync(0xffffffffu, q.x, 1);
        v[4] = lane < 31 ? nx4 : m5;
      }
      const float wdtj = det * w[j];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const float wdti = det * w[i];
        if (NDOF == 1) {
          const float cxx = -(wdtj * xix) * xix, czz = -(wdti * etaz) * etaz;
          B[0][j][i] = (cxx * w[i]) * (m0[i] * B[0][j][i]);
          A[0][j][i] = (czz * w[j]) * (m0[i] * A[0][j][i]);
        } else {
          const float la = m0[i], mu = m1[i];
          const float K = la + 2.f * mu;
          const float gxx = B[0][j][i], gxz = B[1][j][i], gex = A[0][j][i], gez = A[1][j][i];
          const float dxux = xix * gxx, dxuz = xix * gxz, dzux = etaz * gex, dzuz = etaz * gez;
          const float wc = -(wdtj * xix) * w[i];
          const float wr = -(wdti * etaz) * w[j];
          const float sxz = p.kd2 ? etaz : xix;
          B[0][j][i] = wc * (K * dxux + la * dzuz);
          B[1][j][i] = wc * (mu * (dzux + dxuz));
          A[0][j][i] = wr * (mu * (dzux + sxz * gxz));
          A[1][j][i] = wr * (la * dxux + K * dzuz);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        float t[N];
#pragma unroll
        for (int i = 0; i < N; ++i) {
          float a = H[i + N * 0] * B[c][j][0];
#pragma unroll
          for (int q = 1; q < N; ++q) a = a + H[i + N * q] * B[c][j][q];
          t[i] = a;
        }
#pragma unroll
        for (int i = 0; i < N; ++i) B[c][j][i] = t[i];
      }
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
#pragma unroll
      for (int i = 0; i < N; ++i)
#pragma unroll
        for (int j = 0; j < N; ++j) {
          float a = A[c][0][i] * H[j + N * 0];
#pragma unroll
          for (int q = 1; q < N; ++q) a = a + A[c][q][i] * H[j + N * q];
          B[c][j][i] = B[c][j][i] + a;
        }
    float Ls[NDOF][N];
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
#pragma unroll
      for (int j = 0; j < N; ++j) Ls[c][j] = __shfl_up_sync(0xffffffffu, B[c][j][N - 1], 1);
    const int Jt = J0 + N - 1;
    const bool top_last = ez == p.nz - 1;
    const bool top_shared = !top_last && p.row0[ez + 1] == Jt;
    const bool bottom_carry = have_carry;
    if (!halo) {
#pragma unroll
      for (int j = 0; j < N; ++j) {
        if (j == N - 1 && !top_last) break;
        const int J = J0 + j;
        float gres[2][5] = {{0.f, 0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f, 0.f}};
        bool has[5] = {false, false, false, false, false};
        if (rec && p.rec_row[J + 1] > p.rec_row[J]) adj_row_resid(p, J, I0, lane, u.strip, samp, NDOF, *tab, gres, has);
        if (!own) continue;
        const long long g = (long long)J * p.pitch + I0;
        const float4 rq = ldg4(p.rmass + g);
        const float rmv[N] = {rq.x, rq.y, rq.z, rq.w, last_col ? __ldg(p.rmass + g + 4) : 0.f};
        float gm[N] = {0.f, 0.f, 0.f, 0.f, 0.f};
        float lamv[NDOF][N], anv[NDOF][N];
        const bool fv = p.field != 'D';
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          const float4 vq = ldg4(p.Vb + c * pl + g), dq = ldg4(p.Db + c * pl + g), aq = ldg4(p.a + c * pl + g);
          const float vv[N] = {vq.x, vq.y, vq.z, vq.w, last_col ? __ldg(p.Vb + c * pl + g + 4) : 0.f};
          const float dd[N] = {dq.x, dq.y, dq.z, dq.w, last_col ? __ldg(p.Db + c * pl + g + 4) : 0.f};
          const float av[N] = {aq.x, aq.y, aq.z, aq.w, last_col ? __ldg(p.a + c * pl + g + 4) : 0.f};
          float dbn[N], vbn[N];
#pragma unroll
          for (int i = 0; i < N; ++i) {
            const int I = I0 + i;
            float f = (j == 0 && bottom_carry) ? carry[c][i] : 0.f;
            if (i == 0) f = f + Ls[c][j];
            f = f + B[c][j][i];
            float vn = 0.f, lam = 0.f;
            if (i < N - 1 || last_col)
              AdjLambda::at(p, I, J, dd[i], vv[i], rmv[i], c, nslot, fv && has[i], fv ? gres[c][i] : 0.f, vn, lam);
            const float gd = fv ? 0.f : gres[c][i];
            dbn[i] = (gd + dd[i]) + f;
            vbn[i] = vn;
            gm[i] = gm[i] - lam * av[i];
            lamv[c][i] = lam;
            anv[c][i] = av[i];
          }
          *reinterpret_cast<float4 *>(p.Dbn + c * pl + g) = make_float4(dbn[0], dbn[1], dbn[2], dbn[3]);
          *reinterpret_cast<float4 *>(p.Vbn + c * pl + g) = make_float4(vbn[0], vbn[1], vbn[2], vbn[3]);
          if (last_col) {
            p.Dbn[c * pl + g + 4] = dbn[4];
            p.Vbn[c * pl + g + 4] = vbn[4];
          }
        }
        {
          float4 q = *reinterpret_cast<const float4 *>(p.g_M + g);
          q.x = q.x + gm[0];
          q.y = q.y + gm[1];
          q.z = q.z + gm[2];
          q.w = q.w + gm[3];
          *reinterpret_cast<float4 *>(p.g_M + g) = q;
          if (last_col) p.g_M[g + 4] = p.g_M[g + 4] + gm[4];
        }
        // dashpot terms on the perimeter
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int I = I0 + i;
          if (i == N - 1 && !last_col) continue;
          if (J == 0 || J == p.LZ - 1 || I == 0 || I == p.LX - 1)
            adj_dashpot_terms<NDOF>(p, I, J, nslot, lamv[0][i], NDOF == 2 ? lamv[NDOF - 1][i] : 0.f, anv[0][i],
                                    NDOF == 2 ? anv[NDOF - 1][i] : 0.f);
        }
      }
    }
    if (top_shared) {
#pragma unroll
      for (int c = 0; c < NDOF; ++c)
#pragma unroll
        for (int i = 0; i < N; ++i) carry[c][i] = (i == 0 ? Ls[c][N - 1] : 0.f) + B[c][N - 1][i];
    }
    have_carry = top_shared;
  }
}

// ---------------------------------------------------------------------
// pass 2: the moduli products lambda . dF/dtheta d^n
template <int NDOF>
__device__ __forceinline__ void adj_moduli_unit(const MarchAdjParams &p, const MarchUnit &u) {
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
  const int nslot = perimeter_slots(p.LX, p.LZ);
  const float *H = p.H, *w = p.w;

  int zs = u.z0;
  if (u.z0 > 0 && p.row0[u.z0] == p.row0[u.z0 - 1] + (N - 1)) zs = u.z0 - 1;
  float carry[NQ][N];
#pragma unroll
  for (int c = 0; c < NQ; ++c)
#pragma unroll
    for (int i = 0; i < N; ++i) carry[c][i] = 0.f;
  bool have_carry = false;

  for (int ez = zs; ez < u.z1; ++ez) {
    const bool halo = ez < u.z0;
    const int J0 = p.row0[ez];
    const float etaz = act ? p.etaz[ez] : 0.f;
    const float det = dxdxi * (act ? p.dzdeta[ez] : 0.f);
    const float sxz = p.kd2 ? etaz : xix;
    float Lm[NDOF][N][N], Dm[NDOF][N][N];
    adj_lambda_rows<NDOF, true>(p, J0, I0, lane, ld, act, nslot, false, 0, Lm, nullptr, u.strip);
#pragma unroll
    for (int c = 0; c < NDOF; ++c) {
      float4 q[N];
      float d5[N];
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const float *b = p.d + c * pl + (long long)(J0 + j) * p.pitch + I0;
        q[j] = ld ? ldg4(b) : make_float4(0.f, 0.f, 0.f, 0.f);
        d5[j] = (lane == 31 && act) ? __ldg(b + 4) : 0.f;
      }
#pragma unroll
      for (int j = 0; j < N; ++j) {
        Dm[c][j][0] = q[j].x;
        Dm[c][j][1] = q[j].y;
        Dm[c][j][2] = q[j].z;
        Dm[c][j][3] = q[j].w;
        const float nx4 = __shfl_down_sync(0xffffffffu, q[j].x, 1);
        Dm[c][j][4] = lane < 31 ? nx4 : d5[j];
      }
    }
    const bool top_last = ez == p.nz - 1;
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
        float4 q = *reinterpret_cast<const float4 *>(G + g);
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

// 128 registers per thread for SH, 168 for P-SV
template <int NDOF>
__global__ void __launch_bounds__(32 * kMarchWarps, NDOF == 1 ? 4 : 3)
    adj_march_forces(const __grid_constant__ MarchAdjParams p, const MarchUnit *units, int nunits) {
  const int uid = blockIdx.x * kMarchWarps + (threadIdx.x >> 5);
  __shared__ AdjRowTable tab[kMarchWarps];
  if (uid < nunits) adj_forces_unit<NDOF>(p, units[uid], &tab[threadIdx.x >> 5]);
}

template <int NDOF>
__global__ void __launch_bounds__(32 * kMarchWarps, NDOF == 1 ? 4 : 3)
    adj_march_moduli(const __grid_constant__ MarchAdjParams p, const MarchUnit *units, int nunits) {
  const int uid = blockIdx.x * kMarchWarps + (threadIdx.x >> 5);
  if (uid < nunits) adj_moduli_unit<NDOF>(p, units[uid]);
}

}  // namespace sem2d

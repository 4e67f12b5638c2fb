// march_kernel.cuh -- the FP32 time step of NGLL = 5 isotropic problems with
// one element per thread, marching up columns of elements.
//
// Same pass as the strip kernel (solve_leapfrog, solver.f90:140-161, with
// compute_Fint solver.f90:273-316, ELAST_KD1/KD2 mat_elastic.f90:464-775,
// SO_add src_gen.f90:290-317, BC_ABSO_apply bc_abso.f90:286-319,
// BC_DYNFLT_apply bc_dynflt.f90:569-739 and REC_store receivers.f90:309-344)
// for the common case: FP32 fields, NGLL = 5, isotropic material given per
// node or per element, leapfrog, no Kelvin-Voigt, no 2.5D term.
//
// Work decomposition.  A warp owns a strip of 31 element columns and a chunk
// of element rows.  Lane k computes element column 31*strip - 1 + k: lane 0
// is the column left of the strip, whose forces on the strip's left edge
// nodes are needed.  The warp walks up its chunk one element row at a time,
// starting one row below the chunk when that row shares nodes with it.  A
// lane holds its element's 5x5 displacements, gradients, stress terms and
// nodal forces in registers; the 5-point contractions are unrolled FMAs
// with the GLL matrix read from the kernel's constant parameter block.
//
// Assembly without shared memory.  Lower-left node ownership: lane k owns
// nodes i = 0..3, j = 0..3 of its element (plus the right column of the
// last element column and the top row of the last element row).  The
// forces of the element on its left neighbour's shared column come from
// lane k-1 by a warp shuffle; the forces on the node row shared with the
// next element row stay in registers (the carry).  The summation order at
// every node is the strip kernel's: lower element row before upper, left
// element before right, so both kernels assemble identically.
//
// Memory.  A lane reads the 4 node columns it owns of each node row as one
// 16-byte load (the warp reads 512 contiguous bytes) and gets the fifth
// column from the next lane; fields, inverse mass and node material are
// read this way, written the same way.  Nothing is staged: the latency of
// a row's loads is covered by the other resident warps.
//
// State.  Two formulations of the leapfrog state (FST):
//  * displacement state (FST = false): the element pass applies the
//    stiffness to the displacement predictor d, f = -K d, as the reference
//    does (solver.f90:140-161);
//  * force state (FST = true, problems with a fault): the elastic force is
//    carried from step to step, f_el(n) = f_el(n-1) + dt (-K v), and the
//    element pass applies the stiffness to the velocity.  The two agree in
//    exact arithmetic (K is linear and d(n) = d(n-1) + dt v).  In FP32 the
//    displacement next to a fault that has slipped metres is quantised to
//    its ulp (5e-7 m at 5 m), which is the size of the node-to-node
//    differences that carry the dynamic stress: its stiffness products
//    lose about 3 digits and the slip rate and seismograms drift from the
//    FP64 result by parts per thousand over thousands of steps.  The
//    velocity and the net elastic force carry no static offset, so they
//    keep FP32's relative precision.  The displacement is still integrated
//    (d += dt v) for the outputs; the force state costs one more plane
//    read and written per dof.
//
// Fault.  The complete forces of the split node rows jf1 (top of the
// elements below the fault) and jf2 (bottom of the elements above),
// sources and dashpots included, go to a small buffer; a second kernel
// with one thread per fault node pair runs the FP64 fault update
// (fault_node_update) and finishes those nodes.  Inside the march kernel a
// lane would run it for four node pairs in turn, and the rate-and-state
// Newton solves made the fault warps the critical path.
//
// Receivers.  Each unit (strip, chunk) samples the receivers it owns after
// its walk: node receivers read the buffers just written by the warp,
// interpolated displacement receivers read the step's input displacement.
// (Velocity or acceleration receivers on a fault row are sampled by the
// separate receiver kernel after the fault kernel.)
#pragma once

#include "fault_kernel.cuh"
#include "sem2d_common.cuh"

namespace sem2d {

constexpr int kMarchWarps = 4;     // warps per CTA at most (the launch picks 1, 2 or 4)
constexpr int kMarchCols = 31;     // element columns owned by a warp
// resident CTAs per SM the register budget allows: 102 registers per
// thread for SH (20 warps per SM), 168 for P-SV (12 warps; fewer registers
// spill the node-material variant)
template <int NDOF>
struct MarchOcc {
  static constexpr int kMinBlocks = NDOF == 1 ? 5 : 3;
};

// one unit of work: a strip of element columns and a chunk of element rows
// of one problem, with its receivers rec_ids[rec0 .. rec1)
struct MarchUnit {
  int prob, strip, z0, z1, rec0, rec1;
};

struct MarchBatch {
  float H[25], w[5];                 // GLL operator (the same for every problem)
  const BulkParams<float, 5> *sims;  // per problem
  const MarchUnit *units;
  int nunits;
  int *step;
  unsigned *done;
};

__device__ __forceinline__ float4 ldg4(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }

// P-SV: the node update's input rows of an element row are staged in
// shared memory by cp.async when the row starts, so that their loads fly
// while the element forces are computed: per warp, node rows j = 0..4, 16
// bytes per lane and plane, each lane reading back only what it copied.
// The planes are those the element pass has not just read: in the
// displacement state v and the inverse mass (the adjoint step also a^n and
// the mass sum), in the force state the force and displacement and the
// inverse mass.  (SH loads them directly: staged it measured slower.)
__host__ __device__ constexpr bool march_staged(int ndof, bool fst) { return ndof == 2; }
__host__ __device__ constexpr int march_stage_planes(int ndof, bool fst, bool adj) {
  return fst ? 2 * ndof + 1 : (adj ? 2 * ndof + 2 : ndof + 1);
}
__host__ __device__ constexpr int march_stage_f4(int ndof, bool fst, bool adj = false) {
  return 5 * march_stage_planes(ndof, fst, adj) * 32;
}
__host__ __device__ constexpr int march_stage_bytes(int ndof, bool fst, bool adj = false) {
  return march_staged(ndof, fst) ? march_stage_f4(ndof, fst, adj) * 16 : 0;
}

__device__ __forceinline__ void cp_async16(float4 *dst, const float *src) {
  const unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// What one reverse step of the discrete adjoint (ADJ, march_adjoint.cuh)
// reads and writes beyond a forward step's planes: the forward a^n and
// v^{n-1}, and the mass and dashpot gradient sums.
struct MarchAdj {
  const float *a, *vprev;
  float *g_M;               // plane
  float *g_C;               // [c * nslot + perimeter slot]
};

// one unit of one problem (FST: the force-state formulation; ADJ: a
// reverse step of the adjoint, whose state (lambda, w) steps like (d, v))
template <int NDOF, int MAT, bool FST, bool ADJ = false>
__device__ __forceinline__ void march_unit(const BulkParams<float, 5> &p, const float *H, const float *w,
                                           const MarchUnit &u, int it, float4 *stage,
                                           const MarchAdj *x = nullptr) {
  constexpr int N = 5;
  const int lane = threadIdx.x & 31;
  const int ex = kMarchCols * u.strip - 1 + lane;
  const bool act = ex >= 0 && ex < p.nx;         // computes an element
  const bool ld = ex >= 0 && ex <= p.nx;         // loads node columns 4ex..4ex+3
  const bool own = act && lane > 0;              // owns nodes of its element
  const bool last_col = act && ex == p.nx - 1;   // also owns the right column
  const int I0 = 4 * (ex < 0 ? 0 : ex);
  const long long pl = p.plane;
  const float xix = act ? p.xix[ex] : 0.f, dxdxi = act ? p.dxdxi[ex] : 0.f;
  const bool kd2 = p.kd2 != 0;
  const int nslot = perimeter_slots(p.LX, p.LZ);
  const float dt = p.dt, cv = p.cv;
  const bool src_on = it <= p.nt && p.nsrc > 0;
  // the node update reads the step's inputs and writes other buffers
  const float *__restrict__ Vc = p.Vcur;
  const float *__restrict__ Dc = p.Dcur;
  const float *__restrict__ Rm = p.rmass;
  float *__restrict__ Vn = p.Vnext;
  float *__restrict__ Dn = p.Dnext;
  float *__restrict__ An = p.Anext;
  // force state: the elastic force of the step before, and of this step
  const float *__restrict__ Fc = p.Fcur;
  float *__restrict__ Fn = p.Fnext;
  // the field the stiffness is applied to
  const float *__restrict__ Ue = FST ? p.Vcur : p.Dcur;

  // first element row walked: one below the chunk when they share nodes
  int zs = u.z0;
  if (u.z0 > 0 && p.row0[u.z0] == p.row0[u.z0 - 1] + (N - 1)) zs = u.z0 - 1;

  float carry[NDOF][N];  // forces on the node row shared with the next element row
#pragma unroll
  for (int c = 0; c < NDOF; ++c)
#pragma unroll
    for (int i = 0; i < N; ++i) carry[c][i] = 0.f;
  bool have_carry = false;

  // the rows of the next element row are requested while the current
  // row's nodes are updated: 16-byte parts here, the fifth column
  // (shuffled or, for lane 31, loaded) when the row starts
  // (P-SV: requested at the row start instead; carrying them through the
  // node update costs more registers than P-SV has)
  constexpr bool kPrefetch = NDOF == 1;
  float4 nq[NDOF][N];
  float n5[NDOF][N];
  auto fetch_u = [&](int ezn) {
    const long long o = (long long)p.row0[ezn] * p.pitch;
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        const float *b = Ue + c * pl + o + (long long)j * p.pitch + I0;
        nq[c][j] = ld ? ldg4(b) : make_float4(0.f, 0.f, 0.f, 0.f);
        n5[c][j] = (lane == 31 && act) ? __ldg(b + 4) : 0.f;
      }
  };
  if (kPrefetch) fetch_u(zs);

  constexpr int NP = march_stage_planes(NDOF, FST, ADJ);  // staged planes per node row
  constexpr bool kStage = march_staged(NDOF, FST);
  // staged plane index: v (or, in the force state, F then d), inverse mass, a^n, mass sum
  constexpr int PR = FST ? 2 * NDOF : NDOF, PA = NDOF + 1, PG = 2 * NDOF + 1;
  for (int ez = zs; ez < u.z1; ++ez) {
    const bool halo = ez < u.z0;
    const int J0 = p.row0[ez];
    const float etaz = act ? p.etaz[ez] : 0.f;
    const float det = dxdxi * (act ? p.dzdeta[ez] : 0.f);
    const long long eidx = (long long)ez * p.nx + (ex < 0 ? 0 : ex);
    // a source in the node rows of this element row (the lanes test each
    // row's sources only then)
    bool src_row = false;
    if (!ADJ && src_on && !halo)
      for (int s = 0; s < p.nsrc; ++s) src_row = src_row || (p.src_J[s] >= J0 && p.src_J[s] < J0 + N);
    // the node rows this element row updates (below), staged now
    if (kStage && !halo && own) {
      const int nrow = (ez == p.nz - 1 || (p.has_fault && J0 + N - 1 == p.jf1)) ? N : N - 1;
#pragma unroll
      for (int j = 0; j < N; ++j)
        if (j < nrow) {
          const long long g = (long long)(J0 + j) * p.pitch + I0;
#pragma unroll
          for (int c = 0; c < NDOF; ++c) {
            if (FST) {
              cp_async16(stage + (j * NP + c) * 32 + lane, p.Fcur + c * pl + g);
              cp_async16(stage + (j * NP + NDOF + c) * 32 + lane, p.Dcur + c * pl + g);
            } else {
              cp_async16(stage + (j * NP + c) * 32 + lane, p.Vcur + c * pl + g);
            }
          }
          cp_async16(stage + (j * NP + PR) * 32 + lane, p.rmass + g);
          if (ADJ) {
#pragma unroll
            for (int c = 0; c < NDOF; ++c) cp_async16(stage + (j * NP + PA + c) * 32 + lane, x->a + c * pl + g);
            cp_async16(stage + (j * NP + PG) * 32 + lane, x->g_M + g);
          }
        }
      cp_async_commit();
    }

    // ---- element forces: A holds u (d, or v with FST), then d/deta; B holds d/dxi ----
    float A[NDOF][N][N], B[NDOF][N][N];
    if (!kPrefetch) fetch_u(ez);
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
#pragma unroll
      for (int j = 0; j < N; ++j) {
        A[c][j][0] = nq[c][j].x;
        A[c][j][1] = nq[c][j].y;
        A[c][j][2] = nq[c][j].z;
        A[c][j][3] = nq[c][j].w;
        const float nx4 = __shfl_down_sync(0xffffffffu, nq[c][j].x, 1);
        A[c][j][4] = lane < 31 ? nx4 : n5[c][j];
      }
    // d/dxi at (i,j): sum_q H[q + N i] u(q,j)
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
    // d/deta at (i,j): sum_q u(i,q) H[q + N j], column by column in place
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
    // stress terms at every point: column part (weights -W xix) into B,
    // row part (weights -W etaz) into A
    float em0 = 0.f, em1 = 0.f;
    if (MAT == kMatElement && act) {
      em0 = p.mat[0][eidx];
      if (NDOF == 2) em1 = p.mat[1][eidx];
    }
    // node material: the 16-byte parts of row j+1 are requested before row
    // j is used
    float4 mq[2][2];
    float m5[2][2];
    auto fetch_m = [&](int j, int slot) {
      if (MAT != kMatNode) return;
#pragma unroll
      for (int m = 0; m < NDOF; ++m) {
        const float *b = p.mat[m] + (long long)(J0 + j) * p.pitch + I0;
        mq[slot][m] = ld ? ldg4(b) : make_float4(0.f, 0.f, 0.f, 0.f);
        m5[slot][m] = (lane == 31 && act) ? __ldg(b + 4) : 0.f;
      }
    };
    fetch_m(0, 0);
#pragma unroll
    for (int j = 0; j < N; ++j) {
      float m0[N], m1[N];
      if (MAT == kMatNode) {
        if (j + 1 < N) fetch_m(j + 1, (j + 1) & 1);
#pragma unroll
        for (int m = 0; m < NDOF; ++m) {
          const float4 q = mq[j & 1][m];
          float *v = m == 0 ? m0 : m1;
          v[0] = q.x;
          v[1] = q.y;
          v[2] = q.z;
          v[3] = q.w;
          const float nx4 = __shfl_down_sync(0xffffffffu, q.x, 1);
          v[4] = lane < 31 ? nx4 : m5[j & 1][m];
        }
      } else {
#pragma unroll
        for (int i = 0; i < N; ++i) {
          m0[i] = em0;
          m1[i] = em1;
        }
      }
      const float wdtj = det * w[j];
#pragma unroll
      for (int i = 0; i < N; ++i) {
        const float wdti = det * w[i];
        if (NDOF == 1) {
          // SH: mu = m0
          const float cxx = -(wdtj * xix) * xix, czz = -(wdti * etaz) * etaz;
          B[0][j][i] = (cxx * w[i]) * (m0[i] * B[0][j][i]);
          A[0][j][i] = (czz * w[j]) * (m0[i] * A[0][j][i]);
        } else {
          // P-SV: la = m0, mu = m1
          const float la = m0[i], mu = m1[i];
          const float K = la + 2.f * mu;
          const float gxx = B[0][j][i], gxz = B[1][j][i], gex = A[0][j][i], gez = A[1][j][i];
          const float dxux = xix * gxx, dxuz = xix * gxz, dzux = etaz * gex, dzuz = etaz * gez;
          const float wc = -(wdtj * xix) * w[i];
          const float wr = -(wdti * etaz) * w[j];
          const float sxz = kd2 ? etaz : xix;
          B[0][j][i] = wc * (K * dxux + la * dzuz);
          B[1][j][i] = wc * (mu * (dzux + dxuz));
          A[0][j][i] = wr * (mu * (dzux + sxz * gxz));
          A[1][j][i] = wr * (la * dxux + K * dzuz);
        }
      }
    }
    // divergence: column part sum_q H[i + N q] B(q,j) row by row in place
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
    // plus the row part sum_q A(i,q) H[j + N q]: nodal forces into B
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

    // ---- assembly: forces of the left element on column 0 ----
    float L[NDOF][N];
#pragma unroll
    for (int c = 0; c < NDOF; ++c)
#pragma unroll
      for (int j = 0; j < N; ++j) L[c][j] = __shfl_up_sync(0xffffffffu, B[c][j][N - 1], 1);

    if (kPrefetch && ez + 1 < u.z1) fetch_u(ez + 1);

    // the top node row: shared with the next element row (carry), the
    // lattice's top row, a fault side-1 row, or the next chunk's
    const int Jt = J0 + N - 1;
    const bool top_last = ez == p.nz - 1;
    const bool top_shared = !top_last && p.row0[ez + 1] == Jt;
    const bool bottom_carry = have_carry;
    // complete forces at node (i, j) of this element row (j = 0..4)
    auto fsum = [&](int c, int j, int i) -> float {
      float f = (j == 0 && bottom_carry) ? carry[c][i] : 0.f;
      if (i == 0) f = f + L[c][j];
      return f + B[c][j][i];
    };

    // the forces on the shared top row become the next row's carry (after
    // row 0 has used the previous carry)
    auto set_carry = [&]() {
      if (top_shared) {
#pragma unroll
        for (int c = 0; c < NDOF; ++c)
#pragma unroll
          for (int i = 0; i < N; ++i) carry[c][i] = (i == 0 ? L[c][N - 1] : 0.f) + B[c][N - 1][i];
      }
    };

    // rows finished by this element row: j = 0..3 unless halo, j = 4 when
    // the top row is not shared (lattice top or fault side 1) and this
    // chunk owns it
    if (!halo) {
      if (kStage && own) cp_async_wait_all();
#pragma unroll
      for (int j = 0; j < N; ++j) {
        if (j == 1) set_carry();
        const int J = J0 + j;
        if (j == N - 1 && !(top_last || (p.has_fault && J == p.jf1))) break;
        const long long g = (long long)J * p.pitch + I0;
        const bool fault_row = p.has_fault && (J == p.jf1 || J == p.jf2);
        const bool edgeJ = J == 0 || J == p.LZ - 1;
        // the 4 owned columns, plus the right column for the last element
        float f[NDOF][N];
#pragma unroll
        for (int c = 0; c < NDOF; ++c)
#pragma unroll
          for (int i = 0; i < N; ++i) f[c][i] = fsum(c, j, i);
        if (FST && own) {
          // the elastic force of this step: the previous one plus dt (-K v)
#pragma unroll
          for (int c = 0; c < NDOF; ++c) {
            const float4 q = kStage ? stage[(j * NP + c) * 32 + lane] : ldg4(Fc + c * pl + g);
            const float fp[N] = {q.x, q.y, q.z, q.w, last_col ? __ldg(Fc + c * pl + g + 4) : 0.f};
#pragma unroll
            for (int i = 0; i < N; ++i) f[c][i] = fp[i] + dt * f[c][i];
            *reinterpret_cast<float4 *>(Fn + c * pl + g) = make_float4(f[c][0], f[c][1], f[c][2], f[c][3]);
            if (last_col) Fn[c * pl + g + 4] = f[c][4];
          }
        }
        if (!ADJ && src_row) {
          for (int s = 0; s < p.nsrc; ++s) {
            const int sI = p.src_I[s], sJ = p.src_J[s];
            if (sJ == J && own && sI >= I0 && sI < I0 + 4 + (last_col ? 1 : 0)) {
#pragma unroll
              for (int c = 0; c < NDOF; ++c) {
                const float amp = float(p.src_amp[((long long)s * NDOF + c) * (p.nt + 1) + it]);
#pragma unroll
                for (int i = 0; i < N; ++i)
                  if (sI == I0 + i) f[c][i] = f[c][i] + amp;
              }
            }
          }
        }
        if (!own) continue;
        float vv[NDOF][N], rmv[N];
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          const float4 q = (kStage && !FST) ? stage[(j * NP + c) * 32 + lane] : ldg4(Vc + c * pl + g);
          vv[c][0] = q.x;
          vv[c][1] = q.y;
          vv[c][2] = q.z;
          vv[c][3] = q.w;
          vv[c][4] = last_col ? __ldg(Vc + c * pl + g + 4) : 0.f;
        }
        {
          const float4 q = kStage ? stage[(j * NP + PR) * 32 + lane] : ldg4(Rm + g);
          rmv[0] = q.x;
          rmv[1] = q.y;
          rmv[2] = q.z;
          rmv[3] = q.w;
          rmv[4] = last_col ? __ldg(Rm + g + 4) : 0.f;
        }
        // dashpots and the perimeter inverse mass (only lanes with a node on
        // the perimeter in this row look at the table; the adjoint applies
        // the dashpots to its lambda update below)
#pragma unroll
        for (int i = 0; i < N; ++i) {
          const int I = I0 + i;
          if (i == N - 1 && !last_col) continue;
          if (edgeJ || I == 0 || I == p.LX - 1) {
            const int sp = perimeter_slot(I, J, p.LX, p.LZ);
            if (!ADJ) {
#pragma unroll
              for (int c = 0; c < NDOF; ++c) {
                const int so = c * nslot + sp;
                f[c][i] = f[c][i] - p.per_Ca[so] * vv[c][i];
                f[c][i] = f[c][i] - p.per_Cb[so] * vv[c][i];
                if (p.per_bf) f[c][i] = f[c][i] + p.per_bf[so];
              }
            }
            rmv[i] = p.per_rm[sp];  // dof 0 entry; dof 1 below
          }
        }
        if (fault_row) {
          // finished by the fault kernel after the step
          const int side = J == p.jf1 ? 0 : 1;
#pragma unroll
          for (int c = 0; c < NDOF; ++c)
#pragma unroll
            for (int i = 0; i < N; ++i)
              if (i < N - 1 || last_col) p.fault_force[(side * NDOF + c) * p.flt.nflt + I0 + i] = f[c][i];
          continue;
        }
        // a = rmass f, v += dt a, d += dt v
        float dv[NDOF][N];
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          const float4 q = (kStage && FST) ? stage[(j * NP + NDOF + c) * 32 + lane] : ldg4(Dc + c * pl + g);
          dv[c][0] = q.x;
          dv[c][1] = q.y;
          dv[c][2] = q.z;
          dv[c][3] = q.w;
          dv[c][4] = last_col ? __ldg(Dc + c * pl + g + 4) : 0.f;
        }
        float gm[N];
#pragma unroll
        for (int i = 0; i < N; ++i) gm[i] = 0.f;
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          float vn[N], dn[N], an[N];
          float aq[N];
          if (ADJ) {
            const float4 q = kStage ? stage[(j * NP + PA + c) * 32 + lane] : ldg4(x->a + c * pl + g);
            aq[0] = q.x;
            aq[1] = q.y;
            aq[2] = q.z;
            aq[3] = q.w;
            aq[4] = last_col ? __ldg(x->a + c * pl + g + 4) : 0.f;
          }
#pragma unroll
          for (int i = 0; i < N; ++i) {
            float rm = rmv[i];
            const int I = I0 + i;
            const bool edge = (edgeJ || I == 0 || I == p.LX - 1) && (i < N - 1 || last_col);
            if (c == 1 && edge) rm = p.per_rm[nslot + perimeter_slot(I, J, p.LX, p.LZ)];
            if (ADJ) {
              // w^n = w^{n+1} + dt M^-1 F lambda^n;
              // lambda^{n-1} = (1 - dt M^-1 C) lambda^n + dt w^n
              // (the receivers' misfit derivatives are added after the launch)
              const float a = rm * f[c][i];
              an[i] = a;
              vn[i] = vv[c][i] + cv * a;
              float lam = dv[c][i];
              gm[i] = gm[i] - lam * aq[i];  // mass term of the gradient with lambda^n
              if (edge) {
                const int so = c * nslot + perimeter_slot(I, J, p.LX, p.LZ);
                lam = lam - (dt * rm) * ((p.per_Ca[so] + p.per_Cb[so]) * dv[c][i]);
                // dashpot term
                x->g_C[so] += -dv[c][i] * (x->vprev[c * pl + g + i] + (0.5f * dt) * aq[i]);
              }
              dn[i] = lam + dt * vn[i];
            } else {
              const float a = rm * f[c][i];
              an[i] = a;
              vn[i] = vv[c][i] + cv * a;
              dn[i] = dv[c][i] + dt * vn[i];
            }
          }
          *reinterpret_cast<float4 *>(Vn + c * pl + g) = make_float4(vn[0], vn[1], vn[2], vn[3]);
          *reinterpret_cast<float4 *>(Dn + c * pl + g) = make_float4(dn[0], dn[1], dn[2], dn[3]);
          if (An) *reinterpret_cast<float4 *>(An + c * pl + g) = make_float4(an[0], an[1], an[2], an[3]);
          if (last_col) {
            Vn[c * pl + g + 4] = vn[4];
            Dn[c * pl + g + 4] = dn[4];
            if (An) An[c * pl + g + 4] = an[4];
          }
        }
        if (ADJ) {
          float4 q = kStage ? stage[(j * NP + PG) * 32 + lane] : *reinterpret_cast<const float4 *>(x->g_M + g);
          q.x = q.x + gm[0];
          q.y = q.y + gm[1];
          q.z = q.z + gm[2];
          q.w = q.w + gm[3];
          *reinterpret_cast<float4 *>(x->g_M + g) = q;
          if (last_col) x->g_M[g + 4] = x->g_M[g + 4] + gm[4];
        }
      }
    }
    if (halo) set_carry();
    have_carry = top_shared;
  }

  // ---- receivers of this unit ----
  if (!ADJ && p.rec_ids && u.rec1 > u.rec0 && it % p.rec_isamp == 0 && it / p.rec_isamp < p.rec_nsamp) {
    __syncwarp();
    __threadfence_block();
    const int s = it / p.rec_isamp, nr = u.rec1 - u.rec0;
    for (int q = lane; q < nr * NDOF; q += 32) {
      const int r = p.rec_ids[u.rec0 + q % nr], c = q / nr;
      double val;
      if (p.rec_npts == 1) {
        const long long g = (long long)p.rec_J[r] * p.pitch + p.rec_I[r] + c * pl;
        const float *fld = p.rec_field == 'D' ? p.Dcur : (p.rec_field == 'V' ? p.Vnext : p.Anext);
        val = double(__ldcg(fld + g));
      } else {
        const int *RI = p.rec_I + (size_t)r * p.rec_npts, *RJ = p.rec_J + (size_t)r * p.rec_npts;
        const double *W = p.rec_w + (size_t)r * p.rec_npts;
        const float *fld = p.Dcur + c * pl;
        val = W[0] * double(fld[(long long)RJ[0] * p.pitch + RI[0]]);
        for (int k = 1; k < p.rec_npts; ++k) val = val + W[k] * double(fld[(long long)RJ[k] * p.pitch + RI[k]]);
      }
      p.sis[s + (size_t)p.rec_nsamp * (r + (size_t)p.rec_nrec * c)] = val;
    }
  }
}

// the last CTA to finish bumps the step counter
__device__ __forceinline__ void march_done(int *step, unsigned *done, int it) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(done, 1u);
    if (prev == gridDim.x - 1) {
      *done = 0u;
      __threadfence();
      *step = it;
    }
  }
}

// one problem: warp w of CTA b walks unit (warps per CTA)*b + w; the launch
// picks 1, 2 or 4 warps per CTA (with one, a warp that finishes its unit
// frees its slot at once)
template <int NDOF, int MAT, bool FST>
__global__ void __launch_bounds__(32 * kMarchWarps, MarchOcc<NDOF>::kMinBlocks)
    march_step_kernel(const __grid_constant__ BulkParams<float, 5> p, const MarchUnit *units, int nunits) {
  const int warp = threadIdx.x >> 5;
  const int it = *p.step + 1;
  const int uid = blockIdx.x * (blockDim.x >> 5) + warp;
  extern __shared__ float4 march_stage[];
  if (uid < nunits) {
    const MarchUnit u = units[uid];
    march_unit<NDOF, MAT, FST>(p, p.H, p.w, u, it, march_stage + warp * march_stage_f4(NDOF, FST));
  }
  march_done(p.step, p.done, it);
}

// many problems (without faults: the displacement state): the units of all
// problems, each with its parameter block
template <int NDOF, int MAT>
__global__ void __launch_bounds__(32 * kMarchWarps, MarchOcc<NDOF>::kMinBlocks)
    march_batch_kernel(const __grid_constant__ MarchBatch b) {
  const int warp = threadIdx.x >> 5;
  const int it = *b.step + 1;
  const int uid = blockIdx.x * (blockDim.x >> 5) + warp;
  extern __shared__ float4 march_stage[];
  if (uid < b.nunits) {
    const MarchUnit u = b.units[uid];
    march_unit<NDOF, MAT, false>(b.sims[u.prob], b.H, b.w, u, it, march_stage + warp * march_stage_f4(NDOF, false));
  }
  march_done(b.step, b.done, it);
}

// The fault side of a step in one launch (slip- or time-weakening
// friction): CTA s runs the fault-side units of strip s (unit w*nstrips + s
// on warp w, w < nrows), then its threads finish the strip's fault node
// pairs (columns 124 s .. 124 s + 123, and the last column on the last
// strip) from the forces its warps wrote; the last CTA bumps the counter.
template <int NDOF, int MAT, bool FST>
__global__ void __launch_bounds__(32 * kMarchWarps, MarchOcc<NDOF>::kMinBlocks)
    march_fault_side_kernel(const __grid_constant__ BulkParams<float, 5> p, const MarchUnit *units, int nstrips,
                            int nrows) {
  const int warp = threadIdx.x >> 5, s = blockIdx.x;
  const int it = *p.step + 1;
  extern __shared__ float4 march_stage[];
  if (warp < nrows)
    march_unit<NDOF, MAT, FST>(p, p.H, p.w, units[warp * nstrips + s], it,
                               march_stage + warp * march_stage_f4(NDOF, FST));
  __syncthreads();  // the strip's fault-row forces are written (global memory, this block)
  const int t = threadIdx.x, I = 4 * kMarchCols * s + t;
  const bool mine = (t < 4 * kMarchCols && I < p.LX) || (t == 4 * kMarchCols && I == p.LX - 1);
  if (mine) {
    const float *ff = p.fault_force;
    const int nf = p.flt.nflt;
    double f1[2] = {0, 0}, f2[2] = {0, 0};
    for (int c = 0; c < NDOF; ++c) {
      f1[c] = double(ff[(0 * NDOF + c) * nf + I]);
      if (p.flt.two) f2[c] = double(ff[(1 * NDOF + c) * nf + I]);
    }
    fault_node_update(p.flt, I, it, f1, f2);
  }
  march_done(p.step, p.done, it);
}

// the fault node pairs of the step the march kernel just completed
__global__ void march_fault_kernel(const __grid_constant__ FaultParams<float> p, const float *ff) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= p.nflt) return;
  const int it = *p.step;
  double f1[2] = {0, 0}, f2[2] = {0, 0};
  for (int c = 0; c < p.ndof; ++c) {
    f1[c] = double(ff[(0 * p.ndof + c) * p.nflt + k]);
    if (p.two) f2[c] = double(ff[(1 * p.ndof + c) * p.nflt + k]);
  }
  fault_node_update(p, k, it, f1, f2);
}

}  // namespace sem2d

// strip_kernel.cuh -- one fused launch per time step, streaming element rows
// through shared memory with bulk asynchronous copies.
//
// For every lattice node a CTA owns, one launch performs what the reference
// does in one pass of solve_leapfrog / solve_Newmark (solver.f90:42-83,
// 140-161):
//   f = -K d            compute_Fint (solver.f90:273-316) with MAT_Fint ->
//                       ELAST_KD1/KD2 (mat_elastic.f90:464-775), the
//                       Kelvin-Voigt term (mat_kelvin_voigt.f90:137-151) and
//                       the 2.5D term (mat_elastic.f90:447-459)
//   f += sources        SO_add (src_gen.f90:290-317)
//   f -= C v            BC_ABSO_apply (bc_abso.f90:286-319)
//   dynamic fault       BC_DYNFLT_apply (bc_dynflt.f90:569-739), FP64
//   a = rmass f, v += c a, next displacement predictor
//   seismograms         REC_store (receivers.f90:309-344) for the receivers
//                       the CTA owns
// and the last CTA to finish advances the device step counter.
//
// Work decomposition.  A CTA owns a strip of SW element columns and a chunk
// of element rows ztile[y]..ztile[y+1] (lower-left node ownership).  It
// walks up the chunk in batches of R element rows.  Each batch computes
// the SW element columns plus the one to their left (a halo, whose forces
// on the strip's left edge nodes are needed) -- SW1 * R elements, exactly
// one per thread group -- into per-element force arrays, then assembles
// every owned node by summing the arrays of the (at most four) elements
// around it in a fixed order: lower element row before upper, left element
// before right.  A node row shared with the next batch keeps its partial
// sum in a carry buffer; the chunk's first element row is preceded by the
// row below it (a halo row) when the two share nodes.  The summation order
// depends only on element coordinates, so results are bitwise identical for
// every strip/chunk shape.
//
// Data movement.  The lattice rows a batch touches (displacement, node
// material, velocity predictor, inverse mass) are fetched with one
// cp.async.bulk per (row, plane) into one of three stage buffers; the copies
// of batches b+1 and b+2 are in flight while batch b computes (b+2 is
// issued by all threads as soon as batch b-1 has released its stage).
// Every mbarrier wait is bounded: a CTA that times out raises
// SEM2D_E_TIMEOUT, lets its own copies drain and returns.
//
// Element operator.  N threads per element: thread t owns the xi-line
// (x varies) at height t and the eta-line at column t, keeping each
// N-vector in registers.  Gradients dU/dxi = H^T U and dU/deta = U H are
// exchanged through the element's scratch area so that every thread forms
// the stresses of its two lines (the a-coefficients of MAT_ELAST_init_a,
// mat_elastic.f90:323-358, factored as weight x metric x stress) and
// applies the divergence.  For NGLL = 5 in FP32 an xi-line is one 16-byte
// shared load plus one value shuffled from the neighbouring element's
// thread group (a row stride of 20 mod 32 words keeps those loads free of
// bank conflicts).  The scratch area finally holds the element's nodal
// forces.
#pragma once

#include <type_traits>

#include "fault_kernel.cuh"
#include "sem2d_common.cuh"
#include "tma.cuh"

namespace sem2d {

constexpr int kStripThreads = 256;
constexpr int kErrTimeout = -8;  // SEM2D_E_TIMEOUT
constexpr int kMaxChunk = 256;   // element rows of one chunk (host-enforced)
constexpr int kMaxStages = 3;    // stage buffers of the batch pipeline (at most)

template <typename real, int N>
struct StripShape {
  static constexpr int kSlots = 32 / N;                          // elements per warp
  static constexpr int kNSlot = (kStripThreads / 32) * kSlots;   // elements per batch
  static constexpr int SW1 = N == 5 ? 12 : (N == 6 ? 10 : 8);    // element columns with the halo
  static constexpr int R = kNSlot / SW1;                         // element rows per batch
  static constexpr int HR = (N - 1) * R + 2;                     // lattice rows per stage (max)
  static constexpr int AL = 16 / int(sizeof(real));              // copy alignment in words
  // stage buffers: three (batches b+1 and b+2 in flight) unless the FP64
  // stages of NGLL 6 / 9 would not fit, then two
  static constexpr int kStages = (sizeof(real) == 8 && N != 5) ? 2 : kMaxStages;
  static_assert(SW1 * R == kNSlot, "a batch fills every element slot");
};

template <typename real, int NDOF>
struct StripOcc {
  static constexpr int kMinBlocks = sizeof(real) == 4 ? (NDOF == 2 ? 2 : 3) : (NDOF == 2 ? 1 : 2);
};

// row stride (words) of a stage plane: the widest copied row, for NGLL = 5
// in FP32 kept at 20 mod 32 words for conflict-free 16-byte xi-line loads
template <typename real, int N>
__host__ __device__ constexpr int strip_row_stride() {
  using S = StripShape<real, N>;
  const int tw = S::SW1 * (N - 1) + 1 + (S::AL - 1);
  int w = (tw + S::AL - 1) / S::AL * S::AL;
  if (sizeof(real) == 4 && N == 5)
    while (w % 32 != 20) w += S::AL;
  return w;
}

template <typename real, int N, int NDOF>
__host__ __device__ inline size_t strip_smem_bytes(int nplanes) {
  using S = StripShape<real, N>;
  constexpr int tw = strip_row_stride<real, N>();
  const int nscr = NDOF == 2 ? 4 : 1;
  size_t n = size_t(S::kStages) * nplanes * S::HR * tw;  // stage buffers
  n += size_t(S::kNSlot) * nscr * N * N;        // element scratch / nodal forces
  n += 2 * size_t(NDOF) * tw;                   // carry rows (double-buffered)
  n += 2 * size_t(NDOF) * tw;                   // fault-row forces, both sides
  return n * sizeof(real);
}

// One work unit: strip bx of chunk by (gx strips per chunk row) of problem
// p at step it.  bar/ph are the CTA's two stage mbarriers and the parity of
// their next phase; H and w are the GLL operator (shared by all problems of
// a launch).  FAST compiles the common case only: isotropic material,
// leapfrog, no Kelvin-Voigt and no 2.5D term.  Returns false after a bounded
// wait expired.
template <typename real, int N, int NDOF, int MAT, bool FAST>
__device__ __forceinline__ bool strip_unit(const BulkParams<real, N> &p, const real *__restrict__ H,
                                           const real *__restrict__ w, int bx, int by, int gx, int it,
                                           uint64_t *bar, uint32_t *ph, unsigned char *smem_raw) {
  using S = StripShape<real, N>;
  constexpr int NN = N * N, SL = S::kSlots, SW1 = S::SW1, R = S::R, HR = S::HR, AL = S::AL;
  constexpr int NSCR = NDOF == 2 ? 4 : 1;
  constexpr int TWp = strip_row_stride<real, N>();
  constexpr int PS = HR * TWp;  // plane stride in a stage
  constexpr bool kVecX = sizeof(real) == 4 && N == 5;
  constexpr int NW = kStripThreads / 32;
  __shared__ signed char s_r[2][HR], s_j[2][HR], s_stat[HR];
  __shared__ int s_err, s_nsrc;
  __shared__ int s_src[kMaxSrc];
  __shared__ int s_row0[kMaxChunk + 2];  // row0[eza .. ez1]
  __shared__ real s_etaz[kMaxChunk + 1], s_dzdeta[kMaxChunk + 1];
  __shared__ real s_xix[SW1], s_dxdxi[SW1];

  const int NP = p.nplanes;
  const size_t stage_sz = size_t(NP) * PS;
  real *stg = reinterpret_cast<real *>(smem_raw);
  constexpr int NST = S::kStages;
  real *scr = stg + NST * stage_sz;
  real *carry = scr + size_t(S::kNSlot) * NSCR * NN;
  real *fbuf = carry + 2 * NDOF * TWp;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int SW = SW1 - 1;
  const int ex0 = bx * SW, ex1 = min(ex0 + SW, p.nx);
  const int hx = ex0 > 0 ? 1 : 0;
  const int exa = ex0 - hx, ncol = ex1 - exa;
  const int Ia = exa * (N - 1), Ib = (ex1 - 1) * (N - 1) + N;
  const int Ial = Ia & ~(AL - 1), xo = Ia - Ial;
  const int cw = ((Ib + AL - 1) & ~(AL - 1)) - Ial;  // copied row width
  const int I0 = ex0 * (N - 1), I1 = (ex1 == p.nx) ? p.LX : ex1 * (N - 1);
  const int OWc = I1 - I0, ii0 = I0 - Ia;
  const int ez0 = p.ztile[by], ez1 = p.ztile[by + 1];
  const int hz = (ez0 > 0 && p.row0[ez0] == p.row0[ez0 - 1] + (N - 1)) ? 1 : 0;
  const int eza = ez0 - hz;
  const int nb = (ez1 - eza + R - 1) / R;
  const int nm = MAT == kMatNode ? p.nmat : 0;
  const int pV = NDOF + nm, pA = pV + NDOF, pR = NP - 1;
  const bool iso = FAST || p.mat_iso;
  const bool newmark = !FAST && p.scheme != 0;  // Newmark or HHT-alpha
  const bool hht = !FAST && p.scheme == 2;
  const bool kv = !FAST && p.has_kv;
  const real width = FAST ? real(0) : p.width;

  // element-row starts, row and column geometry of this CTA
  for (int k = tid; k <= ez1 - eza; k += kStripThreads) {
    s_row0[k] = p.row0[eza + k];  // row0[nz] == LZ
    if (k < ez1 - eza) {
      s_etaz[k] = p.etaz[eza + k];
      s_dzdeta[k] = p.dzdeta[eza + k];
    }
  }
  for (int k = tid; k < ncol; k += kStripThreads) {
    s_xix[k] = p.xix[exa + k];
    s_dxdxi[k] = p.dxdxi[exa + k];
  }
  if (tid == 0) s_err = 0;
  __syncthreads();
  auto rw = [&](int ez) { return s_row0[ez - eza]; };
  const int J0own = rw(ez0), J1own = rw(ez1);
  if (tid == 0) {
    int n = 0;  // point sources at owned nodes, in source order
    if (it <= p.nt)
      for (int s = 0; s < p.nsrc; ++s) {
        const int I = p.src_I[s], J = p.src_J[s];
        if (I >= I0 && I < I1 && J >= J0own && J < J1own && n < kMaxSrc) s_src[n++] = s;
      }
    s_nsrc = n;
  }

  auto plane_src = [&](int pl) -> const real * {
    if (pl < NDOF) return p.Dcur + pl * p.plane;
    if (pl < pV) return p.mat[pl - NDOF];
    if (pl < pV + NDOF) return p.Vcur + (pl - pV) * p.plane;
    if (pl == pR) return p.rmass;
    return p.Acur + (pl - pA) * p.plane;
  };
  // fetch the lattice rows of batch bb into stage bb % NST; every thread
  // issues at most one of the copies, thread 0 announces the byte count
  auto issue = [&](int bb) {
    const int st = bb % NST;
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

  const int nslot = perimeter_slots(p.LX, p.LZ);
  const int cta = by * gx + bx;
  const int nrec_here = p.rec_tile_start ? p.rec_tile_start[cta + 1] - p.rec_tile_start[cta] : 0;
  const int jflast = p.has_fault ? (p.flt.two ? max(p.jf1, p.jf2) : p.jf1) : -1;

  // per-thread element slot and the geometry that does not change between
  // batches
  const int slot = lane / N, t = lane - slot * N;
  const bool lane_ok = slot < SL;
  const int e_slot = warp * SL + (lane_ok ? slot : 0);
  const int r_slot = e_slot / SW1, c_slot = e_slot - r_slot * SW1;
  real *sc = scr + size_t(e_slot) * NSCR * NN;
  const real xix = lane_ok && c_slot < ncol ? s_xix[c_slot] : real(0);
  const real dxdxi = lane_ok && c_slot < ncol ? s_dxdxi[c_slot] : real(0);
  const real wt = w[t < N ? t : 0];

  for (int b = 0; b < nb; ++b) {
    const int st = b % NST;
    const int eb0 = eza + b * R, eb1 = min(eb0 + R, ez1), nre = eb1 - eb0;
    const int Jlo = rw(eb0), nr = rw(eb1 - 1) + N - Jlo;
    const bool from_carry = b > 0 && rw(eb0) == rw(eb0 - 1) + (N - 1);

    // element rows (batch-local) through each stage row, and the row's fate:
    // 0 not owned here, 1 completed by this batch, 2 carried to the next
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
    if (!mbar_wait(&bar[st], ph[st], p.spin_limit)) atomicOr(&s_err, 1);
    ph[st] ^= 1u;
    __syncthreads();
    if (s_err) {
      if (tid == 0) {
        if (p.error) atomicExch(p.error, kErrTimeout);
        mbar_wait(&bar[st], ph[st] ^ 1u);  // let this CTA's copies drain
        const int s1 = (b + 1) % NST;
        if (b + 1 < nb) mbar_wait(&bar[s1], ph[s1]);
      }
      __syncthreads();
      return false;
    }
    // three stages: batch b-1 has released its stage, fetch batch b+2 into it
    if (NST == 3 && b + 2 < nb) issue(b + 2);

    const real *sg = stg + st * stage_sz;
    const real *sD = sg;
    // force state (leapfrog, no Kelvin-Voigt; Fcur set by the host): the
    // stiffness is applied to the velocity and the elastic force of the
    // step is the previous one plus dt times that, so a large static
    // displacement does not enter the FP32 force
    const bool fst = p.Fcur != nullptr;
    const real *sM = sg + size_t(NDOF) * PS;
    const real *sV = sg + size_t(pV) * PS;
    const real *sA = sg + size_t(pA) * PS;
    const real *sRm = sg + size_t(pR) * PS;
    if (hht) {
      // HHT-alpha: the forces see d_alpha = alpha d_pred + (1-alpha) d_n
      // = d_pred - (1-alpha)(dt v_n + (1/2-beta) dt^2 a_n) (solver.f90:
      // 106-113); the stage holds d_pred, v_n and a_n
      real *sDw = const_cast<real *>(sD);
      for (int q = tid; q < NDOF * PS; q += kStripThreads) {
        const int c = q / PS, o = q - c * PS;
        sDw[q] = sDw[q] - p.cal * (p.dt * sV[c * PS + o] + p.cd2 * sA[c * PS + o]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the stage is refilled by bulk copies
      __syncthreads();
    }

    // ---- element forces of the batch into the scratch areas ----
    {
      const int r = r_slot, c = c_slot;
      const bool act = lane_ok && r < nre && c < ncol;
      const int ez = eb0 + r, ex = exa + c;
      const int eb = act ? (rw(ez) - Jlo) * TWp + xo + c * (N - 1) : 0;
      const real etaz = act ? s_etaz[ez - eza] : real(0);
      const real det = dxdxi * (act ? s_dzdeta[ez - eza] : real(0));
      const long long eidx = (long long)ez * p.nx + ex, eoff = eidx * NN;
      real emat[4] = {0, 0, 0, 0};  // one value per element (MAT == kMatElement)
      if (MAT == kMatElement && act)
        for (int m = 0; m < p.nmat; ++m) emat[m] = p.mat[m][eidx];
      auto matv = [&](int m, int i, int j) -> real {
        if (MAT == kMatPoint) return p.mat[m][eoff + i + N * j];
        if (MAT == kMatElement) return emat[m];
        return sM[m * PS + eb + j * TWp + i];
      };
      // the xi-line at height t of stage plane `pl`
      auto xline = [&](const real *pl, real *v) {
        if constexpr (kVecX) {
          const int base = act ? eb + t * TWp : 0;
          const float4 q4 = *reinterpret_cast<const float4 *>(pl + base);
          v[0] = q4.x;
          v[1] = q4.y;
          v[2] = q4.z;
          v[3] = q4.w;
          // value 4 is value 0 of the next element's line (same node) when
          // that element is computed by the next thread group of the warp
          const float nxt = __shfl_down_sync(0xffffffffu, q4.x, N);
          v[4] = (slot < SL - 1 && c + 1 < ncol) ? nxt : (act ? pl[base + 4] : 0.f);
        } else {
#pragma unroll
          for (int q = 0; q < N; ++q) v[q] = act ? pl[eb + t * TWp + q] : real(0);
        }
      };
      // weights: W(q,t) = det w_q w_t; the a-coefficients are -W times
      // metric factors (mat_elastic.f90:323-358)
      const real wdt = det * wt;
      auto body = [&](auto kv_tag) {
        constexpr bool KV = decltype(kv_tag)::value;
        const real *kve = KV ? p.kveta + eoff : nullptr;
        // displacement (+ eta v, mat_kelvin_voigt.f90:137-151) at (i,j)
        auto uval = [&](int cc, int i, int j) -> real {
          const int idx = eb + j * TWp + i;
          real u = (fst ? sV : sD)[cc * PS + idx];
          if constexpr (KV) {
            real v = sV[cc * PS + idx];
            if (newmark) v = v + (hht ? p.cpa : p.cpred) * sA[cc * PS + idx];  // v_pred or v_alpha
            u = u + kve[i + N * j] * v;
          }
          return u;
        };
        auto xline_u = [&](int cc, real *v) {
          if constexpr (KV) {
#pragma unroll
            for (int q = 0; q < N; ++q) v[q] = act ? uval(cc, q, t) : real(0);
          } else {
            xline((fst ? sV : sD) + cc * PS, v);
          }
        };
        if constexpr (NDOF == 1 && MAT == kMatGeneral) {
          // a grid that is not flat (ELAST_KD1_SH / KD2_SH with nelast = 3,
          // mat_elastic.f90:662-677): the line of point (q,t) is this
          // thread's; dU/deta of (q,t) comes from thread q through the
          // scratch area, as does the eta-part of (t,q)
          real col[N], gxi[N], tA[N], rB[N];
          xline_u(0, col);
          if (act) {
            real rowv[N];
#pragma unroll
            for (int q = 0; q < N; ++q) rowv[q] = uval(0, t, q);
#pragma unroll
            for (int i = 0; i < N; ++i) {
              real a = H[0 + N * i] * col[0];
#pragma unroll
              for (int q = 1; q < N; ++q) a = a + H[q + N * i] * col[q];
              gxi[i] = a;
            }
#pragma unroll
            for (int j = 0; j < N; ++j) {
              real a = rowv[0] * H[0 + N * j];
#pragma unroll
              for (int q = 1; q < N; ++q) a = a + rowv[q] * H[q + N * j];
              sc[t + N * j] = a;  // dU/deta at (t,j)
            }
          }
          __syncwarp();
          if (act) {
            const real *g = p.gen + eoff;
            const long long gs = p.gen_stride;
#pragma unroll
            for (int q = 0; q < N; ++q) {
              const int k = q + N * t;
              const real ge = sc[k];
              const real a1 = g[k], a2 = g[gs + k], a3 = g[2 * gs + k];
              tA[q] = a1 * gxi[q] + a3 * ge;
              sc[k] = a3 * gxi[q] + a2 * ge;  // eta part at (q,t)
            }
          }
          __syncwarp();
          if (act) {
#pragma unroll
            for (int q = 0; q < N; ++q) rB[q] = sc[t + N * q];
          }
          __syncwarp();
          if (act) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              real a = H[i + N * 0] * tA[0];
#pragma unroll
              for (int q = 1; q < N; ++q) a = a + H[i + N * q] * tA[q];
              sc[i + N * t] = a;  // xi part at (i,t)
            }
          }
          __syncwarp();
          if (act) {
#pragma unroll
            for (int j = 0; j < N; ++j) {
              real a = rB[0] * H[j + N * 0];
#pragma unroll
              for (int q = 1; q < N; ++q) a = a + rB[q] * H[j + N * q];
              sc[t + N * j] = sc[t + N * j] + a;  // nodal force of the element at (t,j)
            }
          }
          __syncwarp();
        } else if constexpr (NDOF == 1) {
          real col[N], row[N];
          xline_u(0, col);
          real mx[N];  // mu_x along the xi-line: mu (isotropic) or mux
          if (MAT != kMatNode || !iso) {
#pragma unroll
            for (int q = 0; q < N; ++q) mx[q] = act ? matv(iso ? 0 : 1, q, t) : real(0);
          } else {
            xline(sM, mx);
          }
          if (act) {
#pragma unroll
            for (int q = 0; q < N; ++q) row[q] = uval(0, t, q);
            real gxi[N], geta[N];
#pragma unroll
            for (int i = 0; i < N; ++i) {
              real a = H[0 + N * i] * col[0];
#pragma unroll
              for (int q = 1; q < N; ++q) a = a + H[q + N * i] * col[q];
              gxi[i] = a;
            }
#pragma unroll
            for (int j = 0; j < N; ++j) {
              real a = row[0] * H[0 + N * j];
#pragma unroll
              for (int q = 1; q < N; ++q) a = a + row[q] * H[q + N * j];
              geta[j] = a;
            }
            // column part at points (q,t), row part at points (t,q)
            const real cxx = -(wdt * xix) * xix, czz = -(wdt * etaz) * etaz;
#pragma unroll
            for (int q = 0; q < N; ++q) {
              col[q] = (cxx * w[q]) * (mx[q] * gxi[q]);
              row[q] = (czz * w[q]) * (matv(0, t, q) * geta[q]);
            }
#pragma unroll
            for (int i = 0; i < N; ++i) {
              real a = H[i + N * 0] * col[0];
#pragma unroll
              for (int q = 1; q < N; ++q) a = a + H[i + N * q] * col[q];
              sc[i + N * t] = a;  // column part at (i,t)
            }
          }
          __syncwarp();
          if (act) {
#pragma unroll
            for (int j = 0; j < N; ++j) {
              real a = row[0] * H[j + N * 0];
#pragma unroll
              for (int q = 1; q < N; ++q) a = a + row[q] * H[j + N * q];
              real fl = sc[t + N * j] + a;
              if (width > real(0)) {  // 2.5D term at point (t,j)
                const real pw = real(3.141592653589793) / width;
                const real bt = ((wdt * w[j]) * matv(0, t, j)) * (pw * pw);
                fl = fl - bt * uval(0, t, j);
              }
              sc[t + N * j] = fl;  // nodal force of the element at (t,j)
            }
          }
          __syncwarp();
        } else {
          real *SXX = sc, *SXZ = sc + NN, *SEX = sc + 2 * NN, *SEZ = sc + 3 * NN;
          {
            // gradients of both lines into the scratch area
            real ux[N], uz[N];
            xline_u(0, ux);
            xline_u(1, uz);
            if (act) {
#pragma unroll
              for (int i = 0; i < N; ++i) {
                real a = H[0 + N * i] * ux[0], b2 = H[0 + N * i] * uz[0];
#pragma unroll
                for (int q = 1; q < N; ++q) {
                  a = a + H[q + N * i] * ux[q];
                  b2 = b2 + H[q + N * i] * uz[q];
                }
                SXX[i + N * t] = a;   // dUx/dxi at (i,t)
                SXZ[i + N * t] = b2;  // dUz/dxi at (i,t)
              }
              real vx[N], vz[N];
#pragma unroll
              for (int q = 0; q < N; ++q) {
                vx[q] = uval(0, t, q);
                vz[q] = uval(1, t, q);
              }
#pragma unroll
              for (int j = 0; j < N; ++j) {
                real a = vx[0] * H[0 + N * j], b2 = vz[0] * H[0 + N * j];
#pragma unroll
                for (int q = 1; q < N; ++q) {
                  a = a + vx[q] * H[q + N * j];
                  b2 = b2 + vz[q] * H[q + N * j];
                }
                SEX[t + N * j] = a;   // dUx/deta at (t,j)
                SEZ[t + N * j] = b2;  // dUz/deta at (t,j)
              }
            }
          }
          __syncwarp();
          real cx[N], cz[N], rx[N], rz[N];
          if constexpr (MAT == kMatGeneral) {
            // a grid that is not flat (ELAST_KD1_PSV / KD2_PSV with nelast =
            // 10, mat_elastic.f90:499-516, 620-636): the four products of the
            // gradient at (q,t) with a1..a10, the eta parts handed over in
            // the dU/deta areas
            if (act) {
              const real *g = p.gen + eoff;
              const long long gs = p.gen_stride;
#pragma unroll
              for (int q = 0; q < N; ++q) {
                const int k = q + N * t;
                const real t1 = SXX[k], t2 = SXZ[k], t3 = SEX[k], t4 = SEZ[k];
                const real a1 = g[k], a2 = g[gs + k], a3 = g[2 * gs + k], a4 = g[3 * gs + k],
                           a5 = g[4 * gs + k], a6 = g[5 * gs + k], a7 = g[6 * gs + k], a8 = g[7 * gs + k],
                           a9 = g[8 * gs + k], a10 = g[9 * gs + k];
                cx[q] = a1 * t1 + a7 * t3 + a8 * t2 + a2 * t4;
                cz[q] = a8 * t1 + a5 * t3 + a6 * t2 + a10 * t4;
                SEX[k] = a7 * t1 + a4 * t3 + a5 * t2 + a9 * t4;
                SEZ[k] = a2 * t1 + a9 * t3 + a10 * t2 + a3 * t4;
              }
            }
            __syncwarp();
            if (act) {
#pragma unroll
              for (int q = 0; q < N; ++q) {
                rx[q] = SEX[t + N * q];
                rz[q] = SEZ[t + N * q];
              }
            }
          } else {
            // moduli along the xi-line at height t: (la, mu) or (Kx, la, mu)
            real m0[N], m1[N], m2[N];
            if (MAT == kMatNode && iso) {
              xline(sM, m0);       // la
              xline(sM + PS, m1);  // mu
            } else if (act) {
#pragma unroll
              for (int q = 0; q < N; ++q) {
                if (iso) {
                  m0[q] = matv(0, q, t);
                  m1[q] = matv(1, q, t);
                } else {
                  m2[q] = matv(0, q, t);  // Kx
                  m0[q] = matv(2, q, t);
                  m1[q] = matv(3, q, t);
                }
              }
            }
            if (act) {
              const real wcx = -(wdt * xix);
#pragma unroll
              for (int q = 0; q < N; ++q) {
                // column part at point (q,t): -W xix (sigma_xx, sigma_xz)
                const real la = m0[q], mu = m1[q];
                const real Kx = iso ? la + real(2) * mu : m2[q];
                const int k = q + N * t;
                const real dxux = xix * SXX[k], dxuz = xix * SXZ[k];
                const real dzux = etaz * SEX[k], dzuz = etaz * SEZ[k];
                const real wq = wcx * w[q];
                cx[q] = wq * (Kx * dxux + la * dzuz);
                cz[q] = wq * (mu * (dzux + dxuz));
              }
            }
            if (act) {
              const real wrz = -(wdt * etaz);
              const real sxz = p.kd2 ? etaz : xix;
#pragma unroll
              for (int q = 0; q < N; ++q) {
                // row part at point (t,q): -W etaz (sigma_xz, sigma_zz); the
                // NGLL=5 kernel of the reference uses etaz for both shear
                // terms (mat_elastic.f90:612)
                real la, mu, Kz;
                if (iso) {
                  la = matv(0, t, q);
                  mu = matv(1, t, q);
                  Kz = la + real(2) * mu;
                } else {
                  Kz = matv(1, t, q);
                  la = matv(2, t, q);
                  mu = matv(3, t, q);
                }
                const int k = t + N * q;
                const real dzux = etaz * SEX[k], dzuz = etaz * SEZ[k];
                const real wq = wrz * w[q];
                rx[q] = wq * (mu * (dzux + sxz * SXZ[k]));
                rz[q] = wq * (la * (xix * SXX[k]) + Kz * dzuz);
              }
            }
          }  // flat grid
          __syncwarp();
          if (act) {
#pragma unroll
            for (int i = 0; i < N; ++i) {
              real a = H[i + N * 0] * cx[0], b2 = H[i + N * 0] * cz[0];
#pragma unroll
              for (int q = 1; q < N; ++q) {
                a = a + H[i + N * q] * cx[q];
                b2 = b2 + H[i + N * q] * cz[q];
              }
              SXX[i + N * t] = a;
              SXZ[i + N * t] = b2;
            }
          }
          __syncwarp();
          if (act) {
#pragma unroll
            for (int j = 0; j < N; ++j) {
              real a = rx[0] * H[j + N * 0], b2 = rz[0] * H[j + N * 0];
#pragma unroll
              for (int q = 1; q < N; ++q) {
                a = a + rx[q] * H[j + N * q];
                b2 = b2 + rz[q] * H[j + N * q];
              }
              real flx = SXX[t + N * j] + a, flz = SXZ[t + N * j] + b2;
              if (MAT != kMatGeneral && width > real(0)) {  // 2.5D term at point (t,j), isotropic
                const real la = matv(0, t, j), mu = matv(1, t, j);
                const real nu = (la / (la + mu)) / real(2);
                const real pw = (real(3.141592653589793) * (real(1) - nu)) / width;
                const real bt = ((wdt * w[j]) * mu) * (pw * pw);
                flx = flx - bt * uval(0, t, j);
                flz = flz - bt * uval(1, t, j);
              }
              SXX[t + N * j] = flx;  // nodal forces of the element at (t,j)
              SXZ[t + N * j] = flz;
            }
          }
          __syncwarp();
        }
      };
      if constexpr (FAST) {
        body(std::false_type{});
      } else {
        if (kv) body(std::true_type{});
        else body(std::false_type{});
      }
    }
    __syncthreads();

    // ---- assembly, sources, dashpots, inverse mass, time update ----
    real *cin = carry + ((b & 1) ^ 1) * NDOF * TWp, *cout = carry + (b & 1) * NDOF * TWp;
    // (row, column) pairs over all threads; OWS >= the owned width of a strip
    constexpr int OWS = SW * (N - 1) + 1;
    for (int q = tid; q < nr * OWS; q += kStripThreads) {
      const int jj = q / OWS, io = q - jj * OWS;
      const int fate = s_stat[jj];
      if (fate == 0 || io >= OWc) continue;
      const int ra = s_r[0][jj], ja = s_j[0][jj], rb = s_r[1][jj], jb = s_j[1][jj];
      const int J = Jlo + jj;
      const bool cin_row = jj == 0 && from_carry;
      {
        const int ii = ii0 + io;
        real f[NDOF];
#pragma unroll
        for (int c = 0; c < NDOF; ++c) f[c] = cin_row ? cin[c * TWp + io] : real(0);
        const int ce = ii / (N - 1), il0 = ii - ce * (N - 1);
        // elements (rr, cc) around the node in the fixed order
#pragma unroll
        for (int k = 0; k < 2; ++k) {
          const int rr = k == 0 ? ra : rb, jl = k == 0 ? ja : jb;
          if (rr < 0) continue;
          if (il0 == 0 && ce > 0) {  // right edge of element ce-1
            const real *sl = scr + size_t(rr * SW1 + ce - 1) * NSCR * NN + (N - 1) + N * jl;
#pragma unroll
            for (int c = 0; c < NDOF; ++c) f[c] = f[c] + sl[c * NN];
          }
          if (ce < ncol) {
            const real *sl = scr + size_t(rr * SW1 + ce) * NSCR * NN + il0 + N * jl;
#pragma unroll
            for (int c = 0; c < NDOF; ++c) f[c] = f[c] + sl[c * NN];
          }
        }
        if (fate == 2) {
#pragma unroll
          for (int c = 0; c < NDOF; ++c) cout[c * TWp + io] = f[c];
          continue;
        }
        const int I = I0 + io;
        if (fst) {  // the elastic force of this step: the previous one plus dt (-K v)
          const long long gf = (long long)J * p.pitch + I;
#pragma unroll
          for (int c = 0; c < NDOF; ++c) {
            const real fe = p.Fcur[c * p.plane + gf] + p.dt * f[c];
            p.Fnext[c * p.plane + gf] = fe;
            f[c] = fe;
          }
        }
        for (int k = 0; k < s_nsrc; ++k) {
          const int s = s_src[k];
          if (p.src_I[s] == I && p.src_J[s] == J)
#pragma unroll
            for (int c = 0; c < NDOF; ++c)
              f[c] = f[c] + real(p.src_amp[((long long)s * NDOF + c) * (p.nt + 1) + it]);
        }
        if (p.perio_f && (p.perio_tb ? (J == 0 || J == p.LZ - 1) : (I == 0 || I == p.LX - 1))) {
          // periodic columns (rows): summed and finished after the step
#pragma unroll
          for (int c = 0; c < NDOF; ++c) {
            if (p.perio_tb)
              p.perio_f[(size_t(c) * p.LX + I) * 2 + (J == 0 ? 0 : 1)] = f[c];
            else
              p.perio_f[(size_t(c) * p.LZ + J) * 2 + (I == 0 ? 0 : 1)] = f[c];
          }
          continue;
        }
        const int sidx = jj * TWp + xo + ii;
        const bool edge = (J == 0 || J == p.LZ - 1 || I == 0 || I == p.LX - 1);
        const int sp = edge ? perimeter_slot(I, J, p.LX, p.LZ) : -1;
        const int fside = (J == p.jf1) ? 0 : (J == p.jf2 ? 1 : -1);
        const long long g = (long long)J * p.pitch + I;
#pragma unroll
        for (int c = 0; c < NDOF; ++c) {
          real fc = f[c];
          real vp = sV[c * PS + sidx];
          real vd = vp;  // the dashpots' velocity: v_alpha under HHT-alpha (bc_gen.f90:295)
          if (newmark) {
            const real an = sA[c * PS + sidx];
            vd = vp + (hht ? p.cpa : p.cpred) * an;
            vp = vp + p.cpred * an;
          }
          real rm;
          if (sp >= 0) {
            const int so = c * nslot + sp;
            fc = fc - p.per_Ca[so] * vd;
            fc = fc - p.per_Cb[so] * vd;
            if (p.per_bf) fc = fc + p.per_bf[so];
            if (p.per_kd) fc = fc - p.per_kd[so];
            if (p.per_dir && ((p.per_dir[sp] >> c) & 1)) fc = real(0);  // bc_dirneu.f90:155-167
            rm = p.per_rm[so];
          } else {
            rm = sRm[sidx];
          }
          if (fside >= 0) {  // finished by the fault update
            fbuf[(fside * NDOF + c) * TWp + io] = fc;
            continue;
          }
          const real a = rm * fc;
          const real vnew = vp + p.cv * a;
          real dcur = hht ? p.Dcur[c * p.plane + g] : sD[c * PS + sidx];  // the stage holds d_alpha
          // Newmark corrector d += beta dt^2 a (solver.f90:81-82), then the
          // next step's predictor d + dt v + (1/2 - beta) dt^2 a (:59)
          if (newmark && p.cb != real(0)) dcur = dcur + p.cb * a;
          const real dnext = newmark ? (dcur + p.dt * vnew) + p.cd2 * a : dcur + p.dt * vnew;
          p.Vnext[c * p.plane + g] = vnew;
          p.Dnext[c * p.plane + g] = dnext;
          if (p.Anext) p.Anext[c * p.plane + g] = a;
        }
      }
    }
    __syncthreads();

    // ---- the fault, once its last row is complete (FP64) ----
    if (jflast >= Jlo && jflast < Jlo + nr && s_stat[jflast - Jlo] == 1) {
      for (int I = I0 + tid; I < I1; I += kStripThreads) {
        if (p.perio_f && !p.perio_tb && (I == 0 || I == p.LX - 1)) continue;  // the periodic pass updates these
        const int io = I - I0;
        double f1[2] = {0, 0}, f2[2] = {0, 0};
        for (int c = 0; c < NDOF; ++c) {
          f1[c] = double(fbuf[(0 * NDOF + c) * TWp + io]);
          if (p.flt.two) f2[c] = double(fbuf[(1 * NDOF + c) * TWp + io]);
        }
        fault_node_update(p.flt, I, it, f1, f2);
      }
      __syncthreads();
    }

    // ---- seismograms of this CTA's receivers completed in this batch ----
    if (nrec_here && it % p.rec_isamp == 0 && it / p.rec_isamp < p.rec_nsamp) {
      const int s = it / p.rec_isamp;
      const int r0 = p.rec_tile_start[cta];
      for (int q = tid; q < nrec_here * NDOF; q += kStripThreads) {
        const int r = p.rec_ids[r0 + q % nrec_here], c = q / nrec_here;
        double val;
        if (p.rec_npts == 1) {  // at a node: D, V or A
          const int I = p.rec_I[r], J = p.rec_J[r];
          const int jj = J - Jlo;
          if (jj < 0 || jj >= nr || s_stat[jj] != 1) continue;
          // displacement after the step: the predictor plus the corrector
          const real dp = hht ? p.Dcur[c * p.plane + (long long)J * p.pitch + I]
                              : sD[c * PS + jj * TWp + xo + (I - Ia)];
          val = p.rec_field == 'D'
                    ? (newmark && p.cb != real(0)
                           ? double(dp + p.cb * p.Anext[c * p.plane + (long long)J * p.pitch + I])
                           : double(dp))
                : p.rec_field == 'V' ? double(p.Vnext[c * p.plane + (long long)J * p.pitch + I])
                                     : double(p.Anext[c * p.plane + (long long)J * p.pitch + I]);
        } else {  // interpolated displacement over an element of this batch
          const int *RI = p.rec_I + (size_t)r * p.rec_npts, *RJ = p.rec_J + (size_t)r * p.rec_npts;
          if (RJ[0] < J0own || RJ[0] < Jlo || RJ[p.rec_npts - 1] >= Jlo + nr) continue;
          const double *W = p.rec_w + (size_t)r * p.rec_npts;
          const real *pl = sD + c * PS + xo - Ia - Jlo * TWp;
          val = W[0] * double(pl[RJ[0] * TWp + RI[0]]);
          for (int k = 1; k < p.rec_npts; ++k) val = val + W[k] * double(pl[RJ[k] * TWp + RI[k]]);
        }
        p.sis[s + (size_t)p.rec_nsamp * (r + (size_t)p.rec_nrec * c)] = val;
      }
    }
    __syncthreads();  // the stage, the scratch areas and the row tables are free again
    if (NST == 2 && b + 2 < nb) issue(b + 2);
  }

  return true;
}

// the last CTA to finish a step advances the step counter
__device__ __forceinline__ void strip_step_done(int *step, unsigned *done, int it) {
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned prev = atomicAdd(done, 1u);
    if (prev == gridDim.x * gridDim.y - 1) {
      *done = 0u;
      __threadfence();
      *step = it;
    }
  }
}

__device__ __forceinline__ void strip_init_bars(uint64_t *bar) {
  if (threadIdx.x == 0) {
    for (int k = 0; k < kMaxStages; ++k) mbar_init(&bar[k], 1);
    mbar_fence_init();
  }
  __syncthreads();
}

// one problem: CTA (x, y) is strip x of chunk y
template <typename real, int N, int NDOF, int MAT, bool FAST>
__global__ void __launch_bounds__(kStripThreads, StripOcc<real, NDOF>::kMinBlocks)
    strip_step_kernel(const __grid_constant__ BulkParams<real, N> p) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar[kMaxStages];
  strip_init_bars(bar);
  uint32_t ph[kMaxStages] = {0u, 0u, 0u};
  const int it = *p.step + 1;  // the step this launch computes
  const int chunk = (blockIdx.y + p.chunk_shift) % gridDim.y;
  if (!strip_unit<real, N, NDOF, MAT, FAST>(p, p.H, p.w, blockIdx.x, chunk, gridDim.x, it, bar, ph, smem_raw))
    return;
  strip_step_done(p.step, p.done, it);
}

// Many independent problems of one NGLL / dof count / precision / material
// layout advanced by one launch: a persistent grid walks the work units
// (problem, strip, chunk, strips per chunk row), copying each problem's
// parameters into shared memory when it changes.
template <typename real, int N>
struct BatchParams {
  real H[N * N], w[N];
  const BulkParams<real, N> *sims;  // this step's parameters of every problem
  const int4 *units;                // (problem, strip, chunk, strips per chunk row)
  int nunits;
  int *step;                        // completed steps of the batch
  unsigned *done;                   // CTA completion counter
};

template <typename real, int N, int NDOF, int MAT, bool FAST>
__global__ void __launch_bounds__(kStripThreads, StripOcc<real, NDOF>::kMinBlocks)
    strip_batch_kernel(const __grid_constant__ BatchParams<real, N> bp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ __align__(8) uint64_t bar[kMaxStages];
  __shared__ __align__(16) BulkParams<real, N> sp;
  strip_init_bars(bar);
  uint32_t ph[kMaxStages] = {0u, 0u, 0u};
  const int it = *bp.step + 1;
  int cur = -1;
  for (int u = blockIdx.x; u < bp.nunits; u += gridDim.x) {
    const int4 wu = bp.units[u];
    if (wu.x != cur) {
      __syncthreads();
      const int *src = reinterpret_cast<const int *>(bp.sims + wu.x);
      int *dst = reinterpret_cast<int *>(&sp);
      for (int k = threadIdx.x; k < int(sizeof(sp) / sizeof(int)); k += kStripThreads) dst[k] = src[k];
      __syncthreads();
      cur = wu.x;
    }
    if (!strip_unit<real, N, NDOF, MAT, FAST>(sp, bp.H, bp.w, wu.y, wu.z, wu.w, it, bar, ph, smem_raw)) return;
  }
  strip_step_done(bp.step, bp.done, it);
}

}  // namespace sem2d

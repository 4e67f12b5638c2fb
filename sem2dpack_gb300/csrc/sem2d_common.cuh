// sem2d_common.cuh -- device layout and launch parameters shared by the
// kernels and the host side of the GB300 time step.
//
// Device layout.  The Cartesian mesh of SEM2DPACK (mesh_cartesian.f90) is a
// structured lattice of GLL nodes: LX = nx*(N-1)+1 columns and LZ rows, with
// one extra row where a fault splits the mesh (mesh_structured.f90:78-80).
// Element (ex,ez) covers columns ex*(N-1) .. ex*(N-1)+N-1 and rows
// row0[ez] .. row0[ez]+N-1.  Every nodal field is stored as one plane per
// degree of freedom, row-major with a padded row pitch:
//     field[c*plane + J*pitch + I].
// The reference's global numbering (ibool, RCM element order) is mapped to
// this lattice once at upload and back at download.
#pragma once

#include <cstdint>

namespace sem2d {

constexpr int kMaxN = 9;          // largest NGLL compiled
constexpr int kMaxSrc = 64;

// material layouts: lattice planes (continuous material), one value per
// element GLL point, or one value per element (homogeneous elements); the
// element layouts are in structured element order (ez*nx + ex)
constexpr int kMatNode = 0;
constexpr int kMatPoint = 1;
constexpr int kMatElement = 2;
// a grid that is not flat: the element phase reads the general coefficients
// a1..a10 (P-SV) or a1..a3 (SH) of every element GLL point (gen), which
// hold the moduli, the inverse Jacobian and the weights together
constexpr int kMatGeneral = 3;

// Parameters of the per-node fault update (FP64 fault state).
template <typename real>
struct FaultParams {
  int ndof, LX, pitch;
  long long plane;
  int nflt, two, jf1, jf2;
  const real *f_flt;
  const real *Dcur;
  real *Dnext, *Vnext, *Anext;
  // FP64 shadow of the fault-node fields: [(side*ndof + c)*nflt + k]
  double *d64, *v64, *a64;
  const double *rm;     // [(side*ndof + c)*nflt + k] inverse mass
  const double *n1;     // (nflt,2)
  const double *B;      // [nflt]
  const double *invM1, *invM2, *Z;  // (nflt,ndof)
  const double *T0;     // (nflt,2)
  const double *coh;
  double coefA2V, coefA2D;
  int opening, friction, swf_kind, swf_healing, rsf_kind, normal_kind;
  double normal_V, normal_coef;
  const double *swf_dc, *swf_mus, *swf_mud, *swf_p, *swf_alpha;
  const double *rsf_dc, *rsf_mus, *rsf_a, *rsf_b, *rsf_vstar, *rsf_vc, *rsf_Tc, *rsf_coeft;
  // time weakening (0 = none), alone when friction == 3
  int twf_kind;
  double twf_mus, twf_mud, twf_mu0, twf_X, twf_Z, twf_V, twf_L, twf_T, twf_Dc;
  const double *fxz;    // (2,nflt) positions of the side-1 nodes
  // state
  double *D, *V, *T, *Tstick, *MU, *theta, *sigma;
  // potency terms of this step per node pair, [q*nflt + k] (null: not kept)
  double *pot;
  // outputs: series[(q + onx*(rec + 6*sample))]
  int oit, oitd, oix1, oixd, onx, nsamp;
  double *series;
  // time scheme
  int scheme;
  double dt, cv, cpred, cd2;
  double cb;            // Newmark corrector beta dt^2
  double tshift;        // time of the boundary terms minus it dt: (alpha-1) dt
  const unsigned char *dir_zero;  // [k] bits side*2+c: force zeroed after the fault, or null
  int *step;            // incremented by the last block (stand-alone kernel)
  unsigned int *done;   // block completion counter (reset by the last block)
  int *error;           // sticky device error flag (SEM2D_E_*)
  int nr_maxit;         // iteration cap of the rate-and-state Newton solver
};

// Parameters of the fused element-force + assembly + update kernel.
template <typename real, int N>
struct BulkParams {
  // lattice
  int LX, LZ, pitch;
  long long plane;
  int nx, nz;
  const int *row0;  // [nz+1]; row0[nz] = LZ
  int TX;           // element columns per CTA tile
  const int *ztile; // [ntz+1] element-row boundaries of the tile rows
  // GLL operator
  real H[N * N];    // H(i,j) = h'_i(x_j), column-major
  real w[N];
  // state (ping-pong buffers chosen by the host)
  const real *Dcur;
  real *Dnext;
  const real *Vcur;
  real *Vnext;
  const real *Acur;
  real *Anext;      // null unless accelerations are kept
  const real *Fcur; // march kernel, force state: elastic force of the step before
  real *Fnext;      //   and of this step (null with the displacement state)
  // material
  int mat_iso;      // isotropic: planes (la, mu) [P-SV] or (mu) [SH]
  const real *mat[4];
  int mat_elem;     // material layout: kMatNode, kMatPoint, kMatElement or kMatGeneral
  const real *gen;  // kMatGeneral: a_k at [k*gen_stride + (ez*nx + ex)*N*N + i + N*j]
  long long gen_stride;
  const real *kveta;// per element GLL point or null
  const real *rmass;// lattice plane (both dofs equal away from the perimeter)
  // element geometry (rectilinear): per column / per row
  const real *xix;    // dxi/dx  of element column
  const real *etaz;   // deta/dz of element row
  const real *dxdxi;  // dx/dxi  of element column
  const real *dzdeta; // dz/deta of element row
  // perimeter table: slot -> rmass(dof), dashpots Ca(dof), Cb(dof)
  const real *per_rm, *per_Ca, *per_Cb;
  const real *per_kd;     // Stacey P3 forces [c*nslot + slot] of this step, or null
  const int *per_dir;     // zero-Dirichlet bits c by perimeter slot, or null
  real *perio_f;          // periodic columns I = 0, LX-1: raw forces [(c*LZ + J)*2 + side], or null
  int perio_tb;           // periodic rows J = 0, LZ-1 instead: [(c*LX + I)*2 + side]
  const real *per_bf;     // incident wave and Neumann tractions of this step [c*nslot + slot], or null
  // fault rows (lattice rows of side 1 and side 2, -1 if none); a tile row
  // always holds both rows, so the owning CTA finishes the fault nodes
  int jf1, jf2;
  int has_fault;
  FaultParams<real> flt;
  real *fault_force;      // march kernel: forces of the fault rows [(side*ndof + c)*nflt + I]
  // point sources
  int nsrc;
  const int *src_I, *src_J;
  const double *src_amp;  // [(s*ndof + c)*(nt+1) + it]
  int nt;
  int *step;              // completed steps (device counter, bumped by the last CTA)
  unsigned int *done;     // CTA completion counter
  // receivers sampled by the CTA that owns them: node receivers (D, V or A)
  // and interpolated receivers of D
  int rec_nsamp, rec_isamp, rec_nrec, rec_npts;
  char rec_field;
  const int *rec_tile_start;  // [ntiles+1] into rec_ids
  const int *rec_ids;         // receiver numbers grouped by tile
  const int *rec_I, *rec_J;   // [r*npts + q] lattice position
  const double *rec_w;        // [r*npts + q] weight
  double *sis;
  // time scheme
  int scheme;             // 0 leapfrog, 1 Newmark, 2 HHT-alpha
  real dt, cv, cpred, cd2;// cv: coef a->v, cpred: (1-gamma)dt, cd2: (0.5-beta)dt^2
  real cb;                // Newmark corrector beta dt^2 (0: leapfrog or beta = 0)
  real cal, cpa;          // scheme 2 (HHT-alpha): 1 - alpha, and alpha (1 - gamma) dt, the
                          // acceleration coefficient of v_alpha (cpred otherwise)
  int kd2;
  real width;             // 2.5D seismogenic width W, 0 for a 2D problem
  int nmat;               // material planes (node layout) or arrays (element layout)
  int has_kv;             // Kelvin-Voigt viscosity present
  int nplanes;            // lattice planes staged per batch (strip_planes)
  int *error;             // sticky device error flag (SEM2D_E_*)
  int spin_limit;         // polls of a stage's mbarrier before the step gives up
  int chunk_shift;        // chunk of CTA row y is (y + chunk_shift) % rows: the
                          // fault's chunk (long FP64 work) is scheduled first
};

// Perimeter slot of lattice node (I,J): bottom row, top row, left column,
// right column (corners belong to the rows).
__host__ __device__ inline int perimeter_slot(int I, int J, int LX, int LZ) {
  if (J == 0) return I;
  if (J == LZ - 1) return LX + I;
  if (I == 0) return 2 * LX + (J - 1);
  if (I == LX - 1) return 2 * LX + (LZ - 2) + (J - 1);
  return -1;
}
__host__ __device__ inline int perimeter_slots(int LX, int LZ) { return 2 * LX + 2 * (LZ - 2); }

template <typename real>
struct RecParams {
  int nrec, ndof, nsamp, isamp, npts;  // npts = 1 (at node) or N*N
  long long plane;
  const int *lat;       // [r*npts + q] lattice offset J*pitch+I
  const double *w;      // [r*npts + q] weights (1 at node)
  const real *field;
  const real *acc;      // displacement with the Newmark corrector: field + cb * acc
  real cb;
  double *sis;          // sis(nsamp,nrec,ndof)
  const int *step;
};

}  // namespace sem2d

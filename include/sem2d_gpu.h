/*
 * sem2d_gpu.h -- C-ABI of the GB300 spectral-element time step.
 *
 * This is the drop-in boundary for SEM2DPACK's explicit time step.  In the
 * reference the step is the Fortran call chain
 *     main.f90:54        call solve(pb)
 *     solver.f90:140-161 solve_leapfrog  /  solver.f90:42-83 solve_Newmark
 *     solver.f90:273-316 compute_Fint  (gather, MAT_Fint, scatter-add)
 *     src_gen.f90:290    SO_add        (point forces x Ricker)
 *     bc_gen.f90:256     BC_apply      (absorbing, then dynamic fault)
 *     receivers.f90:309  REC_store     (seismogram sampling)
 *     bc_dynflt.f90:751  BC_DYNFLT_write (fault time series)
 * over the state held in problem_type (problem_class.f90:19-46).
 *
 * sem2d_gpu_create() receives the arrays exactly as the reference's
 * init_main (init.f90:16-131) leaves them: Fortran column-major order,
 * 1-based node numbers, the inverted mass already folded with the absorbing
 * dashpots, the fault impedance Z and the snapshots invM1/invM2.  The
 * library deep-copies everything to the device and keeps its own layout.
 *
 * All functions return 0 on success and a negative SEM2D_E_* code on
 * failure; sem2d_gpu_last_error() then returns a message (the Fortran side
 * maps a non-zero status to IO_abort, stdio.f90:205-213).  A handle is used
 * by one host thread at a time and owns one CUDA stream.
 */
#ifndef SEM2D_GPU_H
#define SEM2D_GPU_H

#ifdef __cplusplus
extern "C" {
#endif

#define SEM2D_GPU_ABI_VERSION 1

/* status codes */
#define SEM2D_OK 0
#define SEM2D_E_ARG (-1)         /* bad argument or inconsistent sizes        */
#define SEM2D_E_CUDA (-2)        /* CUDA runtime error                        */
#define SEM2D_E_UNSUPPORTED (-3) /* mesh or option outside the GPU path      */
#define SEM2D_E_NR (-4)          /* rate-and-state Newton solver did not converge */
#define SEM2D_E_NAN (-5)         /* non-finite field value detected           */
#define SEM2D_E_STATE (-6)       /* call out of sequence                      */
#define SEM2D_E_NOMEM (-7)       /* device or host allocation failed          */
#define SEM2D_E_TIMEOUT (-8)     /* a bounded device wait expired             */

/* time schemes (time.f90:122-315) */
#define SEM2D_TIME_LEAPFROG 0
#define SEM2D_TIME_NEWMARK 1
#define SEM2D_TIME_HHT 2 /* explicit HHT-alpha (solver.f90:89-131)               */

/* friction laws (bc_dynflt.f90:200-213) */
#define SEM2D_FRICTION_SWF 1
#define SEM2D_FRICTION_RSF 2
#define SEM2D_FRICTION_TWF 3 /* time weakening alone (bc_dynflt.f90:656-657) */

/* arithmetic of the bulk fields */
#define SEM2D_PRECISION_FP64 0  /* everything in FP64                       */
#define SEM2D_PRECISION_MIXED 1 /* FP32 fields/forces, FP64 fault state     */

/* source time functions, numbered as stf_gen.f90:23-29 (the reference's
 * BUTTERWORTH aborts as not implemented, butterworth_filter.f90:27-43,
 * and has no number here) */
#define SEM2D_STF_NONE 0
#define SEM2D_STF_RICKER 1
#define SEM2D_STF_TAB 3
#define SEM2D_STF_HARMONIC 4
#define SEM2D_STF_BRUNE 5
#define SEM2D_STF_GAUSSIAN 6
#define SEM2D_STF_USER 7

/* incident plane wave phases (&SRC_WAVE phase, src_wave.f90:56-110) */
#define SEM2D_WAVE_NONE 0
#define SEM2D_WAVE_P 1
#define SEM2D_WAVE_S 2 /* also the SH wave of ndof = 1                  */

/* A source time function (STF_get, stf_gen.f90:99-121), with the values
 * as the reference holds them (the parameters that &STF_GAUSSIAN,
 * &STF_HARMONIC and &STF_USER read into REAL variables are already
 * rounded to FP32 by the caller):
 *   RICKER    -ampli (1 - 2 a) exp(-a), a = (pi f0 (t - onset))^2
 *             (stf_ricker.f90:89-103)
 *   GAUSSIAN  ampli exp(-a)                         (stf_gaussian.f90:76-86)
 *   BRUNE     ampli (1 - (1 + b) exp(-b)), b = 2 pi f0 max(t, 0)
 *             (f0 is the corner frequency fc, stf_brune.f90:73-83)
 *   HARMONIC  ampli sin(2 pi f0 t)                  (stf_harmonic.f90:68-77)
 *   USER      ampli sin(t - onset) + par1 (t - onset)^2 (stf_user.f90:110-122)
 *   TAB       cubic spline through (tab_t, tab_v) with zero end slopes,
 *             t clamped to [tab_t[0], tab_t[ntab-1]]
 *             (stf_tabulated.f90:52-95, utils.f90:652-734) */
typedef struct sem2d_stf {
  int kind; /* SEM2D_STF_*                                                */
  int ntab; /* TAB: rows, >= 2, tab_t increasing                          */
  double f0, onset, ampli, par1, par2;
  const double *tab_t, *tab_v;
} sem2d_stf;

typedef struct sem2d_problem_desc {
  /* ---- sizes (spec_grid.f90:49-64, fields.f90:7-11) ---- */
  int ngll;  /* GLL nodes per element edge                        */
  int ndof;  /* 1 = SH (antiplane), 2 = P-SV (in-plane)           */
  int nelem; /* number of spectral elements                       */
  int npoin; /* number of global GLL nodes                        */

  /* ---- grid ---- */
  const int *ibool;      /* ibool(ngll,ngll,nelem), 1-based global node      */
  const double *coord;   /* coord(2,npoin)                                   */
  const double *hprime;  /* hprime(ngll,ngll), H(i,j) = h'_i(xgll(j))        */
  const double *wgll;    /* wgll(ngll)                                       */

  /* ---- elastic moduli at every element GLL point, (ngll,ngll,nelem) ----
   * mat_elastic.f90:307-321: isotropic -> Kx=Kz=lambda+2mu, la=lambda,
   * mu=mux=mu; VTI -> Kx=c11, Kz=c33, la=c13, mu=c55, mux=c66.          */
  const double *Kx, *Kz, *la, *mu, *mux;
  /* Kelvin-Voigt viscosity eta (already multiplied by dt when ETAxDT),
   * (ngll,ngll,nelem); NULL when no element is Kelvin-Voigt
   * (mat_kelvin_voigt.f90:117-151).                                     */
  const double *kv_eta;
  /* 1 selects the NGLL=5 specialised kernel ELAST_KD2_* of the reference
   * (mat_elastic.f90:589-641), whose flat P-SV shear term uses a4 for both
   * derivatives; 0 selects ELAST_KD1_* (mat_elastic.f90:464-518).       */
  int kd2_form;

  /* ---- inverted mass rmass(npoin,ndof), absorbing fold included ---- */
  const double *rmass;

  /* ---- absorbing boundaries (bc_abso.f90:115-336), one entry per
   * (boundary, node); a node on two boundaries appears twice.          */
  int nabs;
  const int *abs_node;  /* [nabs], 1-based                                  */
  const double *abs_C;  /* abs_C(nabs,ndof) dashpot rho*c*w*|J1D|           */

  /* ---- time scheme (time.f90) ---- */
  int time_scheme; /* SEM2D_TIME_*                                          */
  double dt;
  double beta, gamma; /* Newmark parameters (ignored by leapfrog)          */
  int nt;             /* total number of steps the caller intends to run    */

  /* ---- point-force sources with a Ricker time function
   * (src_gen.f90:290-317, src_force.f90:77-92, stf_ricker.f90:89-103) */
  int nsrc;
  const int *src_node;      /* [nsrc], 1-based                               */
  const double *src_dir;    /* src_dir(2,nsrc): (-sin a, cos a); SH uses 1   */
  const double *src_f0;     /* [nsrc] Ricker centre frequency               */
  const double *src_t0;     /* [nsrc] Ricker onset                          */
  const double *src_ampli;  /* [nsrc] Ricker amplitude                      */
  const double *src_relamp; /* [nsrc] relative amplitude (file column 4) or NULL */
  const double *src_tdelay; /* [nsrc] time delay                            */

  /* ---- receivers (receivers.f90:231-344) ---- */
  int nrec;
  char rec_field;          /* 'D', 'V' or 'A'                                */
  int rec_isamp;           /* sampling stride in steps                       */
  int rec_nsamp;           /* samples stored = nt/isamp + 1                  */
  const int *rec_node;     /* [nrec] 1-based node (AtNode) or NULL           */
  const int *rec_elem;     /* [nrec] 1-based element (interpolated) or NULL  */
  const double *rec_interp;/* interp(ngll*ngll,nrec) Lagrange weights        */

  /* ---- dynamic fault (bc_dynflt.f90:231-778); nflt = 0 if none ---- */
  int nflt;
  const int *flt_node1;    /* [nflt], 1-based, side 1                        */
  const int *flt_node2;    /* [nflt], 1-based, side 2; NULL = one-sided      */
  const double *flt_n1;    /* n1(nflt,2) normal of side 1                    */
  const double *flt_B;     /* B(nflt) boundary weights                       */
  const double *flt_invM1; /* invM1(nflt,ndof)                               */
  const double *flt_invM2; /* invM2(nflt,ndof) or NULL                       */
  const double *flt_Z;     /* Z(nflt,ndof) impedance                         */
  const double *flt_T0;    /* T0(nflt,2) initial (tangent, normal) traction  */
  const double *flt_cohesion; /* [nflt]                                      */
  double flt_coefA2V, flt_coefA2D;
  int flt_opening;         /* allow opening (T_n <= 0)                       */
  int flt_friction;        /* SEM2D_FRICTION_*                               */
  int swf_kind;            /* 1 linear, 2 exponential, 3 power law           */
  int swf_healing;
  const double *swf_dc, *swf_mus, *swf_mud, *swf_p, *swf_alpha; /* [nflt] */
  int rsf_kind;            /* 1..4 (bc_dynflt_rsf.f90:40-48)                 */
  const double *rsf_dc, *rsf_mus, *rsf_a, *rsf_b, *rsf_vstar, *rsf_vc;
  const double *rsf_theta; /* [nflt] initial state                           */
  const double *flt_V0;    /* [nflt] initial slip rate (RSF) or NULL         */
  int normal_kind;         /* 0..3 (bc_dynflt_normal.f90)                    */
  double normal_T, normal_L, normal_V;
  /* output sampling (bc_dynflt.f90:436-440): first step oit, stride oitd,
   * nodes oix1..oixn step oixd (1-based), flt_nsamp samples              */
  int flt_oit, flt_oitd, flt_oix1, flt_oixn, flt_oixd, flt_nsamp;

  /* ---- options ---- */
  int precision; /* SEM2D_PRECISION_*                                      */

  /* ---- 2.5D crustal-plane term f -= beta d, beta = dvol mu (pi/W)^2
   * (SH) or dvol mu (pi (1-nu)/W)^2 (P-SV), nu = lambda/(lambda+mu)/2
   * (mat_elastic.f90:363-383, 447-459; mat_gen.f90:440).  width is W of
   * &GENERAL; width <= 0 (the reference's huge(1d0)) is a 2D problem.
   * Isotropic materials only.                                           */
  double width;

  /* ---- time-weakening friction (bc_dynflt_twf.f90:117-184), alone
   * (flt_friction = SEM2D_FRICTION_TWF) or superimposed on SWF/RSF as
   * mu = min(mu, mu_twf) (bc_dynflt.f90:405-412, 632, 653-657).
   * twf_kind 0 = none, 1..3 = kind of &BC_DYNFLT_TWF; the node positions
   * are those of flt_node1 (bc_dynflt.f90:302).                         */
  int twf_kind;
  double twf_mus, twf_mud, twf_mu0, twf_X, twf_Z, twf_V, twf_L, twf_T, twf_Dc;

  /* ---- density at every element GLL point (ngll,ngll,nelem) ---- */
  const double *rho;
  /* 1 prepares the handle for sem2d_gpu_adjoint (gradients with respect
   * to density and wave speeds at every node, mat_elastic.f90:189-321
   * defines the moduli from rho, cp, cs): rho is required and the material
   * must be continuous at nodes. */
  int adjoint;
  /* 1 records the fault potency of the displacement and the velocity at
   * every step (BC_DYNFLT_potency, bc_dynflt.f90:757,832-855), read with
   * sem2d_gpu_get_fault_potency.  Single problems only (not in a batch). */
  int flt_potency;

  /* ---- Stacey P3 absorbing terms (BC_ABSO_init bc_abso.f90:174-218,
   * BC_ABSO_apply :321-334) of the P-SV sides with stacey=T, one entry t
   * per (boundary element, edge point k).  The force at node
   * stacey_node[t] receives, for each component c,
   *   - stacey_K[t + nstacey*c] * sum_l hprime(l, k_t) D(stacey_edge[l + ngll*t], c)
   * with the element edge's nodes in the traversal order of SE_inquire
   * (spec_grid.f90:876-881): counter-clockwise around the element, so the
   * sum is the derivative along that direction. */
  int nstacey;
  const int *stacey_node;  /* [nstacey], 1-based                            */
  const int *stacey_k;     /* [nstacey], edge point 0..ngll-1               */
  const int *stacey_edge;  /* [ngll*nstacey], 1-based                       */
  const double *stacey_K;  /* stacey_K(nstacey, 2)                          */

  /* ---- zero-Dirichlet components of &BC_DIRNEU sides (bc_DIRNEU_apply,
   * bc_dirneu.f90:148-169; traction time functions are not included): the
   * force component dir_comp[k] at node dir_node[k] is set to zero after
   * the absorbing terms (bc_gen.f90:271-281).  dir_after_fault[k] = 1 when
   * the block follows the fault's in &BC_DEF order: at a node the two
   * share, the zero then overrides the fault traction. */
  int ndir;
  const int *dir_node;        /* [ndir], 1-based                            */
  const int *dir_comp;        /* [ndir], 0 horizontal (SH: the only one), 1 vertical */
  const int *dir_after_fault; /* [ndir]                                     */

  /* HHT-alpha (SEM2D_TIME_HHT): the forces, sources and boundary terms of
   * a step are evaluated at d_alpha = alpha d_pred + (1-alpha) d_n,
   * v_alpha likewise, and t + (alpha-1) dt (solve_HHT_alpha,
   * solver.f90:89-131); beta and gamma hold the Newmark parameters the
   * scheme derives from alpha and rho (time.f90:222-240).  1 otherwise. */
  double alpha;

  /* ---- periodic sides (&BC_DEF kind='PERIOD', bc_periodic.f90:42-104):
   * node pairs (master, slave) whose forces are summed before the other
   * boundary terms and shared (BC_PERIO_set_field, :77-88); rmass already
   * holds the summed mass. */
  int nperio;
  const int *perio_master; /* [nperio], 1-based                             */
  const int *perio_slave;  /* [nperio], 1-based                             */

  /* ---- run-time checks ----
   * Iteration cap of the rate-and-state Newton solver (nr_solver,
   * bc_dynflt_rsf.f90:372 uses 200); 0 selects 200.  A node that exceeds it
   * makes the run fail with SEM2D_E_NR where the reference calls IO_abort
   * (bc_dynflt_rsf.f90:461-466). */
  int flt_nr_maxit;
  /* Every info_every steps (&GENERAL itInfo, default 100: input.f90:95,122)
   * the library takes max|veloc| and max|displ| over the nodes, as the
   * reference prints them (main.f90:73-76), and fails the run with
   * SEM2D_E_NAN when either is not finite; 0 selects 100, a negative value
   * switches the check off.  sem2d_gpu_get_info returns the last values. */
  int info_every;

  /* ---- time function of the point sources (SO_add, src_gen.f90:290-317):
   * NULL keeps the Ricker of src_f0, src_t0, src_ampli; otherwise source s
   * adds src_relamp[s] * STF_get(src_stf, t - src_tdelay[s]) and src_f0,
   * src_t0, src_ampli are not read. */
  const sem2d_stf *src_stf;

  /* ---- incident plane wave (src_wave.f90:128-224, SO_WAVE_get_VT
   * src_gen.f90:322-339), entering across the absorbing entries with
   * abs_wave[k] = 1 (let_wave on a flat side, bc_abso.f90:245-256).  Entry k
   * at node x receives (BC_ABSO_apply, bc_abso.f90:299-306)
   *     + C_k Vin + B_k Tin,   Vin, Tin = STF_get(wave_stf, phase) (P, T(n_k))
   * with phase = t - (x - wave_ref).k/c - wave_tdelay, k = (-sin a, cos a)
   * for the angle a, c = wave_cp (P) or wave_cs (S, SH), the polarisation
   * P = k (P), (cos a, sin a) (S), 1 (SH), and the traction per unit
   * amplitude T(n) = -(lambda (k.P) n + mu ((P.n) k + (k.n) P)) / c
   * (SH: -mu (k.n) / cs).  The material values are those of the reference
   * point (WAVE_init, src_wave.f90:128-180). */
  int wave_phase;         /* SEM2D_WAVE_*                                  */
  double wave_angle;      /* degrees, in [-180, 180]                       */
  double wave_ref[2];     /* reference point (x, z)                        */
  double wave_cp, wave_cs, wave_mu, wave_lambda;
  double wave_tdelay;
  const sem2d_stf *wave_stf;
  const double *abs_B;    /* [nabs] boundary weights w |J1D| (spec_grid.f90:961-1011) */
  const double *abs_n;    /* abs_n(nabs,2) outward unit normal              */
  const int *abs_wave;    /* [nabs] 1 where the wave enters, or NULL       */

  /* ---- time-dependent Neumann tractions of &BC_DIRNEU hstf / vstf
   * (bc_DIRNEU_apply, bc_dirneu.f90:148-169): force component neu_comp[k]
   * at node neu_node[k] receives neu_B[k] * STF_get(neu_stfs[neu_stf[k]], t).
   * A (node, component) may not also be a zero-Dirichlet entry. */
  int nneu;
  const int *neu_node;    /* [nneu], 1-based                                */
  const int *neu_comp;    /* [nneu], 0 horizontal (SH: the only one), 1 vertical */
  const double *neu_B;    /* [nneu] boundary weights                        */
  const int *neu_stf;     /* [nneu] index into neu_stfs                     */
  int nneu_stf;
  const sem2d_stf *neu_stfs;

  /* ---- element geometry of a mesh that is not rectilinear (the
   * reference's grid%flat = F, e.g. MESH_LAYERS_build, mesh_layers.f90:338):
   * xjaci(2,2,ngll,ngll,nelem) = [dxi/dx dxi/dz; deta/dx deta/dz] at every
   * element GLL point (SE_InverseJacobian, spec_grid.f90:621-643) and
   * dvol(ngll,ngll,nelem) = wgll(i) wgll(j) det J (SE_VolumeWeights,
   * :590-602).  The element forces then take the general coefficients
   * (nelast = 10 in P-SV, 3 in SH: MAT_ELAST_init_a, mat_elastic.f90:
   * 290-360, and ELAST_KD1/KD2, :464-518, 589-641).  NULL: a rectilinear
   * mesh, whose geometry follows from coord (nelast = 6 or 2). */
  const double *xjaci, *dvol;
} sem2d_problem_desc;

typedef struct sem2d_handle sem2d_handle;

/* Library ABI version (SEM2D_GPU_ABI_VERSION). */
int sem2d_gpu_version(void);

/* Number of visible CUDA devices, or a negative status. */
int sem2d_gpu_device_count(void);

/* Replaces the start of the time loop, init.f90:16-131 -> main.f90:51:
 * uploads the problem and records the step-0 outputs (main.f90:35,
 * bc_gen.f90:247).  *out receives a new handle. */
int sem2d_gpu_create(const sem2d_problem_desc *desc, sem2d_handle **out);

/* Many independent problems advanced together: one launch per time step
 * walks the work units (strip x chunk) of all of them.  The reference runs
 * one problem per process; this replaces nsim runs of init_main + the time
 * loop (main.f90:16-96) with one handle.  Every member must share NGLL,
 * ndof, precision, time scheme, nt and material layout (homogeneous
 * elements, GLL-point values or continuous node values); mesh sizes,
 * materials, sources and receivers may differ.  *out receives the batch;
 * step / step_timed / sync / reset / destroy act on all members. */
int sem2d_gpu_create_batch(const sem2d_problem_desc *descs, int nsim, sem2d_handle **out);
/* The same batch built one member at a time, so that a caller holds one
 * problem description at a time: open an empty batch, add members (each is
 * uploaded at once), close it (units and parameter blocks are built). */
int sem2d_gpu_batch_open(sem2d_handle **out);
int sem2d_gpu_batch_add(sem2d_handle *h, const sem2d_problem_desc *desc);
/* n members at once, set up on up to SEM2D_HOST_THREADS host threads
 * (default: the hardware threads, at most 16) and added in the order
 * given; the descriptions are read during the call only.  On failure no
 * member of the call is added.  sem2d_gpu_create_batch adds its members
 * this way. */
int sem2d_gpu_batch_add_many(sem2d_handle *h, const sem2d_problem_desc *descs, int n);
int sem2d_gpu_batch_close(sem2d_handle *h);
/* Number of members of a batch (0 for a single problem). */
int sem2d_gpu_batch_size(sem2d_handle *h);
/* Member i of a batch (owned by the batch, valid until it is destroyed),
 * for the get_* calls; NULL if out of range. */
sem2d_handle *sem2d_gpu_batch_member(sem2d_handle *h, int i);

/* ---- gradient of a seismogram misfit (no counterpart in the reference:
 * SEM2DPACK has no adjoint) ----------------------------------------------
 * For a handle created with desc->adjoint = 1: keep the forward state every
 * `every` steps during the next run from step 0 (every <= 0 disables).
 * Memory: (nt/every + 1) x 2 x ndof lattice planes. */
int sem2d_gpu_checkpoint_every(sem2d_handle *h, int every);
/* After all nt steps with checkpoints: the gradient of a misfit J with
 * respect to density, P and S wave speed at every global node (npoin
 * values each, NULL to skip), given resid = dJ/dsis laid out like the
 * seismograms (rec_nsamp, nrec, ndof).  Discrete adjoint of the leapfrog
 * step (reverse steps of the same element operator, the inverse mass and
 * dashpot terms) with segment-wise recomputation from the checkpoints; the
 * gradient covers the moduli, the mass and the absorbing dashpots.  NGLL=5,
 * isotropic material continuous at nodes, leapfrog, no fault, Kelvin-Voigt
 * or 2.5D term, receivers at nodes recording V or D.  Device scratch of
 * the call (3 x every + 8 lattice planes of ndof fields and a few more)
 * comes from a stream-ordered pool of the library that keeps the memory
 * reserved for later calls of the process. */
int sem2d_gpu_adjoint(sem2d_handle *h, const double *resid, double *grad_rho, double *grad_vp,
                      double *grad_vs);

/* Replaces nsteps iterations of `do it=1,nt; call solve(pb); REC_store;
 * BC_write` (main.f90:51-96).  Asynchronous on the handle's stream; the
 * status of device-side checks is reported by the next call that
 * synchronises (get_* / sync / destroy). */
int sem2d_gpu_step(sem2d_handle *h, int nsteps);

/* Measurement variant of sem2d_gpu_step: runs nsteps steps with direct
 * launches and a CUDA event pair around each kernel on the handle's
 * stream, waits, and stores the summed kernel durations in milliseconds:
 * ms[0] bulk kernel, ms[1] fault kernel (or step-counter kernel), ms[2]
 * receiver kernel.  Results are identical to sem2d_gpu_step. */
int sem2d_gpu_step_timed(sem2d_handle *h, int nsteps, double *ms);

/* The CUDA stream (a cudaStream_t) the handle launches on, so that a
 * caller can order its own work after the steps or record events on it. */
void *sem2d_gpu_stream(sem2d_handle *h);

/* Waits for all queued steps; returns device-side error status. */
int sem2d_gpu_sync(sem2d_handle *h);

/* Steps completed so far. */
int sem2d_gpu_current_step(sem2d_handle *h);

/* Copies displ, veloc, accel (npoin,ndof) in the reference's global
 * numbering into caller buffers; any pointer may be NULL. */
int sem2d_gpu_get_fields(sem2d_handle *h, double *displ, double *veloc,
                         double *accel);

/* Copies seismograms sis(rec_nsamp,nrec,ndof) (receivers.f90:12) as FP64;
 * samples not yet recorded are zero. */
int sem2d_gpu_get_seismograms(sem2d_handle *h, double *sis);

/* Copies the fault time series as FP64, laid out (onx, 6, flt_nsamp) with
 * the 6 records of BC_DYNFLT_write: slip, slip rate, shear traction,
 * normal traction, friction coefficient, T_stick (bc_dynflt.f90:760-767). */
int sem2d_gpu_get_fault(sem2d_handle *h, double *out);

/* Copies the fault potency series of a handle created with
 * desc->flt_potency = 1 (the FltXX_potency_sem2d.tab records of
 * BC_DYNFLT_write, bc_dynflt.f90:757 with BC_DYNFLT_potency :832-855):
 * out[6*it + q], it = 0..nt, q = 0..2 the potency of the displacement
 * (P-SV: p11, p22, p12; SH: p13, p23, 0) and q = 3..5 that of the velocity,
 * after step it (row 0: the initial state).  Rows of steps not yet run are
 * zero. */
int sem2d_gpu_get_fault_potency(sem2d_handle *h, double *out);

/* Strain and stress at every element GLL point from the displacement that
 * sem2d_gpu_get_fields returns, laid out e(ngll,ngll,ndof+1,nelem) in the
 * reference's element order: MAT_strain_PSV/SH (mat_gen.f90:727-774) --
 * P-SV e11, e22, e12; SH e13, e23 -- and MAT_ELAST_stress
 * (mat_elastic.f90:804-862): P-SV sigma11, sigma22, sigma12 (isotropic or
 * VTI), SH sigma13, sigma23.  Either pointer may be NULL.  Single problems
 * (a batch member reads its own). */
int sem2d_gpu_get_strain_stress(sem2d_handle *h, double *strain, double *stress);

/* The progress information of main.f90:73-76: *vmax = max|veloc| and
 * *dmax = max|displ| over all nodes and components at the last multiple
 * of info_every steps (step 0 before the first), and *step = that step.
 * A batch returns the maxima over its members.  Either pointer may be
 * NULL. */
int sem2d_gpu_get_info(sem2d_handle *h, int *step, double *vmax, double *dmax);

/* Current fault state D(nflt,ndof), V(nflt,ndof), T(nflt,2), MU(nflt),
 * state variable theta(nflt) (RSF, else zeros); any pointer may be NULL. */
int sem2d_gpu_get_fault_state(sem2d_handle *h, double *D, double *V,
                              double *T, double *MU, double *theta);

/* Returns the handle to its state right after create (zero fields, step
 * 0, initial fault state); the uploaded problem is kept.  Lets a caller
 * rerun the same problem without a new upload. */
int sem2d_gpu_reset(sem2d_handle *h);

/* Kernels launched by this handle since creation (graph replays count
 * every kernel node). */
long long sem2d_gpu_kernel_launches(sem2d_handle *h);

/* Work unit of the step kernel: a strip of TX element columns and a chunk
 * of (about) TZ element rows.  FP32 problems with NGLL = 5, isotropic
 * material per node or per element, leapfrog and no Kelvin-Voigt or 2.5D
 * term run the one-element-per-thread kernel: a warp per unit, TX = 31
 * (SEM2D_MARCH_CZ=TZ overrides its chunk height, SEM2D_MARCH=0 selects the
 * strip kernel).  Every other problem runs the strip kernel: a CTA per
 * unit (SEM2D_CHUNK=TZ overrides its chunk height).  The environment is
 * read at create time.  The march kernel's shape comes from the tuning
 * cache (SEM2D_TUNE_CACHE) when it holds the class of the problem; else
 * five shapes are timed on the first 85 steps of the first step call that
 * runs at least 85 steps between checks (every shape gives the same
 * results), and the fastest is kept and recorded (SEM2D_AUTOTUNE=0: the
 * analytic shape). */
int sem2d_gpu_tile_shape(sem2d_handle *h, int *tx, int *tz);

/* Releases device memory; h becomes invalid. */
int sem2d_gpu_destroy(sem2d_handle *h);

/* Message of the last failed call on h (or, when h is NULL, of the last
 * failed create or sem2d_gpu_step_noalloc). */
const char *sem2d_gpu_last_error(sem2d_handle *h);

/* ---- stepping caller-owned device arrays without allocating ----------
 *
 * Device lattice layout.  The library stores a Cartesian problem on the
 * structured lattice of GLL nodes: LX = nx*(ngll-1)+1 columns and LZ rows,
 * element row ez starting at lattice row row0[ez] (row0[nz] = LZ).  A nodal
 * field is ndof planes of pitch*LZ values, value (I,J) of dof c at
 * [c*pitch*LZ + J*pitch + I].  Values are double for SEM2D_PRECISION_FP64
 * and float for SEM2D_PRECISION_MIXED.  Rows are fetched with 16-byte bulk
 * copies: pitch times the value size is a multiple of 16 bytes and every
 * device plane starts 16-byte aligned.  The state between steps is the
 * displacement of the next step (the reference's displ + dt*veloc for
 * leapfrog) and the velocity (the reference's veloc). */
typedef struct sem2d_lattice_args {
  int ngll, ndof, precision;
  int nx, nz, LX, LZ, pitch;
  const int *row0;            /* device, [nz+1]                              */
  const double *hprime, *wgll;/* host, H(ngll,ngll) and the GLL weights      */
  void *d, *v;                /* device state, updated in place              */
  const void *rmass;          /* device plane: inverse mass                  */
  const void *per_rm, *per_Ca, *per_Cb; /* device perimeter tables
                                 [c*nslot + s]: inverse mass and the dashpots
                                 of up to two absorbing sides at slot s; node
                                 (I,J) has slot I (J=0), LX+I (J=LZ-1),
                                 2LX+J-1 (I=0), 2LX+LZ-2+J-1 (I=LX-1), and
                                 nslot = 2LX + 2(LZ-2)                        */
  int mat_iso;                /* 1: planes (lambda, mu) [P-SV] or (mu) [SH];
                                 0: (Kx, Kz, lambda, mu) [P-SV] or (mu, mux) */
  const void *mat[4];         /* device material planes                      */
  const void *xix, *etaz, *dxdxi, *dzdeta; /* device, per element column (x)
                                 and row (z): dxi/dx, deta/dz, dx/dxi, dz/deta */
  int nsrc;
  const int *src_I, *src_J;   /* device lattice positions of the sources     */
  const double *src_amp;      /* device ((s*ndof + c)*(nt+1) + it) amplitudes */
  int nt;                     /* last step covered by src_amp                */
  int step0;                  /* steps already done before this call         */
  double dt;
  int kd2_form;
  int *status;                /* device int or NULL: a step that fails on the
                                 device (a bounded wait for its shared-memory
                                 copies that ran out: SEM2D_E_TIMEOUT) stores
                                 its SEM2D_E_* code here; the library never
                                 clears it.  Read it once the stream has
                                 finished.  With NULL such failures go
                                 unreported.                                 */
} sem2d_lattice_args;

/* Advances nsteps leapfrog steps of the elastic bulk (element forces,
 * sources, absorbing dashpots, inverse mass, update) on the caller's device
 * arrays a->d, a->v, queued on `stream` (a cudaStream_t, NULL = default
 * stream), without allocating any device memory.
 *
 * For callers that cannot call cudaMalloc -- code running inside another
 * framework's memory pool (a PyTorch caching allocator that owns all device
 * memory), inside a CUDA graph being captured, or under a fixed memory
 * budget.  This entry point has no counterpart in the reference.  It is the
 * bulk step kernel of sem2d_gpu_step with its scratch (the partner
 * displacement and velocity buffers of the double-buffered update and the
 * step and CTA counters) in one file-scope device array of
 * SEM2D_NOALLOC_SCRATCH_BYTES that every GPU loading the library keeps until
 * the process exits; problems whose partner buffers do not fit are rejected
 * with SEM2D_E_ARG.  The first call on a device looks up that array's
 * address, so make it before any stream capture.  All calls share the one
 * array: calls that overlap on the GPU (other streams, other threads) race
 * and must be ordered by the caller.  NGLL 3, 5, 6 and 9 are taken.  The
 * return value covers the arguments and the launches; failures inside the
 * kernels reach the caller only through a->status.  Messages of rejected
 * calls: sem2d_gpu_last_error(NULL). */
#define SEM2D_NOALLOC_SCRATCH_BYTES (8u << 20)
int sem2d_gpu_step_noalloc(const sem2d_lattice_args *a, int nsteps, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SEM2D_GPU_H */

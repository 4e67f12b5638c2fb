/*
 * sem2d_host.h -- host-side problem builder (the reference's input and
 * initialisation phases for the Cartesian solver path).
 *
 * The reference reads a Par.inp of Fortran NAMELIST blocks (input.f90:12-62)
 * and builds the solver state in init_main (init.f90:16-131).  sem2d_deck
 * carries the values of the blocks this path uses; the builder restates
 *   MESH_CART  / MESH_CART_DOMAIN   mesh_cartesian.f90:86-314
 *   element renumbering (RCM)       mesh_structured.f90:204-269, rcm.f90
 *   GLL numbering, coordinates      spec_grid.f90:149-374
 *   boundary node tables            spec_grid.f90:676-822
 *   materials, CHECK_grid, TIME     mat_gen.f90:204-303, init.f90:145-289,
 *                                   time.f90:323-341
 *   mass, absorbing fold, fault     mat_mass.f90:29-61, bc_abso.f90:115-266,
 *                                   bc_dynflt.f90:231-520
 *   sources, receivers              src_gen.f90:216-262, receivers.f90:168-303
 * and fills a sem2d_problem_desc for sem2d_gpu_create().
 *
 * Spatially variable inputs (the DIST_* blocks of the reference) are given
 * as arrays already evaluated at the GLL points (materials) or at the fault
 * nodes (fault parameters); sem2d_grid_* exposes the coordinates and the
 * boundary node tables needed to evaluate them.
 */
#ifndef SEM2D_HOST_H
#define SEM2D_HOST_H

#include "sem2d_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define SEM2D_MAX_DOMAINS 64
#define SEM2D_MAX_MATS 64
#define SEM2D_MAX_BCS 16
#define SEM2D_MAX_LAYERS 32

/* &MESH_CART_DOMAIN tag, ex, ez (mesh_cartesian.f90:64-79), 1-based */
typedef struct sem2d_domain {
  int tag;
  int ex[2];
  int ez[2];
} sem2d_domain;

/* &MATERIAL tag + &MAT_ELASTIC (+ &MAT_KV) (mat_elastic.f90:69-189) */
typedef struct sem2d_material {
  int tag;
  int aniso;  /* 0: rho, cp, cs;  1: rho, c11, c13, c33, c55, c66       */
  double rho, cp, cs;
  double c11, c13, c33, c55, c66;
  int hetero; /* 1: the values of this tag come from the deck's h_* arrays */
  int kv;     /* Kelvin-Voigt damping present                           */
  double kv_eta;
  int kv_etaxdt; /* eta given in units of dt (ETAxDT, default true)      */
} sem2d_material;

/* &BC_DEF kind, tag(s) (bc_gen.f90:84-186) */
#define SEM2D_BC_ABSORB 1
#define SEM2D_BC_DYNFLT 2
#define SEM2D_BC_DIRNEU 3
#define SEM2D_BC_PERIOD 4 /* tag[0] master side, tag[1] slave side      */
typedef struct sem2d_bc {
  int kind;
  int tag[2];
  int stacey; /* &BC_ABSORB stacey (bc_abso.f90:55-100); P-SV only        */
  int dirichlet; /* &BC_DIRNEU: bit 0 h='D', bit 1 v='D' (bc_dirneu.f90:50-112) */
  int no_wave;   /* &BC_ABSORB let_wave = F: the incident wave of the
                  * sources does not enter across this side (0, the
                  * reference's default let_wave = T, lets it in)        */
  /* &BC_DIRNEU hstf, vstf: time functions of the horizontal and vertical
   * tractions of a Neumann component (kind SEM2D_STF_NONE: none; a
   * Dirichlet component ignores its own, bc_dirneu.f90:70-101)          */
  sem2d_stf hstf, vstf;
} sem2d_bc;

/* Per-node fault inputs of &BC_DYNFLT, &BC_DYNFLT_SWF and &BC_DYNFLT_RSF */
enum {
  SEM2D_FP_TT = 0, SEM2D_FP_TN, SEM2D_FP_SXX, SEM2D_FP_SXY, SEM2D_FP_SXZ,
  SEM2D_FP_SYZ, SEM2D_FP_SZZ, SEM2D_FP_COHESION, SEM2D_FP_V0,
  SEM2D_FP_SWF_DC, SEM2D_FP_SWF_MUS, SEM2D_FP_SWF_MUD, SEM2D_FP_SWF_P,
  SEM2D_FP_SWF_ALPHA,
  SEM2D_FP_RSF_DC, SEM2D_FP_RSF_MUS, SEM2D_FP_RSF_A, SEM2D_FP_RSF_B,
  SEM2D_FP_RSF_VSTAR, SEM2D_FP_RSF_THETA, SEM2D_FP_RSF_VC,
  SEM2D_FP_NPARAM
};

typedef struct sem2d_deck {
  /* &GENERAL (input.f90:101-169) */
  int ngll, ndof;
  double fmax;

  /* &MESH_CART */
  double xlim[2], zlim[2];
  int nelem[2];
  int ezflt;  /* 0 none, -1 middle, k>0 fault above element row k      */
  int fztag, fznz;
  int ndomains;
  sem2d_domain domains[SEM2D_MAX_DOMAINS];

  /* materials */
  int nmats;
  sem2d_material mats[SEM2D_MAX_MATS];
  /* per element GLL point values (ngll,ngll,nelem) for hetero tags */
  const double *h_rho, *h_cp, *h_cs;
  const double *h_c11, *h_c13, *h_c33, *h_c55, *h_c66;
  const double *h_kveta;

  /* boundary conditions in &BC_DEF order (the order matters:
   * bc_gen.f90:229-246) */
  int nbcs;
  sem2d_bc bcs[SEM2D_MAX_BCS];

  /* the dynamic fault (at most one DYNFLT boundary) */
  int flt_friction;   /* SEM2D_FRICTION_SWF or SEM2D_FRICTION_RSF          */
  int swf_kind, swf_healing, rsf_kind;
  int normal_kind;
  double normal_T, normal_L, normal_V;
  int flt_opening;
  double flt_ot1, flt_otd;
  int flt_oxi[3];     /* first, last (<=0: last fault node), stride        */
  double flt_value[SEM2D_FP_NPARAM];        /* uniform values            */
  const double *flt_array[SEM2D_FP_NPARAM]; /* or per fault node (NULL)   */

  /* &TIME (time.f90:122-315) */
  int time_kind;      /* SEM2D_TIME_*                                       */
  double dt;          /* > 0: fixed timestep                                */
  double courant;     /* used when dt == 0                                  */
  double total_time;  /* > 0: sets nsteps                                   */
  int nsteps;
  double beta, gamma; /* &TIME_NEWMARK                                      */
  double hht_alpha, hht_rho; /* &TIME_HHTA alpha, rho (time.f90:222-240)     */

  /* &SRC_DEF (mechanism and time function: src_mech and stf below) */
  int nsrc;
  const double *src_coord;  /* (2,nsrc) requested positions                */
  const double *src_tdelay; /* [nsrc] or NULL                              */
  const double *src_ampli;  /* [nsrc] or NULL                              */
  double ricker_f0, ricker_onset, ricker_ampli; /* read as REAL (FP32)     */
  double force_angle;       /* degrees, counterclockwise from z-up          */

  /* &REC_LINE (receivers.f90:62-163) */
  int rec_number;
  double rec_first[2], rec_last[2];
  const double *rec_coord;  /* (2,rec_number) explicit positions or NULL   */
  int rec_atnode;
  int rec_isamp;
  char rec_field;

  /* options passed through to the descriptor */
  int precision;  /* SEM2D_PRECISION_*                                      */
  int kd2_form;   /* -1: as the reference (ngll == 5), 0 or 1 to force     */

  /* W of &GENERAL (2.5D term); <= 0 for a 2D problem                     */
  double width;
  /* &BC_DYNFLT_TWF (bc_dynflt_twf.f90:52-100); twf_kind 0 = absent.  With
   * flt_friction = SEM2D_FRICTION_TWF it is the only friction law,
   * otherwise it is superimposed on SWF/RSF.  Defaults of the reference:
   * kind 1, MuS 0.6, MuD 0.5, Mu0 0.6, X = Z = 0, V 1e3, L 1, T = Dc = huge */
  int twf_kind;
  double twf_mus, twf_mud, twf_mu0, twf_X, twf_Z, twf_V, twf_L, twf_T, twf_Dc;
  /* 1: record the fault potency every step (the FltXX_potency_sem2d.tab
   * file of the reference, bc_dynflt.f90:436,757)                        */
  int flt_potency;
  /* &SRC_DEF mechanism (src_moment.f90:27-110): 0 FORCE, 1 EXPLOSION,
   * 2 DOUBLE_COUPLE (&SRC_DOUBLE_COUPLE dip, degrees), 3 MOMENT
   * (&SRC_MOMENT Mxx, Mxz, Mzx, Mzz; SH: Myx, Myz in src_M[0], src_M[1]) */
  int src_mech;
  double src_M[4];
  double src_dip;
  /* &SRC_DEF stf (stf_gen.f90:45-97): kind SEM2D_STF_NONE or RICKER uses
   * ricker_f0, ricker_onset, ricker_ampli; the other kinds carry their
   * &STF_* values as written in the input (the builder rounds the ones the
   * reference reads as REAL) */
  sem2d_stf stf;
  /* &SRC_WAVE angle, phase (src_wave.f90:56-110) for src_mech = 4 (WAVE):
   * phase SEM2D_WAVE_P or SEM2D_WAVE_S (ignored in SH) */
  double wave_angle;
  int wave_phase;

  /* &MESH_DEF method: 0 'CARTESIAN' (the &MESH_CART values above), 1
   * 'LAYERED' (&MESH_LAYERED + &MESH_LAYER, mesh_layers.f90:120-300): xlim
   * and nelem[0] (nx) above, zmin, and the layers from the bottom up, each
   * with its element rows, material tag, control nodes (4: a flat or
   * piecewise-linear top, 9: any other distribution) and its top boundary
   * z at the nxp control abscissae xlim[0] + (xlim[1]-xlim[0]) i/(nxp-1),
   * nxp = nx+1 when every layer has 4 control nodes, else 2 nx+1.  ezflt,
   * fztag, fznz above apply to the layered mesh too. */
  int mesh_method;
  double zmin;
  int nlayer;
  int layer_nz[SEM2D_MAX_LAYERS];
  int layer_tag[SEM2D_MAX_LAYERS];
  int layer_ngnod[SEM2D_MAX_LAYERS];
  const double *layer_top[SEM2D_MAX_LAYERS];
} sem2d_deck;

typedef struct sem2d_grid sem2d_grid;
typedef struct sem2d_problem sem2d_problem;

/* Mesh + spectral grid (MESH_build then SE_init, init.f90:53-54). */
int sem2d_grid_build(const sem2d_deck *deck, sem2d_grid **out);
int sem2d_grid_sizes(const sem2d_grid *g, int *nelem, int *npoin, int *ngll);
/* ibool(ngll,ngll,nelem) 1-based, coord(2,npoin), tag(nelem) */
int sem2d_grid_ibool(const sem2d_grid *g, int *ibool);
int sem2d_grid_coord(const sem2d_grid *g, double *coord);
int sem2d_grid_tags(const sem2d_grid *g, int *tag);
/* Bulk nodes of boundary `tag` sorted along the boundary
 * (BC_set_bulk_node, spec_grid.f90:676-822); *npoin receives the count,
 * nodes (1-based) may be NULL to query the size. */
int sem2d_grid_boundary(const sem2d_grid *g, int tag, int *npoin, int *nodes);
/* GLL points, weights and H (gll.f90:19-36). */
int sem2d_grid_gll(const sem2d_grid *g, double *xgll, double *wgll,
                   double *hprime);
void sem2d_grid_destroy(sem2d_grid *g);

/* Everything else of init_main; the grid must outlive the problem. */
int sem2d_problem_build(const sem2d_grid *g, const sem2d_deck *deck,
                        sem2d_problem **out);
/* Descriptor whose arrays point into the problem (valid until destroy). */
int sem2d_problem_get_desc(const sem2d_problem *p, sem2d_problem_desc *out);
/* Timestep and the Courant number obtained (TIME_init). */
int sem2d_problem_time(const sem2d_problem *p, double *dt, int *nt,
                       double *courant);
/* Positions of receivers and sources after relocation, (2,n). */
int sem2d_problem_rec_coord(const sem2d_problem *p, double *coord);
int sem2d_problem_fault_coord(const sem2d_problem *p, double *coord);
void sem2d_problem_destroy(sem2d_problem *p);

/* Values of a time function at n times, as the library evaluates it for
 * the point sources and the boundary forces (SEM2D_E_ARG for a bad
 * description, message in sem2d_gpu_last_error(NULL)). */
int sem2d_stf_eval(const sem2d_stf *stf, int n, const double *t, double *out);

/* Message of the last failed builder call (thread local). */
const char *sem2d_host_last_error(void);

/* sizeof(sem2d_problem_desc) and sizeof(sem2d_deck) as compiled, so that
 * foreign-language bindings can check their struct layouts. */
int sem2d_abi_struct_sizes(int *desc_size, int *deck_size);

/* Offsets (bytes) of every member of a C-ABI structure as compiled, in
 * declaration order: which = 0 sem2d_problem_desc, 1 sem2d_deck,
 * 2 sem2d_lattice_args, 3 sem2d_stf.  Writes min(n, count) offsets when offsets is not
 * NULL and returns the member count (SEM2D_E_ARG for an unknown which). */
int sem2d_abi_field_offsets(int which, long long *offsets, int n);

/* ---- tuning cache of the one-element-per-thread kernel's launch shape
 * (no counterpart in the reference, which is serial).  The first handle of
 * a class of problems times candidate shapes on the device and records the
 * fastest; later handles of the class read it.  The cache is a text file of
 * one JSON object per line (see autotune.cpp); its path is SEM2D_TUNE_CACHE,
 * else $XDG_CACHE_HOME/sem2dpack_gb300/tune.json, else
 * $HOME/.cache/sem2dpack_gb300/tune.json.  SEM2D_AUTOTUNE=0 switches the
 * timing off (the analytic shape is used). */
typedef struct sem2d_tune_entry {
  int chunk_rows;     /* element rows per work unit                       */
  int warps_per_cta;  /* 1, 2 or 4                                        */
  double ms_per_step; /* measured                                         */
} sem2d_tune_entry;
/* The cache path into buf (n bytes); returns 0, or the bytes needed when
 * buf is NULL or too small, or SEM2D_E_STATE when no location is known. */
int sem2d_tune_cache_path(char *buf, int n);
/* The key of a class: dof count, material layout (0 node planes, 2 one
 * value per element), node count and member count (0: a single problem)
 * to a power of two, SM count. */
int sem2d_tune_key(int ndof, int mat_layout, long long nodes, int members, int nsm, char *buf, int n);
/* 1 and *out when the cache holds key, 0 when it does not. */
int sem2d_tune_lookup(const char *path, const char *key, sem2d_tune_entry *out);
/* Records (or replaces) the entry of key; the file is rewritten atomically. */
int sem2d_tune_record(const char *path, const char *key, const sem2d_tune_entry *e);
/* Index of the fastest of n timed candidates; candidate 0 (the analytic
 * shape) is kept unless another is faster by more than keep_margin (a
 * fraction of its time). */
int sem2d_tune_select(const sem2d_tune_entry *cands, int n, double keep_margin);

#ifdef __cplusplus
}
#endif

#endif /* SEM2D_HOST_H */

/*
 * ORACLE -- test infrastructure only.
 *
 * A plain-C, FP64 restatement of SEM2DPACK's initialisation and explicit
 * time step for the Cartesian-mesh solver path.  It is the checker for the
 * GB300 product: only the tests, the smoke check and the CPU-baseline leg of
 * the benchmark load it.  Nothing in the product links or calls it.
 *
 * Two halves:
 *   oc_setup_*  restates init_main (init.f90:16-131) for a sem2d_deck and
 *               exports the result as a sem2d_problem_desc;
 *   oc_sim_*    restates solve_leapfrog / solve_Newmark (solver.f90) with
 *               compute_Fint, SO_add, BC_apply, REC_store and
 *               BC_DYNFLT_write, driven by a sem2d_problem_desc -- the same
 *               input the GPU library receives.
 */
#ifndef SEM2D_ORACLE_H
#define SEM2D_ORACLE_H

#include "../include/sem2d_host.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oc_setup oc_setup;
typedef struct oc_sim oc_sim;

/* GLL helpers (gll.f90) */
void oc_gll_info(int n, double *x, double *w, double *H);
double oc_hgll(int i, double z, const double *zgll, int nz);
double oc_pnleg(double z, int n);
double oc_pndleg(double z, int n);

/* ---- initialisation ---- */
/* Restates MESH_build + SE_init + MAT_init_prop + CHECK_grid + TIME_init
 * + MAT_MASS_init + BC_init + REC_init + SO_init + mass inversion.
 * Returns NULL on error (message in err). */
oc_setup *oc_setup_build(const sem2d_deck *deck, char *err, int errlen);
/* grid only (MESH_build + SE_init), for the boundary/coordinate queries */
oc_setup *oc_grid_build(const sem2d_deck *deck, char *err, int errlen);
void oc_setup_free(oc_setup *s);
void oc_setup_sizes(const oc_setup *s, int *nelem, int *npoin, int *ngll);
void oc_setup_ibool(const oc_setup *s, int *ibool);   /* 1-based */
void oc_setup_coord(const oc_setup *s, double *coord);
void oc_setup_tags(const oc_setup *s, int *tag);
void oc_setup_knods(const oc_setup *s, int *knods);   /* 1-based, (4,nelem) */
int oc_setup_boundary(const oc_setup *s, int tag, int *nodes); /* count */
void oc_setup_time(const oc_setup *s, double *dt, int *nt, double *courant);
int oc_setup_desc(const oc_setup *s, sem2d_problem_desc *d);
int oc_setup_rec_coord(const oc_setup *s, double *coord); /* returns nrec */
int oc_setup_fault_coord(const oc_setup *s, double *coord); /* nflt */

/* ---- time stepping from a descriptor ---- */
oc_sim *oc_sim_create(const sem2d_problem_desc *d, char *err, int errlen);
/* advances nsteps; returns 0, or a negative SEM2D_E_* status */
int oc_sim_run(oc_sim *s, int nsteps);
int oc_sim_step_count(const oc_sim *s);
void oc_sim_fields(const oc_sim *s, double *displ, double *veloc, double *accel);
void oc_sim_seismograms(const oc_sim *s, double *sis);
void oc_sim_fault_series(const oc_sim *s, double *out);
/* [6*it + q], it = 0..nt: fault potency of d (q = 0..2) and v (q = 3..5) */
void oc_sim_fault_potency(const oc_sim *s, double *out);
/* strain and stress e/sig(ngll,ngll,ndof+1,nelem) of the current displacement */
void oc_sim_strain_stress(const oc_sim *s, double *strain, double *stress);
/* test hook: overwrite the displacement field d(npoin, ndof) */
void oc_sim_set_displacement(oc_sim *s, const double *d);
void oc_sim_fault_state(const oc_sim *s, double *D, double *V, double *T,
                        double *MU, double *theta);
void oc_sim_free(oc_sim *s);
/* STF_get of a time function at n times (test hook) */
int oc_stf_eval(const sem2d_stf *stf, int n, const double *t, double *out);

#ifdef __cplusplus
}
#endif

#endif

/*
 * ORACLE (test infrastructure only -- never part of the product path).
 *
 * FP64 restatement of SEM2DPACK's explicit time step, driven by the same
 * sem2d_problem_desc the GPU library receives:
 *   solve_leapfrog / solve_Newmark   solver.f90:42-83, 140-161
 *   compute_Fint                      solver.f90:273-316, fields.f90:113-189
 *   MAT_Fint -> MAT_KV_add_etav       mat_gen.f90:418-460,
 *               MAT_ELAST_f            mat_kelvin_voigt.f90:137-151,
 *               ELAST_KD1/KD2_PSV/SH   mat_elastic.f90:396-775
 *   a coefficients (MAT_ELAST_init_a) mat_elastic.f90:290-360
 *   SO_add + FORCE_add + ricker       src_gen.f90:290-317,
 *                                     src_force.f90:77-92, stf_ricker.f90:89-103
 *   STF_get (other time functions)    stf_gen.f90:99-121, stf_gaussian.f90:76-86,
 *                                     stf_brune.f90:73-83, stf_harmonic.f90:68-77,
 *                                     stf_user.f90:110-122, stf_tabulated.f90:83-95,
 *                                     spline/splint/hunt utils.f90:596-734
 *   BC_ABSO_apply (+ incident wave)   bc_abso.f90:286-336, SO_WAVE_get_VT
 *                                     src_gen.f90:322-339, src_wave.f90:181-224
 *   bc_DIRNEU_apply (tractions)       bc_dirneu.f90:148-169
 *   BC_DYNFLT_apply                   bc_dynflt.f90:569-739
 *   swf_*                             bc_dynflt_swf.f90:142-194
 *   rsf_*                             bc_dynflt_rsf.f90:165-568
 *   normal_update                     bc_dynflt_normal.f90:106-133
 *   REC_store                         receivers.f90:309-344
 *   BC_DYNFLT_write                   bc_dynflt.f90:751-778
 * Operation order follows the Fortran expressions; compile without FMA
 * contraction.
 */
#include <float.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sem2d_oracle.h"

#define PI_REF 3.141592653589793
#define V_HEALING 1.0e-14 /* bc_dynflt_swf.f90:27 */
#define NR_MAXIT 200      /* bc_dynflt_rsf.f90:372 */
#define NR_MAXBRACKET 200 /* the reference loop at :393-398 has no bound */

/* a source time function with the spline second derivatives of a table
 * and the bracket the last lookup found (splint keeps it, utils.f90:709) */
typedef struct {
  sem2d_stf s;
  double *t, *v, *y2;
  int klo;
} oc_stf;

struct oc_sim {
  int ngll, ndof, nelem, npoin, nelast, kd2;
  double *coord; /* (2,npoin) node positions (incident wave phases) */
  oc_stf *src_stf; /* NULL: the Ricker of src_f0, src_t0, src_amp */
  /* incident plane wave across the absorbing entries with abs_wave */
  int wave;
  double wave_k[2], wave_p[2], wave_s[2], wave_ref[2], wave_cp, wave_cs, wave_mu, wave_lambda, wave_tdelay;
  oc_stf *wave_stf;
  double *abs_B, *abs_n;
  int *abs_wave;
  /* Neumann tractions of &BC_DIRNEU */
  int nneu, nneu_stf;
  int *neu_node, *neu_comp, *neu_stf;
  double *neu_B;
  oc_stf *neu_stfs;
  int *ibool;
  double *H;
  double *acoef; /* (ngll,ngll,nelast,nelem) */
  double *dxidx, *detadz;      /* (ngll,ngll,nelem) inverse Jacobian (flat elements) */
  double *xjaci;               /* (2,2,ngll,ngll,nelem) inverse Jacobian of a grid that is not flat, or NULL */
  double *mKx, *mKz, *mla, *mmu; /* (ngll,ngll,nelem) moduli for MAT_ELAST_stress */
  double *beta25; /* (ngll,ngll,nelem) 2.5D coefficients or NULL */
  double *kveta;
  double *rmass;
  int nabs;
  int *abs_node;
  double *abs_C;
  int nstacey;
  int *st_node, *st_k, *st_edge;
  double *st_K;
  /* KxD of BC_ABSO_apply: per node (npoin,2), the nodes it touches, and the
   * periodic pairs at the ends of a side whose sums are shared */
  double *st_f;
  int nst_nodes, nst_pairs;
  int *st_nodes, *st_pm, *st_ps;
  int ndir;
  int *dir_node, *dir_comp, *dir_after;
  int nperio;
  int *per_m, *per_s;
  int scheme;
  double dt, beta, gamma;
  int nt;
  int nsrc;
  int *src_node;
  double *src_dir, *src_f0, *src_t0, *src_amp, *src_rel, *src_tdelay;
  int nrec, rec_isamp, rec_nsamp;
  char rec_field;
  int *rec_node, *rec_elem;
  double *rec_interp;
  double *sis;
  /* fault */
  int nflt, two, friction, swf_kind, swf_healing, rsf_kind, normal_kind, opening;
  int *node1, *node2;
  double *n1, *B, *invM1, *invM2, *Z, *T0, *coh;
  double coefA2V, coefA2D, nT, nL, nV, ncoef;
  double *swf_dc, *swf_mus, *swf_mud, *swf_p, *swf_alpha, *theta;
  double *rsf_dc, *rsf_mus, *rsf_a, *rsf_b, *rsf_vstar, *rsf_vc, *rsf_Tc, *rsf_coeft;
  double *D, *V, *T, *Tstick, *MU, *sigma;
  int twf_kind;
  double twf_mus, twf_mud, twf_mu0, twf_X, twf_Z, twf_V, twf_L, twf_T, twf_Dc;
  double *fcoord; /* (2,nflt) positions of node1 (bc_dynflt.f90:302) */
  int oit, oitd, oix1, oixn, oixd, fnsamp, onx, fsamp;
  double *fseries;
  int pot_rows;   /* nt + 1 */
  double *pseries; /* [6*it + q]: potency of d (q < 3) and v (q >= 3) */
  /* fields */
  double *d, *v, *a;
  double alpha;                /* HHT-alpha alpha */
  double tshift;               /* (alpha-1) dt: the time of the boundary terms */
  double *dal, *val;           /* HHT-alpha: d_alpha, v_alpha (NULL otherwise) */
  int it;
  int status;
};

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}
static double *dupd(const double *src, size_t n) {
  if (!src) return NULL;
  double *p = xcalloc(n, sizeof(double));
  memcpy(p, src, n * sizeof(double));
  return p;
}
static int *dupi(const int *src, size_t n) {
  if (!src) return NULL;
  int *p = xcalloc(n, sizeof(int));
  memcpy(p, src, n * sizeof(int));
  return p;
}
static double *dupd_or(const double *src, size_t n, double fill) {
  double *p = xcalloc(n, sizeof(double));
  for (size_t k = 0; k < n; k++) p[k] = src ? src[k] : fill;
  return p;
}

/* ------------------------------------------------------------------ */
/* MAT_ELAST_init_a for a grid that is not flat (mat_elastic.f90:290-360,
 * nelast 3 in SH, 10 in P-SV) from the inverse Jacobian and the weights the
 * descriptor carries (SE_InverseJacobian, SE_VolumeWeights) */
static void init_acoef_general(oc_sim *s, const sem2d_problem_desc *dd) {
  int n = s->ngll, ne = s->nelem, na = s->nelast;
  size_t st = (size_t)n * n;
  s->xjaci = dupd(dd->xjaci, 4 * st * ne);
  for (int e = 0; e < ne; e++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        size_t p = i + (size_t)n * j + st * e;
        const double *X = dd->xjaci + 4 * p;
        double DxiDx = X[0], DetaDx = X[1], DxiDz = X[2], DetaDz = X[3];
        double w = dd->dvol[p];
        double Kx = dd->Kx[p], Kz = dd->Kz[p], la = dd->la[p], mu = dd->mu[p], mux = dd->mux[p];
        double muz = mu;
        double *A = s->acoef + st * na * e + i + n * j;
        s->dxidx[p] = DxiDx;
        s->detadz[p] = DetaDz;
        s->mKx[p] = Kx;
        s->mKz[p] = Kz;
        s->mla[p] = la;
        s->mmu[p] = mu;
        if (s->beta25) {
          double pw;
          if (s->ndof == 1) {
            pw = PI_REF / dd->width;
          } else {
            double nu = (la / (la + mu)) / 2.0;
            pw = (PI_REF * (1.0 - nu)) / dd->width;
          }
          s->beta25[p] = (w * mu) * (pw * pw);
        }
        double a[10];
        if (na == 3) {
          a[0] = (mux * DxiDx) * DxiDx + (muz * DxiDz) * DxiDz;
          a[1] = (mux * DetaDx) * DetaDx + (muz * DetaDz) * DetaDz;
          a[2] = (mux * DxiDx) * DetaDx + (muz * DxiDz) * DetaDz;
        } else {
          a[0] = (Kx * DxiDx) * DxiDx + (mu * DxiDz) * DxiDz;
          a[1] = (la * DxiDx) * DetaDz + (mu * DxiDz) * DetaDx;
          a[2] = (Kz * DetaDz) * DetaDz + (mu * DetaDx) * DetaDx;
          a[3] = (Kx * DetaDx) * DetaDx + (mu * DetaDz) * DetaDz;
          a[4] = (la * DxiDz) * DetaDx + (mu * DxiDx) * DetaDz;
          a[5] = (Kz * DxiDz) * DxiDz + (mu * DxiDx) * DxiDx;
          a[6] = (Kx * DxiDx) * DetaDx + (mu * DxiDz) * DetaDz;
          a[7] = ((la + mu) * DxiDx) * DxiDz;
          a[8] = ((la + mu) * DetaDx) * DetaDz;
          a[9] = (Kz * DxiDz) * DetaDz + (mu * DxiDx) * DetaDx;
        }
        for (int k = 0; k < na; k++) A[k * st] = -(w * a[k]);
      }
}

/* MAT_ELAST_init_a for flat elements: Jacobian from the four corner
 * nodes (Q4, elem_q4.f90), inverse Jacobian by invert2 (utils.f90:92-114),
 * weights = det(J)*wgll(i)*wgll(j) (spec_grid.f90:590-602)             */
static void init_acoef(oc_sim *s, const sem2d_problem_desc *dd) {
  int n = s->ngll, ne = s->nelem, na = s->nelast;
  double *xg = xcalloc((size_t)n, sizeof(double)), *wg = xcalloc((size_t)n, sizeof(double));
  double *Hd = xcalloc((size_t)n * n, sizeof(double));
  oc_gll_info(n, xg, wg, Hd);
  free(Hd);
  s->acoef = xcalloc((size_t)n * n * na * ne, sizeof(double));
  s->dxidx = xcalloc((size_t)n * n * ne, sizeof(double));
  s->detadz = xcalloc((size_t)n * n * ne, sizeof(double));
  s->mKx = xcalloc((size_t)n * n * ne, sizeof(double));
  s->mKz = xcalloc((size_t)n * n * ne, sizeof(double));
  s->mla = xcalloc((size_t)n * n * ne, sizeof(double));
  s->mmu = xcalloc((size_t)n * n * ne, sizeof(double));
  s->beta25 = dd->width > 0.0 ? xcalloc((size_t)n * n * ne, sizeof(double)) : NULL;
  if (dd->xjaci) {
    init_acoef_general(s, dd);
    free(xg);
    free(wg);
    return;
  }
  for (int e = 0; e < ne; e++) {
    int cidx[4][2] = {{0, 0}, {n - 1, 0}, {n - 1, n - 1}, {0, n - 1}};
    double c[8];
    for (int k = 0; k < 4; k++) {
      int p = dd->ibool[cidx[k][0] + n * (cidx[k][1] + n * e)] - 1;
      c[2 * k] = dd->coord[2 * p];
      c[2 * k + 1] = dd->coord[2 * p + 1];
    }
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        double s_ = xg[i], t = xg[j];
        double sp = s_ + 1.0, sm = s_ - 1.0, tp = t + 1.0, tm = t - 1.0;
        double ds[8] = {0.25 * tm, -(0.25 * tm), 0.25 * tp, -(0.25 * tp),
                        0.25 * sm, -(0.25 * sp), 0.25 * sp, -(0.25 * sm)};
        double jac[4];
        for (int b = 0; b < 2; b++)
          for (int a = 0; a < 2; a++) {
            double acc = c[a] * ds[4 * b];
            for (int k = 1; k < 4; k++) acc = acc + c[a + 2 * k] * ds[k + 4 * b];
            jac[a + 2 * b] = acc;
          }
        double det = jac[0] * jac[3] - jac[2] * jac[1];
        double DxiDx = jac[3] / det, DetaDz = jac[0] / det;
        double w = det * (wg[i] * wg[j]);
        size_t p = i + (size_t)n * j + (size_t)n * n * e;
        double *A = s->acoef + (size_t)n * n * na * e + i + n * j;
        size_t st = (size_t)n * n;
        double Kx = dd->Kx[p], Kz = dd->Kz[p], la = dd->la[p], mu = dd->mu[p], mux = dd->mux[p];
        s->dxidx[p] = DxiDx;
        s->detadz[p] = DetaDz;
        s->mKx[p] = Kx;
        s->mKz[p] = Kz;
        s->mla[p] = la;
        s->mmu[p] = mu;
        if (s->beta25) {
          /* MAT_ELAST_init_25D (mat_elastic.f90:363-383), dvol = w */
          double pw;
          if (s->ndof == 1) {
            pw = PI_REF / dd->width;
          } else {
            double nu = (la / (la + mu)) / 2.0;
            pw = (PI_REF * (1.0 - nu)) / dd->width;
          }
          s->beta25[p] = (w * mu) * (pw * pw);
        }
        if (na == 2) {
          A[0] = -(w * ((mux * DxiDx) * DxiDx));
          A[st] = -(w * ((mu * DetaDz) * DetaDz));
        } else {
          A[0] = -(w * ((Kx * DxiDx) * DxiDx));
          A[st] = -(w * ((la * DxiDx) * DetaDz));
          A[2 * st] = -(w * ((Kz * DetaDz) * DetaDz));
          A[3 * st] = -(w * ((mu * DetaDz) * DetaDz));
          A[4 * st] = -(w * ((mu * DxiDx) * DetaDz));
          A[5 * st] = -(w * ((mu * DxiDx) * DxiDx));
        }
      }
  }
  free(xg);
  free(wg);
}

/* C = A*B for n x n column-major matrices, c(i,j) = sum_k a(i,k)b(k,j) in
 * increasing k (mxmlib.f90:12-31, My_MATMUL mat_elastic.f90:779-799) */
static void mxm(const double *A, const double *B, double *C, int n) {
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      double acc = A[i] * B[n * j];
      for (int k = 1; k < n; k++) acc = acc + A[i + n * k] * B[k + n * j];
      C[i + n * j] = acc;
    }
}

static void elem_forces(const oc_sim *s, int e, const double *dl, double *fl) {
  int n = s->ngll, n2 = n * n;
  const double *H = s->H;
  double Ht[400], t1[400], t2[400], t3[400], t4[400], tmp[400], tmp2[400];
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) Ht[i + n * j] = H[j + n * i];
  const double *A = s->acoef + (size_t)n2 * s->nelast * e;
  if (s->ndof == 1 && s->nelast == 3) { /* ELAST_KD1_SH / KD2_SH, general grid */
    mxm(Ht, dl, t1, n);
    mxm(dl, H, t2, n);
    for (int q = 0; q < n2; q++) tmp[q] = A[q] * t1[q] + A[2 * n2 + q] * t2[q];
    mxm(H, tmp, fl, n);
    for (int q = 0; q < n2; q++) tmp[q] = A[2 * n2 + q] * t1[q] + A[n2 + q] * t2[q];
    mxm(tmp, Ht, tmp2, n);
    for (int q = 0; q < n2; q++) fl[q] = fl[q] + tmp2[q];
    return;
  }
  if (s->ndof == 1) {
    mxm(Ht, dl, t1, n); /* dU_dxi  */
    mxm(dl, H, t2, n);  /* dU_deta */
    for (int q = 0; q < n2; q++) tmp[q] = A[q] * t1[q];
    mxm(H, tmp, fl, n);
    for (int q = 0; q < n2; q++) tmp[q] = A[n2 + q] * t2[q];
    mxm(tmp, Ht, tmp2, n);
    for (int q = 0; q < n2; q++) fl[q] = fl[q] + tmp2[q];
    return;
  }
  const double *ux = dl, *uz = dl + n2;
  double *fx = fl, *fz = fl + n2;
  mxm(Ht, ux, t1, n); /* dUx_dxi  */
  mxm(Ht, uz, t2, n); /* dUz_dxi  */
  mxm(ux, H, t3, n);  /* dUx_deta */
  mxm(uz, H, t4, n);  /* dUz_deta */
  const double *a1 = A, *a2 = A + n2, *a3 = A + 2 * n2, *a4 = A + 3 * n2, *a5 = A + 4 * n2,
               *a6 = A + 5 * n2;
  if (s->nelast == 10) { /* ELAST_KD1_PSV / KD2_PSV, general grid (mat_elastic.f90:499-516, 620-636) */
    const double *a7 = A + 6 * n2, *a8 = A + 7 * n2, *a9 = A + 8 * n2, *a10 = A + 9 * n2;
    for (int q = 0; q < n2; q++) tmp[q] = a1[q] * t1[q] + a7[q] * t3[q] + a8[q] * t2[q] + a2[q] * t4[q];
    mxm(H, tmp, fx, n);
    for (int q = 0; q < n2; q++) tmp[q] = a7[q] * t1[q] + a4[q] * t3[q] + a5[q] * t2[q] + a9[q] * t4[q];
    mxm(tmp, Ht, tmp2, n);
    for (int q = 0; q < n2; q++) fx[q] = fx[q] + tmp2[q];
    for (int q = 0; q < n2; q++) tmp[q] = a8[q] * t1[q] + a5[q] * t3[q] + a6[q] * t2[q] + a10[q] * t4[q];
    mxm(H, tmp, fz, n);
    for (int q = 0; q < n2; q++) tmp[q] = a2[q] * t1[q] + a9[q] * t3[q] + a10[q] * t2[q] + a3[q] * t4[q];
    mxm(tmp, Ht, tmp2, n);
    for (int q = 0; q < n2; q++) fz[q] = fz[q] + tmp2[q];
    return;
  }
  for (int q = 0; q < n2; q++) tmp[q] = a1[q] * t1[q] + a2[q] * t4[q];
  mxm(H, tmp, fx, n);
  if (s->kd2)
    for (int q = 0; q < n2; q++) tmp[q] = a4[q] * (t3[q] + t2[q]);
  else
    for (int q = 0; q < n2; q++) tmp[q] = a4[q] * t3[q] + a5[q] * t2[q];
  mxm(tmp, Ht, tmp2, n);
  for (int q = 0; q < n2; q++) fx[q] = fx[q] + tmp2[q];
  for (int q = 0; q < n2; q++) tmp[q] = a5[q] * t3[q] + a6[q] * t2[q];
  mxm(H, tmp, fz, n);
  for (int q = 0; q < n2; q++) tmp[q] = a2[q] * t1[q] + a3[q] * t4[q];
  mxm(tmp, Ht, tmp2, n);
  for (int q = 0; q < n2; q++) fz[q] = fz[q] + tmp2[q];
}

/* compute_Fint (solver.f90:273-316) */
static void compute_fint(oc_sim *s, double *f, const double *d, const double *v) {
  int n = s->ngll, n2 = n * n, nd = s->ndof, np = s->npoin;
  double dl[800], fl[800];
  memset(f, 0, (size_t)np * nd * sizeof(double));
  for (int e = 0; e < s->nelem; e++) {
    const int *ib = s->ibool + (size_t)n2 * e;
    for (int k = 0; k < nd; k++)
      for (int q = 0; q < n2; q++) dl[q + n2 * k] = d[(ib[q] - 1) + (size_t)np * k];
    if (s->kveta) {
      const double *eta = s->kveta + (size_t)n2 * e;
      for (int k = 0; k < nd; k++)
        for (int q = 0; q < n2; q++)
          dl[q + n2 * k] = dl[q + n2 * k] + eta[q] * v[(ib[q] - 1) + (size_t)np * k];
    }
    elem_forces(s, e, dl, fl);
    if (s->beta25) { /* MAT_ELAST_add_25D_f (mat_elastic.f90:447-459) */
      const double *b = s->beta25 + (size_t)n2 * e;
      for (int k = 0; k < nd; k++)
        for (int q = 0; q < n2; q++) fl[q + n2 * k] = fl[q + n2 * k] - b[q] * dl[q + n2 * k];
    }
    for (int q = 0; q < n2; q++)
      for (int k = 0; k < nd; k++) {
        size_t g = (ib[q] - 1) + (size_t)np * k;
        f[g] = f[g] + fl[q + n2 * k];
      }
  }
}

static double ricker(double t, double f0, double t0, double ampli) {
  double arg = PI_REF * f0 * (t - t0);
  arg = arg * arg;
  return -((ampli * (1.0 - 2.0 * arg)) * exp(-arg));
}

/* spline (utils.f90:652-691) with the end slopes STF_TAB_read gives, zero */
static void stf_spline(const double *x, const double *y, int n, double *y2) {
  double *u = xcalloc((size_t)n, sizeof(double));
  double yp1 = 0.0, ypn = 0.0;
  y2[0] = -0.5;
  u[0] = (3.0 / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - yp1);
  for (int i = 1; i < n - 1; i++) {
    double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    double p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) /
                (x[i + 1] - x[i - 1]) -
            sig * u[i - 1]) /
           p;
  }
  double qn = 0.5, un = (3.0 / (x[n - 1] - x[n - 2])) * (ypn - (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]));
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.0);
  for (int k = n - 2; k >= 0; k--) y2[k] = y2[k] * y2[k + 1] + u[k];
  free(u);
}

static void stf_init(oc_stf *o, const sem2d_stf *in) {
  memset(o, 0, sizeof(*o));
  o->s = *in;
  o->klo = 1;
  if (in->kind == SEM2D_STF_TAB) {
    int n = in->ntab;
    o->t = dupd(in->tab_t, (size_t)n);
    o->v = dupd(in->tab_v, (size_t)n);
    o->y2 = xcalloc((size_t)n, sizeof(double));
    stf_spline(o->t, o->v, n, o->y2);
    o->s.tab_t = o->t;
    o->s.tab_v = o->v;
  }
}
static void stf_free(oc_stf *o) {
  if (!o) return;
  free(o->t); free(o->v); free(o->y2);
}

/* hunt (utils.f90:596-646), 1-based jlo in and out: the index before x */
static int hunt(const double *xx, int n, double x, int jlo) {
  int jhi, inc = 1;
  const int ascnd = xx[n - 1] > xx[0];
  if (jlo <= 0 || jlo > n) {
    jlo = 0;
    jhi = n + 1;
  } else if ((x >= xx[jlo - 1]) == ascnd) {
    for (;;) {
      jhi = jlo + inc;
      if (jhi > n) { jhi = n + 1; break; }
      if ((x >= xx[jhi - 1]) == ascnd) { jlo = jhi; inc = inc + inc; }
      else break;
    }
  } else {
    jhi = jlo;
    for (;;) {
      jlo = jhi - inc;
      if (jlo < 1) { jlo = 0; break; }
      if ((x < xx[jlo - 1]) == ascnd) { jhi = jlo; inc = inc + inc; }
      else break;
    }
  }
  while (jhi - jlo != 1) {
    int jm = (jhi + jlo) / 2;
    if ((x > xx[jm - 1]) == ascnd) jlo = jm;
    else jhi = jm;
  }
  return jlo;
}

/* STF_get (stf_gen.f90:99-121) */
static double stf_get(oc_stf *o, double t) {
  const sem2d_stf *s = &o->s;
  double arg;
  switch (s->kind) {
    case SEM2D_STF_RICKER:
      return ricker(t, s->f0, s->onset, s->ampli);
    case SEM2D_STF_GAUSSIAN:
      arg = PI_REF * s->f0 * (t - s->onset);
      arg = arg * arg;
      return s->ampli * exp(-arg);
    case SEM2D_STF_BRUNE:
      arg = 2 * PI_REF * s->f0 * (t > 0.0 ? t : 0.0);
      return s->ampli * (1.0 - (1.0 + arg) * exp(-arg));
    case SEM2D_STF_HARMONIC:
      return s->ampli * sin(2.0 * PI_REF * t * s->f0);
    case SEM2D_STF_USER:
      arg = t - s->onset;
      return s->ampli * sin(arg) + s->par1 * (arg * arg);
    case SEM2D_STF_TAB: {
      int n = s->ntab;
      double tb = t > o->t[0] ? t : o->t[0];
      tb = tb < o->t[n - 1] ? tb : o->t[n - 1];
      /* splint (utils.f90:697-734) from the bracket of the last call; at
       * the first abscissa hunt can return 0, an index before the table
       * whose value at that abscissa is ya(1) all the same: kept in range */
      int klo = hunt(o->t, n, tb, o->klo);
      if (klo < 1) klo = 1;
      if (klo > n - 1) klo = n - 1;
      o->klo = klo;
      int khi = klo + 1;
      double h = o->t[khi - 1] - o->t[klo - 1];
      double a = (o->t[khi - 1] - tb) / h, b = (tb - o->t[klo - 1]) / h;
      return a * o->v[klo - 1] + b * o->v[khi - 1] +
             ((a * a * a - a) * o->y2[klo - 1] + (b * b * b - b) * o->y2[khi - 1]) * (h * h) / 6.0;
    }
    default:
      return 0.0;
  }
}

static void so_add(oc_sim *s, double t, double *f) {
  for (int k = 0; k < s->nsrc; k++) {
    double ampli = s->src_stf ? stf_get(s->src_stf, t - s->src_tdelay[k])
                              : ricker(t - s->src_tdelay[k], s->src_f0[k], s->src_t0[k], s->src_amp[k]);
    ampli = ampli * s->src_rel[k];
    size_t g = s->src_node[k] - 1;
    if (s->ndof == 1) {
      f[g] = f[g] + ampli;
    } else {
      f[g] = f[g] + s->src_dir[2 * k] * ampli;
      f[g + s->npoin] = f[g + s->npoin] + s->src_dir[2 * k + 1] * ampli;
    }
  }
}

/* SO_WAVE_get_VT (src_gen.f90:322-339) for absorbing entry k: the
 * incident velocity and traction, SRC_WAVE_get_VT (src_wave.f90:190-224)
 * times STF_get at SRC_WAVE_get_phase (:181-187) minus the delay */
static void wave_vt(oc_sim *s, int k, double time, double *Vin, double *Tin) {
  double n0 = s->abs_n[k], n1 = s->abs_n[k + s->nabs];
  double KN = s->wave_k[0] * n0 + s->wave_k[1] * n1;
  if (s->ndof == 1) {
    Vin[0] = 1.0;
    Tin[0] = -s->wave_mu / s->wave_cs * KN;
  } else {
    Vin[0] = s->wave_p[0];
    Vin[1] = s->wave_p[1];
    if (s->wave == SEM2D_WAVE_P) {
      Tin[0] = -1.0 / s->wave_cp * (s->wave_lambda * n0 + 2.0 * s->wave_mu * KN * s->wave_k[0]);
      Tin[1] = -1.0 / s->wave_cp * (s->wave_lambda * n1 + 2.0 * s->wave_mu * KN * s->wave_k[1]);
    } else {
      double PN = s->wave_p[0] * n0 + s->wave_p[1] * n1;
      Tin[0] = -s->wave_mu / s->wave_cs * (PN * s->wave_k[0] + KN * s->wave_p[0]);
      Tin[1] = -s->wave_mu / s->wave_cs * (PN * s->wave_k[1] + KN * s->wave_p[1]);
    }
  }
  const double *c = s->coord + 2 * (size_t)(s->abs_node[k] - 1);
  double phase = time - (c[0] - s->wave_ref[0]) * s->wave_s[0] - (c[1] - s->wave_ref[1]) * s->wave_s[1];
  phase = phase - s->wave_tdelay;
  double ampli = stf_get(s->wave_stf, phase);
  for (int d = 0; d < s->ndof; d++) {
    Vin[d] = ampli * Vin[d];
    Tin[d] = ampli * Tin[d];
  }
}

static void abso_apply(oc_sim *s, double *f, const double *v, const double *dsp, double time) {
  for (int k = 0; k < s->nabs; k++) {
    size_t g = s->abs_node[k] - 1;
    if (s->wave && s->abs_wave[k]) {
      /* total field = incident + diffracted: T = T_i - C (V - V_i)
       * (bc_abso.f90:279-306) */
      double Vin[2], Tin[2];
      wave_vt(s, k, time, Vin, Tin);
      for (int d = 0; d < s->ndof; d++) {
        size_t gg = g + (size_t)s->npoin * d;
        f[gg] = f[gg] - s->abs_C[k + (size_t)s->nabs * d] * (v[gg] - Vin[d]) + s->abs_B[k] * Tin[d];
      }
      continue;
    }
    for (int d = 0; d < s->ndof; d++) {
      size_t gg = g + (size_t)s->npoin * d;
      f[gg] = f[gg] - s->abs_C[k + (size_t)s->nabs * d] * v[gg];
    }
  }
  /* Stacey P3 (BC_ABSO_apply, bc_abso.f90:321-334): KxD accumulates, for
   * each boundary element edge point k, K(k,c,e) times the derivative of
   * D(:,c) along the edge's traversal order, sum_l Ht(k,l) D(node_l, c)
   * with Ht(k,l) = hprime(l,k); a side that crosses periodic sides shares
   * the sum of its two ends (:329-332); then MxA -= KxD */
  if (!s->nstacey) return;
  const size_t np = (size_t)s->npoin;
  for (int u = 0; u < s->nst_nodes; u++) {
    s->st_f[(size_t)s->st_nodes[u] - 1] = 0.0;
    s->st_f[(size_t)s->st_nodes[u] - 1 + np] = 0.0;
  }
  for (int t = 0; t < s->nstacey; t++) {
    const int n = s->ngll, k = s->st_k[t];
    const size_t g = (size_t)s->st_node[t] - 1;
    for (int c = 0; c < 2; c++) {
      double dd = 0.0;
      for (int l = 0; l < n; l++)
        dd += s->H[l + (size_t)n * k] * dsp[(size_t)s->st_edge[l + (size_t)n * t] - 1 + np * c];
      s->st_f[g + np * c] = s->st_f[g + np * c] + s->st_K[t + (size_t)s->nstacey * c] * dd;
    }
  }
  for (int q = 0; q < s->nst_pairs; q++)
    for (int c = 0; c < 2; c++) {
      size_t a = (size_t)s->st_pm[q] - 1 + np * c, b = (size_t)s->st_ps[q] - 1 + np * c;
      s->st_f[a] = s->st_f[a] + s->st_f[b];
      s->st_f[b] = s->st_f[a];
    }
  for (int u = 0; u < s->nst_nodes; u++)
    for (int c = 0; c < 2; c++) {
      size_t g = (size_t)s->st_nodes[u] - 1 + np * c;
      f[g] = f[g] - s->st_f[g];
    }
}

/* periodic sides: the forces of each node pair summed on the master and
 * copied to the slave (bc_perio_apply = BC_PERIO_set_field,
 * bc_periodic.f90:77-88), first of the boundary terms (bc_gen.f90:271-275) */
static void perio_apply(oc_sim *s, double *f) {
  for (int c = 0; c < s->ndof; c++)
    for (int k = 0; k < s->nperio; k++) {
      size_t m = (size_t)s->per_m[k] - 1 + (size_t)s->npoin * c, q = (size_t)s->per_s[k] - 1 + (size_t)s->npoin * c;
      f[m] = f[m] + f[q];
      f[q] = f[m];
    }
}

/* zero-Dirichlet components of the &BC_DIRNEU sides that come before (after
 * = 0) or after (after = 1) the fault in &BC_DEF order (bc_DIRNEU_apply,
 * bc_dirneu.f90:148-169; bc_apply, bc_gen.f90:271-281) */
static void dirneu_apply(oc_sim *s, double *f, int after) {
  for (int k = 0; k < s->ndir; k++)
    if (s->dir_after[k] == after)
      f[(size_t)s->dir_node[k] - 1 + (size_t)s->npoin * s->dir_comp[k]] = 0.0;
}

/* time-dependent Neumann tractions: field(node,c) += STF_get(stf, t) B
 * (bc_DIRNEU_apply, bc_dirneu.f90:157-167) */
static void neumann_apply(oc_sim *s, double *f, double time) {
  for (int k = 0; k < s->nneu; k++) {
    size_t g = (size_t)s->neu_node[k] - 1 + (size_t)s->npoin * s->neu_comp[k];
    f[g] = f[g] + stf_get(&s->neu_stfs[s->neu_stf[k]], time) * s->neu_B[k];
  }
}

/* ---------------- friction laws ---------------- */
static double swf_mu(const oc_sim *s, int k) {
  double th = s->theta[k], mu;
  if (s->swf_kind == 1) {
    double r = th / s->swf_dc[k];
    mu = s->swf_mus[k] - (s->swf_mus[k] - s->swf_mud[k]) * (r < 1.0 ? r : 1.0);
  } else if (s->swf_kind == 2) {
    mu = s->swf_mud[k] - (s->swf_mud[k] - s->swf_mus[k]) * exp(-th / s->swf_dc[k]);
  } else {
    mu = s->swf_mud[k] + (s->swf_mus[k] - s->swf_mud[k]) / pow(1.0 + th / s->swf_dc[k], s->swf_p[k]);
  }
  return mu + s->swf_alpha[k] * th;
}

static double rsf_mu(const oc_sim *s, int k, double v) {
  double av = fabs(v), a = s->rsf_a[k], b = s->rsf_b[k], th = s->theta[k];
  switch (s->rsf_kind) {
    case 1:
      return s->rsf_mus[k] + a * av / (av + s->rsf_vstar[k]) - b * th / (th + s->rsf_dc[k]);
    case 4:
      return a * asinh(av / (2.0 * s->rsf_vstar[k]) *
                       exp((s->rsf_mus[k] + b * log(s->rsf_vc[k] * th / s->rsf_dc[k] + 1.0)) / a));
    default:
      return a * asinh(av / (2.0 * s->rsf_vstar[k]) *
                       exp((s->rsf_mus[k] + b * log(s->rsf_vstar[k] * th / s->rsf_dc[k])) / a));
  }
}

static double rsf_update_theta(const oc_sim *s, int k, double theta, double v) {
  double th;
  switch (s->rsf_kind) {
    case 1:
      th = theta * s->rsf_coeft[k] + s->rsf_Tc[k] * fabs(v) * (1.0 - s->rsf_coeft[k]);
      if (th < 1.0e-12) th = 0.0;
      return th;
    case 3:
      th = s->rsf_dc[k] / fabs(v);
      return th * pow(theta / th, exp(-s->dt / th));
    default: {
      double x = fabs(v) / s->rsf_dc[k];
      double ex = exp(-(s->dt * x));
      if (s->dt * x > 1.0e-8) return theta * ex + (1.0 - ex) / x;
      return theta * ex + s->dt * (1.0 - 0.5 * s->dt * x);
    }
  }
}

/* nr_fric_func_tau (bc_dynflt_rsf.f90:533-568) */
static void nr_func(const oc_sim *s, int k, double theta, double tau, double tau_stick,
                    double sigma, double Z, double *fn, double *dfn, double *v) {
  double tmp;
  if (s->rsf_kind == 4)
    tmp = s->rsf_mus[k] + s->rsf_b[k] * log(s->rsf_vc[k] * theta / s->rsf_dc[k] + 1.0);
  else
    tmp = s->rsf_mus[k] + s->rsf_b[k] * log(s->rsf_vstar[k] * theta / s->rsf_dc[k]);
  tmp = 2.0 * s->rsf_vstar[k] * exp(-tmp / s->rsf_a[k]);
  double sa = -sigma * s->rsf_a[k];
  *v = sinh(tau / sa) * tmp;
  *fn = tau_stick - Z * (*v) - tau;
  double dv = cosh(tau / sa) * tmp / sa;
  *dfn = -Z * dv - 1.0;
}

/* nr_solver (bc_dynflt_rsf.f90:369-468): bracketed Newton-Raphson with
 * bisection.  The value returned is the slip rate of the last function
 * evaluation, exactly as in the reference. */
static double nr_solver(oc_sim *s, int k, double xL, double xR, double xacc, double theta,
                        double tau_stick, double sigma, double Z) {
  double flo, fhi, dfn, v, xl = xL, xr = xR;
  nr_func(s, k, theta, xL, tau_stick, sigma, Z, &flo, &dfn, &v);
  nr_func(s, k, theta, xR, tau_stick, sigma, Z, &fhi, &dfn, &v);
  int guard = 0;
  while (flo * fhi > 0) {
    if (++guard > NR_MAXBRACKET) {
      s->status = SEM2D_E_NR;
      return v;
    }
    xl = xl / 2.0;
    xr = xr * 2.0;
    nr_func(s, k, theta, xl, tau_stick, sigma, Z, &flo, &dfn, &v);
    nr_func(s, k, theta, xr, tau_stick, sigma, Z, &fhi, &dfn, &v);
  }
  double xlow, xhigh;
  if (flo == 0) return v;
  if (fhi == 0) return v;
  if (flo < 0) {
    xlow = xl;
    xhigh = xr;
  } else {
    xhigh = xl;
    xlow = xr;
  }
  double xest = 0.5 * (xl + xr), dxold = fabs(xr - xl), dx = dxold, fx;
  nr_func(s, k, theta, xest, tau_stick, sigma, Z, &fx, &dfn, &v);
  for (int is = 1; is <= NR_MAXIT; is++) {
    if (((xest - xhigh) * dfn - fx) * ((xest - xlow) * dfn - fx) > 0 ||
        fabs(2 * fx) > fabs(dxold * dfn)) {
      dxold = dx;
      dx = 0.5 * (xhigh - xlow);
      xest = xlow + dx;
      if (xlow == xest) return v;
    } else {
      dxold = dx;
      dx = fx / dfn;
      double temp = xest;
      xest = xest - dx;
      if (temp == xest) return v;
    }
    if (fabs(dx) < fabs(xacc)) {
      nr_func(s, k, theta, xest, tau_stick, sigma, Z, &fx, &dfn, &v);
      return v;
    }
    nr_func(s, k, theta, xest, tau_stick, sigma, Z, &fx, &dfn, &v);
    if (fx < 0)
      xlow = xest;
    else
      xhigh = xest;
  }
  s->status = SEM2D_E_NR;
  return v;
}

static double rsf_update_V(oc_sim *s, int k, double tau_stick, double sigma, double theta,
                           double Z) {
  if (s->rsf_kind == 1) {
    /* rsf_mu_no_direct uses the stored (old) state variable */
    double mnd = s->rsf_mus[k] - s->rsf_b[k] * s->theta[k] / (s->theta[k] + s->rsf_dc[k]);
    double v = (tau_stick + sigma * mnd) / Z;
    double tmp = v - s->rsf_vstar[k] + sigma * s->rsf_a[k] / Z;
    v = 0.5 * (tmp + sqrt(tmp * tmp + 4.0 * v * s->rsf_vstar[k]));
    v = v > 0.0 ? v : 0.0;
    if (v < 1.0e-12) v = 0.0;
    return v;
  }
  double tol = -0.001 * s->rsf_a[k] * sigma;
  double lo = tau_stick < 0.0 ? tau_stick : 0.0, hi = tau_stick > 0.0 ? tau_stick : 0.0;
  return nr_solver(s, k, lo, hi, tol, theta, tau_stick, sigma, Z);
}

/* twf_mu (bc_dynflt_twf.f90:117-184) at fault node k, time t, slip d.
 * Kind 3 leaves mu undefined beyond r > V T in the reference; here it is
 * the large value, so the other law (or sticking) decides there.        */
static double twf_mu(const oc_sim *s, int k, double time, double d) {
  const double big = DBL_MAX;
  double x = s->fcoord[2 * k] - s->twf_X, z = s->fcoord[2 * k + 1] - s->twf_Z;
  double dist = sqrt(x * x + z * z);
  if (s->twf_kind == 1 || s->twf_kind == 2) {
    double t, r;
    if (s->twf_kind == 1) {
      t = time + ((s->twf_mus - s->twf_mu0) * s->twf_L) / ((s->twf_mus - s->twf_mud) * s->twf_V);
      if (t > s->twf_T) t = 0.0;
      r = s->twf_V * t;
    } else {
      t = time + (0.5 * s->twf_T) *
                     (1.0 - sqrt(1.0 - ((4.0 * (s->twf_mus - s->twf_mu0)) * s->twf_L) /
                                           (((s->twf_mus - s->twf_mud) * s->twf_T) * s->twf_V)));
      if (t > s->twf_T) t = s->twf_T;
      r = (s->twf_V * t) * (1.0 - t / s->twf_T);
    }
    r = dist - r;
    if (r < -s->twf_L) return s->twf_mud;
    if (r <= s->twf_L) return s->twf_mus + ((s->twf_mus - s->twf_mud) / s->twf_L) * r;
    return big;
  }
  /* kind 3: cohesive nucleation front at V t */
  double vt = s->twf_V * time;
  if (dist <= s->twf_V * s->twf_T) {
    if (d <= s->twf_Dc) {
      if (dist < vt - s->twf_L) return s->twf_mud;
      if (dist >= vt - s->twf_L && dist <= vt)
        return s->twf_mus + ((s->twf_mus - s->twf_mud) / s->twf_L) * (dist - vt);
      return big;
    }
    return big;
  }
  return big;
}

/* BC_DYNFLT_apply (bc_dynflt.f90:569-689) */
static void dynflt_apply(oc_sim *s, double *f, const double *v, const double *d) {
  int nf = s->nflt, nd = s->ndof, np = s->npoin;
  for (int k = 0; k < nf; k++) {
    size_t g1 = s->node1[k] - 1, g2 = s->two ? (size_t)(s->node2[k] - 1) : 0;
    double dD[2] = {0, 0}, dV[2] = {0, 0}, dA[2] = {0, 0}, T[2] = {0, 0}, Ts[2] = {0, 0};
    for (int c = 0; c < nd; c++) {
      size_t o = (size_t)np * c;
      if (s->two) {
        dD[c] = d[g2 + o] - d[g1 + o];
        dV[c] = v[g2 + o] - v[g1 + o];
        dA[c] = s->invM2[k + nf * c] * f[g2 + o] - s->invM1[k + nf * c] * f[g1 + o];
      } else {
        dD[c] = -2.0 * d[g1 + o];
        dV[c] = -2.0 * v[g1 + o];
        dA[c] = -2.0 * s->invM1[k + nf * c] * f[g1 + o];
      }
      T[c] = s->Z[k + nf * c] * (dV[c] + s->coefA2V * dA[c]);
    }
    double nx = s->n1[k], nz = s->n1[k + nf];
    if (nd == 2) {
      double r0, r1;
      r0 = nz * dD[0] - nx * dD[1]; r1 = nx * dD[0] + nz * dD[1]; dD[0] = r0; dD[1] = r1;
      r0 = nz * dV[0] - nx * dV[1]; r1 = nx * dV[0] + nz * dV[1]; dV[0] = r0; dV[1] = r1;
      r0 = nz * dA[0] - nx * dA[1]; r1 = nx * dA[0] + nz * dA[1]; dA[0] = r0; dA[1] = r1;
      r0 = nz * T[0] - nx * T[1]; r1 = nx * T[0] + nz * T[1]; T[0] = r0; T[1] = r1;
    }
    if (!s->two || nd == 1) T[1] = 0.0;
    T[0] = T[0] + s->T0[k];
    T[1] = T[1] + s->T0[k + nf];
    if (s->opening) T[1] = T[1] < 0.0 ? T[1] : 0.0;
    /* normal_update */
    switch (s->normal_kind) {
      case 1: s->sigma[k] = T[1]; break;
      case 2: s->sigma[k] = T[1] + s->ncoef * (s->sigma[k] - T[1]); break;
      case 3: s->sigma[k] = T[1] + exp(-(fabs(dV[0]) + s->nV) * s->ncoef) * (s->sigma[k] - T[1]); break;
      default: break;
    }
    double sig = s->sigma[k];
    if (s->friction == SEM2D_FRICTION_RSF) {
      double vold = s->V[k];
      double th1 = rsf_update_theta(s, k, s->theta[k], vold);
      double vnew = rsf_update_V(s, k, T[0], sig, th1, s->Z[k]);
      double th2 = rsf_update_theta(s, k, s->theta[k], 0.5 * (vold + vnew));
      vnew = rsf_update_V(s, k, T[0], sig, th2, s->Z[k]);
      s->theta[k] = th2;
      s->V[k] = vnew;
      s->MU[k] = rsf_mu(s, k, s->V[k]);
      if (s->twf_kind) {
        double mt = twf_mu(s, k, s->it * s->dt + s->tshift, s->D[k]);
        if (mt < s->MU[k]) s->MU[k] = mt;
      }
      double strength = -s->MU[k] * sig;
      T[0] = copysign(fabs(strength), T[0]);
      /* T_stick is not defined on this branch of the reference
       * (bc_dynflt.f90:581); record zero before the T0 shift */
      Ts[0] = 0.0;
      Ts[1] = 0.0;
    } else {
      if (s->friction == SEM2D_FRICTION_SWF) {
        if (s->coefA2D == 0.0) {
          if (s->swf_healing) {
            s->theta[k] = s->theta[k] + fabs(dV[0]) * s->dt;
            if (fabs(dV[0]) < V_HEALING) s->theta[k] = 0.0;
          } else {
            s->theta[k] = fabs(dD[0]);
          }
        } else {
          s->theta[k] = fabs(s->D[k]);
        }
        s->MU[k] = swf_mu(s, k);
        if (s->twf_kind) {
          double mt = twf_mu(s, k, s->it * s->dt + s->tshift, s->D[k]);
          if (mt < s->MU[k]) s->MU[k] = mt;
        }
      } else { /* time weakening alone */
        s->MU[k] = twf_mu(s, k, s->it * s->dt + s->tshift, s->D[k]);
      }
      double strength = s->coh[k] - s->MU[k] * sig;
      Ts[0] = T[0];
      Ts[1] = T[1];
      double at = fabs(T[0]);
      T[0] = copysign(fabs(at < strength ? at : strength), T[0]);
    }
    T[0] = T[0] - s->T0[k];
    T[1] = T[1] - s->T0[k + nf];
    Ts[0] = Ts[0] - s->T0[k];
    Ts[1] = Ts[1] - s->T0[k + nf];
    s->T[k] = T[0];
    s->T[k + nf] = T[1];
    s->Tstick[k] = Ts[0];
    s->Tstick[k + nf] = Ts[1];
    double Tx[2] = {T[0], T[1]};
    if (nd == 2) {
      Tx[0] = nz * T[0] + nx * T[1];
      Tx[1] = -nx * T[0] + nz * T[1];
    }
    for (int c = 0; c < nd; c++) {
      size_t o = (size_t)np * c;
      f[g1 + o] = f[g1 + o] + s->B[k] * Tx[c];
      if (s->two) f[g2 + o] = f[g2 + o] - s->B[k] * Tx[c];
    }
    for (int c = 0; c < nd; c++) {
      double dAc = dA[c] - s->T[k + nf * c] / (s->Z[k + nf * c] * s->coefA2V);
      s->D[k + nf * c] = dD[c] + s->coefA2D * dAc;
      s->V[k + nf * c] = dV[c] + s->coefA2V * dAc;
    }
  }
}

static void rec_store(oc_sim *s) {
  if (s->nrec == 0 || s->it % s->rec_isamp != 0) return;
  int isamp = s->it / s->rec_isamp;
  if (isamp >= s->rec_nsamp) return;
  const double *fld = s->rec_field == 'D' ? s->d : (s->rec_field == 'A' ? s->a : s->v);
  int n2 = s->ngll * s->ngll, np = s->npoin;
  for (int r = 0; r < s->nrec; r++)
    for (int c = 0; c < s->ndof; c++) {
      double val;
      if (s->rec_node) {
        val = fld[(s->rec_node[r] - 1) + (size_t)np * c];
      } else {
        const int *ib = s->ibool + (size_t)n2 * (s->rec_elem[r] - 1);
        const double *w = s->rec_interp + (size_t)n2 * r;
        val = w[0] * fld[(ib[0] - 1) + (size_t)np * c];
        for (int q = 1; q < n2; q++) val = val + w[q] * fld[(ib[q] - 1) + (size_t)np * c];
      }
      s->sis[isamp + (size_t)s->rec_nsamp * (r + (size_t)s->nrec * c)] = val;
    }
}

/* BC_DYNFLT_potency (bc_dynflt.f90:832-855) of the displacement and the
 * velocity after the step, written every step (bc_dynflt.f90:757); the
 * jump is get_jump (bc_dynflt.f90:692-704).  P-SV: p11, p22, p12; SH: p13,
 * p23 (third entry zero). */
static void flt_potency(oc_sim *s) {
  if (s->nflt == 0 || s->it >= s->pot_rows) return;
  const int nf = s->nflt, nd = s->ndof;
  const size_t np = (size_t)s->npoin;
  double *o = s->pseries + 6 * (size_t)s->it;
  for (int f = 0; f < 2; f++) {
    const double *x = f == 0 ? s->d : s->v;
    double p0 = 0.0, p1 = 0.0, p2 = 0.0;
    for (int k = 0; k < nf; k++) {
      double dl[2] = {0.0, 0.0};
      for (int c = 0; c < nd; c++) {
        const double x1 = x[(size_t)(s->node1[k] - 1) + np * c];
        dl[c] = s->two ? x[(size_t)(s->node2[k] - 1) + np * c] - x1 : -2.0 * x1;
      }
      const double nx = s->n1[k], nz = s->n1[k + nf], b = s->B[k];
      if (nd == 2) {
        p0 = p0 + nx * dl[0] * b;
        p1 = p1 + nz * dl[1] * b;
        p2 = p2 + (nx * dl[1] + nz * dl[0]) * b;
      } else {
        p0 = p0 + nx * dl[0] * b;
        p1 = p1 + nz * dl[0] * b;
      }
    }
    if (nd == 2) {
      o[3 * f] = p0;
      o[3 * f + 1] = p1;
      o[3 * f + 2] = 0.5 * p2;
    } else {
      o[3 * f] = 0.5 * p0;
      o[3 * f + 1] = 0.5 * p1;
      o[3 * f + 2] = 0.0;
    }
  }
}

static void flt_write(oc_sim *s) {
  if (s->nflt == 0 || s->it < s->oit) return;
  if (s->fsamp < s->fnsamp) {
    int nf = s->nflt, q = 0;
    double *o = s->fseries + (size_t)s->onx * 6 * s->fsamp;
    for (int k = s->oix1 - 1; k <= s->oixn - 1; k += s->oixd, q++) {
      o[q] = s->D[k];
      o[q + s->onx] = s->V[k];
      o[q + 2 * s->onx] = s->T[k];
      o[q + 3 * s->onx] = s->T[k + nf];
      o[q + 4 * s->onx] = s->MU[k];
      o[q + 5 * s->onx] = s->Tstick[k];
    }
  }
  s->fsamp++;
  s->oit += s->oitd;
}

oc_sim *oc_sim_create(const sem2d_problem_desc *dd, char *err, int el) {
  if (!dd || dd->ngll < 2 || dd->ngll > 20 || (dd->ndof != 1 && dd->ndof != 2) || dd->nelem <= 0 ||
      dd->npoin <= 0) {
    if (err) snprintf(err, (size_t)el, "oc_sim_create: bad descriptor");
    return NULL;
  }
  oc_sim *s = xcalloc(1, sizeof(oc_sim));
  int n = dd->ngll, n2 = n * n, nd = dd->ndof, np = dd->npoin, ne = dd->nelem;
  s->ngll = n;
  s->ndof = nd;
  s->nelem = ne;
  s->npoin = np;
  s->nelast = dd->xjaci ? (nd == 1 ? 3 : 10) : (nd == 1 ? 2 : 6);
  s->kd2 = dd->kd2_form;
  s->ibool = dupi(dd->ibool, (size_t)n2 * ne);
  s->H = dupd(dd->hprime, (size_t)n2);
  init_acoef(s, dd);
  s->kveta = dupd(dd->kv_eta, (size_t)n2 * ne);
  s->rmass = dupd(dd->rmass, (size_t)np * nd);
  s->nabs = dd->nabs;
  s->abs_node = dupi(dd->abs_node, (size_t)dd->nabs);
  s->abs_C = dupd(dd->abs_C, (size_t)dd->nabs * nd);
  s->nstacey = dd->nstacey;
  s->st_node = dupi(dd->stacey_node, (size_t)dd->nstacey);
  s->st_k = dupi(dd->stacey_k, (size_t)dd->nstacey);
  s->st_edge = dupi(dd->stacey_edge, (size_t)dd->nstacey * n);
  s->st_K = dupd(dd->stacey_K, (size_t)dd->nstacey * 2);
  if (dd->nstacey > 0) {
    char *has = xcalloc((size_t)np, 1);
    s->st_f = xcalloc(2 * (size_t)np, sizeof(double));
    s->st_nodes = xcalloc((size_t)dd->nstacey, sizeof(int));
    for (int t = 0; t < dd->nstacey; t++) {
      int g = dd->stacey_node[t] - 1;
      if (!has[g]) s->st_nodes[s->nst_nodes++] = g + 1;
      has[g] = 1;
    }
    s->st_pm = xcalloc((size_t)dd->nperio + 1, sizeof(int));
    s->st_ps = xcalloc((size_t)dd->nperio + 1, sizeof(int));
    for (int q = 0; q < dd->nperio; q++) {
      int a = dd->perio_master[q], b = dd->perio_slave[q];
      if (has[a - 1] && has[b - 1]) {
        s->st_pm[s->nst_pairs] = a;
        s->st_ps[s->nst_pairs] = b;
        s->nst_pairs++;
      }
    }
    free(has);
  }
  s->ndir = dd->ndir;
  s->dir_node = dupi(dd->dir_node, (size_t)dd->ndir);
  s->dir_comp = dupi(dd->dir_comp, (size_t)dd->ndir);
  s->dir_after = dupi(dd->dir_after_fault, (size_t)dd->ndir);
  s->nperio = dd->nperio;
  s->per_m = dupi(dd->perio_master, (size_t)dd->nperio);
  s->per_s = dupi(dd->perio_slave, (size_t)dd->nperio);
  s->scheme = dd->time_scheme;
  s->alpha = dd->time_scheme == SEM2D_TIME_HHT ? dd->alpha : 1.0;
  s->dt = dd->dt;
  s->beta = dd->beta;
  s->gamma = dd->gamma;
  s->nt = dd->nt;
  s->coord = dupd(dd->coord, 2 * (size_t)np);
  if (dd->src_stf) {
    s->src_stf = xcalloc(1, sizeof(oc_stf));
    stf_init(s->src_stf, dd->src_stf);
  }
  if (dd->wave_phase != SEM2D_WAVE_NONE && dd->nabs > 0 && dd->abs_wave) {
    /* WAVE_init (src_wave.f90:158-172): K, P and the slowness s = K/c */
    double ang = PI_REF * dd->wave_angle / 180.0;
    s->wave = dd->wave_phase;
    s->wave_k[0] = -sin(ang);
    s->wave_k[1] = cos(ang);
    if (s->wave == SEM2D_WAVE_P) {
      s->wave_p[0] = -sin(ang);
      s->wave_p[1] = cos(ang);
    } else {
      s->wave_p[0] = cos(ang);
      s->wave_p[1] = sin(ang);
    }
    double c = s->wave == SEM2D_WAVE_P ? dd->wave_cp : dd->wave_cs;
    s->wave_s[0] = s->wave_k[0] / c;
    s->wave_s[1] = s->wave_k[1] / c;
    s->wave_ref[0] = dd->wave_ref[0];
    s->wave_ref[1] = dd->wave_ref[1];
    s->wave_cp = dd->wave_cp;
    s->wave_cs = dd->wave_cs;
    s->wave_mu = dd->wave_mu;
    s->wave_lambda = dd->wave_lambda;
    s->wave_tdelay = dd->wave_tdelay;
    s->wave_stf = xcalloc(1, sizeof(oc_stf));
    stf_init(s->wave_stf, dd->wave_stf);
    s->abs_B = dupd(dd->abs_B, (size_t)dd->nabs);
    s->abs_n = dupd(dd->abs_n, 2 * (size_t)dd->nabs);
    s->abs_wave = dupi(dd->abs_wave, (size_t)dd->nabs);
  }
  if (dd->nneu > 0) {
    s->nneu = dd->nneu;
    s->neu_node = dupi(dd->neu_node, (size_t)dd->nneu);
    s->neu_comp = dupi(dd->neu_comp, (size_t)dd->nneu);
    s->neu_stf = dupi(dd->neu_stf, (size_t)dd->nneu);
    s->neu_B = dupd(dd->neu_B, (size_t)dd->nneu);
    s->nneu_stf = dd->nneu_stf;
    s->neu_stfs = xcalloc((size_t)dd->nneu_stf, sizeof(oc_stf));
    for (int q = 0; q < dd->nneu_stf; q++) stf_init(&s->neu_stfs[q], &dd->neu_stfs[q]);
  }
  s->nsrc = dd->nsrc;
  s->src_node = dupi(dd->src_node, (size_t)dd->nsrc);
  s->src_dir = dupd(dd->src_dir, 2 * (size_t)dd->nsrc);
  s->src_f0 = dupd(dd->src_f0, (size_t)dd->nsrc);
  s->src_t0 = dupd(dd->src_t0, (size_t)dd->nsrc);
  s->src_amp = dupd(dd->src_ampli, (size_t)dd->nsrc);
  s->src_rel = dupd_or(dd->src_relamp, (size_t)dd->nsrc, 1.0);
  s->src_tdelay = dupd_or(dd->src_tdelay, (size_t)dd->nsrc, 0.0);
  s->nrec = dd->nrec;
  s->rec_isamp = dd->rec_isamp > 0 ? dd->rec_isamp : 1;
  s->rec_nsamp = dd->rec_nsamp;
  s->rec_field = dd->rec_field;
  s->rec_node = dupi(dd->rec_node, (size_t)dd->nrec);
  s->rec_elem = dd->rec_node ? NULL : dupi(dd->rec_elem, (size_t)dd->nrec);
  s->rec_interp = dd->rec_node ? NULL : dupd(dd->rec_interp, (size_t)n2 * dd->nrec);
  s->sis = xcalloc((size_t)dd->rec_nsamp * dd->nrec * nd + 1, sizeof(double));
  s->d = xcalloc((size_t)np * nd, sizeof(double));
  s->v = xcalloc((size_t)np * nd, sizeof(double));
  s->a = xcalloc((size_t)np * nd, sizeof(double));
  int nf = dd->nflt;
  s->nflt = nf;
  if (nf > 0) {
    s->two = dd->flt_node2 != NULL;
    s->friction = dd->flt_friction;
    s->swf_kind = dd->swf_kind;
    s->swf_healing = dd->swf_healing;
    s->rsf_kind = dd->rsf_kind;
    s->normal_kind = dd->normal_kind;
    s->opening = dd->flt_opening;
    s->node1 = dupi(dd->flt_node1, (size_t)nf);
    s->node2 = dupi(dd->flt_node2, (size_t)nf);
    s->n1 = dupd(dd->flt_n1, 2 * (size_t)nf);
    s->B = dupd(dd->flt_B, (size_t)nf);
    s->invM1 = dupd(dd->flt_invM1, (size_t)nf * nd);
    s->invM2 = dupd(dd->flt_invM2, (size_t)nf * nd);
    s->Z = dupd(dd->flt_Z, (size_t)nf * nd);
    s->T0 = dupd(dd->flt_T0, 2 * (size_t)nf);
    s->coh = dupd_or(dd->flt_cohesion, (size_t)nf, 0.0);
    s->coefA2V = dd->flt_coefA2V;
    s->coefA2D = dd->flt_coefA2D;
    s->nT = dd->normal_T;
    s->nL = dd->normal_L;
    s->nV = dd->normal_V;
    if (s->normal_kind == 2) s->ncoef = exp(-s->dt / s->nT);
    if (s->normal_kind == 3) s->ncoef = s->dt / s->nL;
    s->D = xcalloc((size_t)nf * nd, sizeof(double));
    s->V = xcalloc((size_t)nf * nd, sizeof(double));
    s->T = xcalloc(2 * (size_t)nf, sizeof(double));
    s->Tstick = xcalloc(2 * (size_t)nf, sizeof(double));
    s->MU = xcalloc((size_t)nf, sizeof(double));
    s->sigma = xcalloc((size_t)nf, sizeof(double));
    s->theta = xcalloc((size_t)nf, sizeof(double));
    for (int k = 0; k < nf; k++) s->sigma[k] = s->T0[k + nf];
    if (s->friction == SEM2D_FRICTION_SWF) {
      s->swf_dc = dupd(dd->swf_dc, nf);
      s->swf_mus = dupd(dd->swf_mus, nf);
      s->swf_mud = dupd(dd->swf_mud, nf);
      s->swf_p = dupd_or(dd->swf_p, nf, 3.0);
      s->swf_alpha = dupd_or(dd->swf_alpha, nf, 0.0);
      for (int k = 0; k < nf; k++) s->MU[k] = swf_mu(s, k);
    } else if (s->friction == SEM2D_FRICTION_RSF) {
      s->rsf_dc = dupd(dd->rsf_dc, nf);
      s->rsf_mus = dupd(dd->rsf_mus, nf);
      s->rsf_a = dupd(dd->rsf_a, nf);
      s->rsf_b = dupd(dd->rsf_b, nf);
      s->rsf_vstar = dupd(dd->rsf_vstar, nf);
      s->rsf_vc = dupd_or(dd->rsf_vc, nf, 1e-6);
      s->rsf_Tc = xcalloc((size_t)nf, sizeof(double));
      s->rsf_coeft = xcalloc((size_t)nf, sizeof(double));
      for (int k = 0; k < nf; k++) {
        s->theta[k] = dd->rsf_theta ? dd->rsf_theta[k] : 0.0;
        s->rsf_Tc[k] = s->rsf_dc[k] / s->rsf_vstar[k];
        s->rsf_coeft[k] = exp(-s->dt / s->rsf_Tc[k]);
        s->V[k] = dd->flt_V0 ? dd->flt_V0[k] : 1e-12;
        s->MU[k] = rsf_mu(s, k, s->V[k]);
      }
    }
    s->twf_kind = dd->twf_kind;
    if (s->friction == SEM2D_FRICTION_TWF && s->twf_kind == 0) s->twf_kind = 1;
    if (s->twf_kind) {
      s->twf_mus = dd->twf_mus;
      s->twf_mud = dd->twf_mud;
      s->twf_mu0 = dd->twf_mu0;
      s->twf_X = dd->twf_X;
      s->twf_Z = dd->twf_Z;
      s->twf_V = dd->twf_V;
      s->twf_L = dd->twf_L;
      s->twf_T = dd->twf_T;
      s->twf_Dc = dd->twf_Dc;
      s->fcoord = xcalloc(2 * (size_t)nf, sizeof(double));
      for (int k = 0; k < nf; k++) {
        s->fcoord[2 * k] = dd->coord[2 * (size_t)(dd->flt_node1[k] - 1)];
        s->fcoord[2 * k + 1] = dd->coord[2 * (size_t)(dd->flt_node1[k] - 1) + 1];
      }
      /* initial friction (bc_dynflt.f90:405-413), time 0, slip 0 */
      for (int k = 0; k < nf; k++) {
        double mt = twf_mu(s, k, 0.0, 0.0);
        if (s->friction == SEM2D_FRICTION_TWF || mt < s->MU[k]) s->MU[k] = mt;
      }
    }
    s->oit = dd->flt_oit;
    s->oitd = dd->flt_oitd > 0 ? dd->flt_oitd : 1;
    s->oix1 = dd->flt_oix1 > 0 ? dd->flt_oix1 : 1;
    s->oixn = dd->flt_oixn > 0 ? dd->flt_oixn : nf;
    s->oixd = dd->flt_oixd > 0 ? dd->flt_oixd : 1;
    s->fnsamp = dd->flt_nsamp;
    s->onx = (s->oixn - s->oix1) / s->oixd + 1;
    s->fseries = xcalloc((size_t)s->onx * 6 * (s->fnsamp > 0 ? s->fnsamp : 1), sizeof(double));
    s->pot_rows = (dd->nt > 0 ? dd->nt : 0) + 1;
    s->pseries = xcalloc((size_t)6 * s->pot_rows, sizeof(double));
  }
  /* step-0 outputs: REC_store(rec,0) (main.f90:35), BC_write(bc,0) (bc_gen.f90:247) */
  s->it = 0;
  flt_write(s);
  flt_potency(s);
  rec_store(s);
  return s;
}

int oc_sim_run(oc_sim *s, int nsteps) {
  int nd = s->ndof;
  size_t nn = (size_t)s->npoin * nd;
  double *d = s->d, *v = s->v, *a = s->a;
  const int hht = s->scheme == SEM2D_TIME_HHT;
  if (hht && !s->dal) {
    s->dal = xcalloc(nn, sizeof(double));
    s->val = xcalloc(nn, sizeof(double));
  }
  for (int st = 0; st < nsteps; st++) {
    s->it++;
    double t = s->it * s->dt;
    if (s->scheme == SEM2D_TIME_NEWMARK || hht) {
      /* predictors (solver.f90:59-60, 110-111); HHT-alpha keeps
       * d_alpha = alpha d_pred + (1-alpha) d_n and v_alpha alike (:106-113) */
      double cd = (0.5 - s->beta) * s->dt * s->dt, cv = (1.0 - s->gamma) * s->dt;
      for (size_t q = 0; q < nn; q++) {
        double d0 = d[q], v0 = v[q];
        d[q] = d[q] + s->dt * v[q] + cd * a[q];
        v[q] = v[q] + cv * a[q];
        if (hht) {
          s->dal[q] = s->alpha * d[q] + (1.0 - s->alpha) * d0;
          s->val[q] = s->alpha * v[q] + (1.0 - s->alpha) * v0;
        }
      }
    } else {
      for (size_t q = 0; q < nn; q++) d[q] = d[q] + s->dt * v[q];
    }
    const double *df = hht ? s->dal : d, *vf = hht ? s->val : v;
    /* HHT-alpha evaluates sources and boundaries at t + (alpha-1) dt
     * (solver.f90:116-122) */
    if (hht) t = t + (s->alpha - 1.0) * s->dt;
    s->tshift = hht ? (s->alpha - 1.0) * s->dt : 0.0;
    compute_fint(s, a, df, vf); /* f aliases accel */
    so_add(s, t, a);
    perio_apply(s, a);
    abso_apply(s, a, vf, df, t);
    neumann_apply(s, a, t);
    dirneu_apply(s, a, 0);
    if (s->nflt) dynflt_apply(s, a, v, d);
    dirneu_apply(s, a, 1);
    for (size_t q = 0; q < nn; q++) a[q] = s->rmass[q] * a[q];
    if (s->scheme == SEM2D_TIME_NEWMARK || hht) {
      double cv = s->gamma * s->dt, cd = s->beta * s->dt * s->dt;
      for (size_t q = 0; q < nn; q++) {
        v[q] = v[q] + cv * a[q];
        d[q] = d[q] + cd * a[q];
      }
    } else {
      for (size_t q = 0; q < nn; q++) v[q] = v[q] + s->dt * a[q];
    }
    rec_store(s);
    flt_write(s);
    flt_potency(s);
    if (s->status) return s->status;
  }
  return s->status;
}

int oc_sim_step_count(const oc_sim *s) { return s->it; }

/* test hook: overwrite the displacement field (npoin, ndof) */
void oc_sim_set_displacement(oc_sim *s, const double *d) {
  memcpy(s->d, d, (size_t)s->npoin * s->ndof * sizeof(double));
}

void oc_sim_fields(const oc_sim *s, double *d, double *v, double *a) {
  size_t nn = (size_t)s->npoin * s->ndof * sizeof(double);
  if (d) memcpy(d, s->d, nn);
  if (v) memcpy(v, s->v, nn);
  if (a) memcpy(a, s->a, nn);
}

void oc_sim_seismograms(const oc_sim *s, double *sis) {
  memcpy(sis, s->sis, (size_t)s->rec_nsamp * s->nrec * s->ndof * sizeof(double));
}

void oc_sim_fault_series(const oc_sim *s, double *out) {
  if (s->nflt) memcpy(out, s->fseries, (size_t)s->onx * 6 * s->fnsamp * sizeof(double));
}

/* MAT_strain_PSV/SH (mat_gen.f90:727-774) and MAT_ELAST_stress
 * (mat_elastic.f90:804-862) of the current displacement at every element
 * GLL point, e/sig(ngll,ngll,ndof+1,nelem); flat elements (dxi/dy =
 * deta/dx = 0).  Isotropic: Kx = Kz = lambda + 2 mu. */
void oc_sim_strain_stress(const oc_sim *s, double *eo, double *so) {
  int n = s->ngll, n2 = n * n, nd = s->ndof, nc = nd + 1;
  double Ht[400], dl[400], gx[400], ge[400];
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) Ht[i + n * j] = s->H[j + n * i];
  /* the stress of a Kelvin-Voigt element is that of d + eta v
   * (MAT_stress_dv, mat_gen.f90:626-641; MAT_KV_add_etav) */
  for (int e = 0; e < s->nelem; e++) {
    double g[2][2][400], gk[2][2][400];
    const double *eta = s->kveta ? s->kveta + (size_t)n2 * e : NULL;
    for (int k = 0; k < (eta ? 2 : 1); k++)
      for (int c = 0; c < nd; c++) {
        for (int q = 0; q < n2; q++) {
          size_t gq = (size_t)(s->ibool[q + (size_t)n2 * e] - 1) + (size_t)s->npoin * c;
          dl[q] = k == 0 ? s->d[gq] : s->d[gq] + eta[q] * s->v[gq];
        }
        mxm(Ht, dl, gx, n);
        mxm(dl, s->H, ge, n);
        memcpy(k == 0 ? g[c][0] : gk[c][0], gx, sizeof(double) * n2);
        memcpy(k == 0 ? g[c][1] : gk[c][1], ge, sizeof(double) * n2);
      }
    if (!eta) memcpy(gk, g, sizeof(g));
    for (int q = 0; q < n2; q++) {
      size_t p = q + (size_t)n2 * e;
      double *ev = eo + q + (size_t)n2 * nc * e, *sv = so + q + (size_t)n2 * nc * e;
      double dx = s->dxidx[p], dz = s->detadz[p];
      if (s->xjaci) { /* MAT_strain_SH / _PSV on a grid that is not flat (mat_gen.f90:736-772) */
        const double *X = s->xjaci + 4 * p;
        double xx = X[0], ex = X[1], xz = X[2], ez = X[3];
        if (nd == 1) {
          ev[0] = 0.5 * (g[0][0][q] * xx + g[0][1][q] * ex);
          ev[n2] = 0.5 * (g[0][0][q] * xz + g[0][1][q] * ez);
          sv[0] = 2.0 * s->mmu[p] * (0.5 * (gk[0][0][q] * xx + gk[0][1][q] * ex));
          sv[n2] = 2.0 * s->mmu[p] * (0.5 * (gk[0][0][q] * xz + gk[0][1][q] * ez));
        } else {
          ev[0] = g[0][0][q] * xx + g[0][1][q] * ex;
          ev[n2] = g[1][0][q] * xz + g[1][1][q] * ez;
          ev[2 * n2] = 0.5 * (g[0][0][q] * xz + g[0][1][q] * ez + g[1][0][q] * xx + g[1][1][q] * ex);
          double k0 = gk[0][0][q] * xx + gk[0][1][q] * ex, k1 = gk[1][0][q] * xz + gk[1][1][q] * ez;
          double k2 = 0.5 * (gk[0][0][q] * xz + gk[0][1][q] * ez + gk[1][0][q] * xx + gk[1][1][q] * ex);
          sv[0] = s->mKx[p] * k0 + s->mla[p] * k1;
          sv[n2] = s->mla[p] * k0 + s->mKz[p] * k1;
          sv[2 * n2] = 2.0 * s->mmu[p] * k2;
        }
        continue;
      }
      if (nd == 1) {
        ev[0] = 0.5 * (g[0][0][q] * dx);
        ev[n2] = 0.5 * (g[0][1][q] * dz);
        sv[0] = 2.0 * s->mmu[p] * (0.5 * (gk[0][0][q] * dx));
        sv[n2] = 2.0 * s->mmu[p] * (0.5 * (gk[0][1][q] * dz));
      } else {
        ev[0] = g[0][0][q] * dx;
        ev[n2] = g[1][1][q] * dz;
        ev[2 * n2] = 0.5 * (g[0][1][q] * dz + g[1][0][q] * dx);
        double k0 = gk[0][0][q] * dx, k1 = gk[1][1][q] * dz, k2 = 0.5 * (gk[0][1][q] * dz + gk[1][0][q] * dx);
        sv[0] = s->mKx[p] * k0 + s->mla[p] * k1;
        sv[n2] = s->mla[p] * k0 + s->mKz[p] * k1;
        sv[2 * n2] = 2.0 * s->mmu[p] * k2;
      }
    }
  }
}

void oc_sim_fault_potency(const oc_sim *s, double *out) {
  if (s->nflt) memcpy(out, s->pseries, (size_t)6 * s->pot_rows * sizeof(double));
}

void oc_sim_fault_state(const oc_sim *s, double *D, double *V, double *T, double *MU,
                        double *theta) {
  int nf = s->nflt, nd = s->ndof;
  if (!nf) return;
  if (D) memcpy(D, s->D, (size_t)nf * nd * sizeof(double));
  if (V) memcpy(V, s->V, (size_t)nf * nd * sizeof(double));
  if (T) memcpy(T, s->T, 2 * (size_t)nf * sizeof(double));
  if (MU) memcpy(MU, s->MU, (size_t)nf * sizeof(double));
  if (theta) memcpy(theta, s->theta, (size_t)nf * sizeof(double));
}

int oc_stf_eval(const sem2d_stf *stf, int n, const double *t, double *out) {
  oc_stf o;
  stf_init(&o, stf);
  for (int k = 0; k < n; k++) out[k] = stf_get(&o, t[k]);
  stf_free(&o);
  return 0;
}

void oc_sim_free(oc_sim *s) {
  if (!s) return;
  stf_free(s->src_stf);
  stf_free(s->wave_stf);
  for (int q = 0; q < s->nneu_stf; q++) stf_free(&s->neu_stfs[q]);
  free(s->src_stf); free(s->wave_stf); free(s->neu_stfs); free(s->coord);
  free(s->abs_B); free(s->abs_n); free(s->abs_wave);
  free(s->neu_node); free(s->neu_comp); free(s->neu_stf); free(s->neu_B);
  free(s->st_f); free(s->st_nodes); free(s->st_pm); free(s->st_ps);
  void *ptrs[] = {s->ibool, s->H, s->acoef, s->kveta, s->rmass, s->abs_node, s->abs_C,
                  s->st_node, s->st_k, s->st_edge, s->st_K, s->dir_node, s->dir_comp, s->dir_after,
                  s->dal, s->val, s->per_m, s->per_s,
                  s->src_node, s->src_dir, s->src_f0, s->src_t0, s->src_amp, s->src_rel,
                  s->src_tdelay, s->rec_node, s->rec_elem, s->rec_interp, s->sis, s->node1,
                  s->node2, s->n1, s->B, s->invM1, s->invM2, s->Z, s->T0, s->coh, s->swf_dc,
                  s->swf_mus, s->swf_mud, s->swf_p, s->swf_alpha, s->theta, s->rsf_dc,
                  s->rsf_mus, s->rsf_a, s->rsf_b, s->rsf_vstar, s->rsf_vc, s->rsf_Tc,
                  s->rsf_coeft, s->D, s->V, s->T, s->Tstick, s->MU, s->sigma, s->fseries,
                  s->d, s->v, s->a, s->beta25, s->fcoord, s->pseries, s->dxidx, s->detadz, s->xjaci,
                  s->mKx, s->mKz, s->mla, s->mmu};
  for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++) free(ptrs[k]);
  free(s);
}

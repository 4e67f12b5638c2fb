/*
 * ORACLE (test infrastructure only -- never part of the product path).
 *
 * FP64 restatement of SEM2DPACK's initialisation phase for the Cartesian
 * mesh (init_main, init.f90:16-131).  Each step follows the reference
 * routine cited beside it, in the same order of operations.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sem2d_oracle.h"

#define PI_REF 3.141592653589793      /* constants.f90:34 */
#define TINY_XABS 1.0e-3              /* constants.f90:30 */

typedef struct {
  int tag, nelem, npoin;
  int *elem, *edge;   /* 1-based bulk element, edge 1..4 */
  int *node;          /* [npoin] 1-based bulk node        */
  int *ibool;         /* (ngll,nelem) 1-based bc node     */
} oc_bnd;

struct oc_setup {
  int ngll, ndof, nelem, npoin;
  int nx, nz, ezflt;
  /* control-node (Q4) mesh */
  int fem_npoin;
  double *fem_coord; /* (2,fem_npoin) */
  int ngnod;         /* control nodes per element: 4 (Q4) or 9 (Q9)        */
  int flat;          /* grid%flat: rectangles (MESH_CART), not MESH_LAYERS  */
  int *knods;        /* (ngnod,nelem) 1-based */
  double *xjaci, *dvol; /* a grid that is not flat: SE_InverseJacobian, SE_VolumeWeights */
  int *tag;          /* [nelem] */
  int nbnds;
  oc_bnd bnds[8];
  /* spectral grid */
  double *xgll, *wgll, *H, *shape, *dshape;
  int *ibool;        /* (ngll,ngll,nelem) 1-based */
  double *coord;     /* (2,npoin) */
  /* material at element GLL points */
  double *rho, *cp, *cs, *Kx, *Kz, *la, *mu, *mux, *kveta;
  int has_kv;
  /* time */
  int time_kind;
  double dt, courant, total, beta, gamma, alpha;
  int nt;
  /* mass -> inverse mass */
  double *rmass;     /* (npoin,ndof) */
  /* absorbing entries in BC order */
  int nabs;
  int *abs_node;
  double *abs_C;     /* (nabs,ndof) */
  double *abs_B, *abs_nx, *abs_nz, *abs_n; /* weights, normals; abs_n (nabs,2) at export */
  int *abs_wave;
  /* time-dependent Neumann tractions of &BC_DIRNEU */
  int nneu, nneu_stf;
  int *neu_node, *neu_comp, *neu_stf;
  double *neu_B;
  sem2d_stf neu_stfs[2 * SEM2D_MAX_BCS];
  /* time function of the sources other than Ricker, incident plane wave;
   * TAB rows copied into tabs */
  int has_src_stf;
  sem2d_stf src_stf;
  int wave_phase;
  double wave_angle, wave_ref[2], wave_cp, wave_cs, wave_mu, wave_lambda, wave_tdelay;
  sem2d_stf wave_stf;
  int ntabs;
  double *tabs[4 * SEM2D_MAX_BCS + 4];
  /* Stacey P3 terms, one per (boundary element, edge point) */
  int nst;
  int *st_node, *st_k, *st_edge;
  double *st_K;      /* (nst,2) once the build ends; K(:,1) then K(:,2) while it grows */
  double *st_K1;
  /* periodic node pairs and zero-Dirichlet components */
  int nper;
  int *per_m, *per_s;
  int ndir;
  int *dir_node, *dir_comp, *dir_after;
  /* fault */
  int nflt, two_sides;
  int *node1, *node2;
  double *fcoord, *n1, *B, *invM1, *invM2, *Z, *T0, *coh;
  double coefA2V, coefA2D;
  double *prm[SEM2D_FP_NPARAM];
  int oit, oitd, oix1, oixn, oixd, fnsamp;
  /* sources */
  int nsrc;
  int *src_node;
  double *src_dir, *src_f0, *src_t0, *src_amp, *src_rel, *src_tdelay;
  /* receivers */
  int nrec, rec_isamp, rec_nsamp, rec_atnode;
  char rec_field;
  int *rec_node, *rec_elem;
  double *rec_interp, *rec_coord;
  const sem2d_deck *deck;
};

/* ------------------------------------------------------------------ */
static void seterr(char *err, int len, const char *fmt, ...) {
  if (!err || len <= 0) return;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(err, (size_t)len, fmt, ap);
  va_end(ap);
}

static void *xcalloc(size_t n, size_t sz) {
  void *p = calloc(n ? n : 1, sz);
  if (!p) {
    fprintf(stderr, "oracle: out of memory\n");
    abort();
  }
  return p;
}

#define IB(s, i, j, e) ((s)->ibool[(i) + (s)->ngll * ((j) + (s)->ngll * (e))])

/* Q4 shape functions and derivatives (elem_q4.f90:43-95) */
static void q4_shape(double s, double t, double *sh) {
  double sp = s + 1.0, sm = s - 1.0, tp = t + 1.0, tm = t - 1.0;
  sh[0] = 0.25 * sm * tm;
  sh[1] = -(0.25 * sp * tm);
  sh[2] = 0.25 * sp * tp;
  sh[3] = -(0.25 * sm * tp);
}
static void q4_dershape(double s, double t, double *d /* (4,2) */) {
  double sp = s + 1.0, sm = s - 1.0, tp = t + 1.0, tm = t - 1.0;
  d[0] = 0.25 * tm;
  d[1] = -(0.25 * tm);
  d[2] = 0.25 * tp;
  d[3] = -(0.25 * tp);
  d[4 + 0] = 0.25 * sm;
  d[4 + 1] = -(0.25 * sp);
  d[4 + 2] = 0.25 * sp;
  d[4 + 3] = -(0.25 * sm);
}

/* Q9 shape functions and derivatives (elem_q9.f90:40-110) */
static void q9_shape(double s, double t, double *sh) {
  double sp = s + 1.0, sm = s - 1.0, tp = t + 1.0, tm = t - 1.0, ss = s * s, tt = t * t, st = s * t;
  sh[0] = 0.25 * sm * st * tm;
  sh[1] = 0.25 * sp * st * tm;
  sh[2] = 0.25 * sp * st * tp;
  sh[3] = 0.25 * sm * st * tp;
  sh[4] = 0.5 * tm * t * (1.0 - ss);
  sh[5] = 0.5 * sp * s * (1.0 - tt);
  sh[6] = 0.5 * tp * t * (1.0 - ss);
  sh[7] = 0.5 * sm * s * (1.0 - tt);
  sh[8] = (1.0 - ss) * (1.0 - tt);
}
static void q9_dershape(double s, double t, double *d /* (9,2) */) {
  double sp = s + 1.0, sm = s - 1.0, tp = t + 1.0, tm = t - 1.0, ss = s * s, tt = t * t, st = s * t;
  double s2 = s * 2.0, t2 = t * 2.0;
  d[0] = 0.25 * tm * t * (s2 - 1.0);
  d[1] = 0.25 * tm * t * (s2 + 1.0);
  d[2] = 0.25 * tp * t * (s2 + 1.0);
  d[3] = 0.25 * tp * t * (s2 - 1.0);
  d[9 + 0] = 0.25 * sm * s * (t2 - 1.0);
  d[9 + 1] = 0.25 * sp * s * (t2 - 1.0);
  d[9 + 2] = 0.25 * sp * s * (t2 + 1.0);
  d[9 + 3] = 0.25 * sm * s * (t2 + 1.0);
  d[4] = -1.0 * st * tm;
  d[5] = 0.5 * (1.0 - tt) * (s2 + 1.0);
  d[6] = -1.0 * st * tp;
  d[7] = 0.5 * (1.0 - tt) * (s2 - 1.0);
  d[9 + 4] = 0.5 * (1.0 - ss) * (t2 - 1.0);
  d[9 + 5] = -1.0 * st * sp;
  d[9 + 6] = 0.5 * (1.0 - ss) * (t2 + 1.0);
  d[9 + 7] = -1.0 * st * sm;
  d[8] = -1.0 * s2 * (1.0 - tt);
  d[9 + 8] = -1.0 * t2 * (1.0 - ss);
}
/* FE_getshape / FE_getdershape (fem_grid.f90) for ngnod 4 or 9:
 * d(k + ngnod*b) */
static void shape_n(int ng, double s, double t, double *sh) {
  if (ng == 9) q9_shape(s, t, sh);
  else q4_shape(s, t, sh);
}
static void dershape_n(int ng, double s, double t, double *d) {
  if (ng == 9) q9_dershape(s, t, d);
  else q4_dershape(s, t, d);
}

static void elem_coorg(const oc_setup *s, int e, double *c /* (2,ngnod) */) {
  for (int k = 0; k < s->ngnod; k++) {
    int n = s->knods[k + s->ngnod * e] - 1;
    c[2 * k] = s->fem_coord[2 * n];
    c[2 * k + 1] = s->fem_coord[2 * n + 1];
  }
}

/* jac = matmul(coorg, dshape(:,:,i,j))  (spec_grid.f90:551-568) */
static void jacobian(const oc_setup *s, const double *c, int i, int j, double *jac) {
  int ng = s->ngnod;
  const double *ds = s->dshape + 2 * ng * (i + s->ngll * j);
  for (int b = 0; b < 2; b++)
    for (int a = 0; a < 2; a++) {
      double acc = c[a] * ds[0 + ng * b];
      for (int k = 1; k < ng; k++) acc = acc + c[a + 2 * k] * ds[k + ng * b];
      jac[a + 2 * b] = acc;
    }
}

/* ------------------------------------------------------------------ */
/* Reverse Cuthill-McKee (rcm.f90, George & Liu via Burkardt).
 * Arrays are 1-based like the reference (index 0 unused).              */
static void rcm_degree(int root, int *adj_row, const int *adj, const int *mask,
                       int *deg, int *iccsze, int *ls) {
  ls[1] = root;
  adj_row[root] = -adj_row[root];
  int lvlend = 0;
  *iccsze = 1;
  for (;;) {
    int lbegin = lvlend + 1;
    lvlend = *iccsze;
    for (int i = lbegin; i <= lvlend; i++) {
      int node = ls[i];
      int jstrt = -adj_row[node];
      int jstop = abs(adj_row[node + 1]) - 1;
      int ideg = 0;
      for (int j = jstrt; j <= jstop; j++) {
        int nbr = adj[j];
        if (mask[nbr] != 0) {
          ideg++;
          if (0 <= adj_row[nbr]) {
            adj_row[nbr] = -adj_row[nbr];
            (*iccsze)++;
            ls[*iccsze] = nbr;
          }
        }
      }
      deg[node] = ideg;
    }
    if (*iccsze - lvlend == 0) break;
  }
  for (int i = 1; i <= *iccsze; i++) {
    int node = ls[i];
    adj_row[node] = -adj_row[node];
  }
}

static void rcm_level_set(int root, const int *adj_row, const int *adj, int *mask,
                          int *level_num, int *level_row, int *level) {
  mask[root] = 0;
  level[1] = root;
  *level_num = 0;
  int lvlend = 0, iccsze = 1;
  for (;;) {
    int lbegin = lvlend + 1;
    lvlend = iccsze;
    (*level_num)++;
    level_row[*level_num] = lbegin;
    for (int i = lbegin; i <= lvlend; i++) {
      int node = level[i];
      for (int j = adj_row[node]; j <= adj_row[node + 1] - 1; j++) {
        int nbr = adj[j];
        if (mask[nbr] != 0) {
          iccsze++;
          level[iccsze] = nbr;
          mask[nbr] = 0;
        }
      }
    }
    if (iccsze - lvlend <= 0) break;
  }
  level_row[*level_num + 1] = lvlend + 1;
  for (int i = 1; i <= iccsze; i++) mask[level[i]] = 1;
}

static void rcm_root_find(int *root, const int *adj_row, const int *adj, int *mask,
                          int *level_num, int *level_row, int *level) {
  rcm_level_set(*root, adj_row, adj, mask, level_num, level_row, level);
  int iccsze = level_row[*level_num + 1] - 1;
  if (*level_num == 1) return;
  if (*level_num == iccsze) return;
  for (;;) {
    int mindeg = iccsze;
    int jstrt = level_row[*level_num];
    *root = level[jstrt];
    if (jstrt < iccsze) {
      for (int j = jstrt; j <= iccsze; j++) {
        int node = level[j], ndeg = 0;
        for (int k = adj_row[node]; k <= adj_row[node + 1] - 1; k++)
          if (0 < mask[adj[k]]) ndeg++;
        if (ndeg < mindeg) {
          *root = node;
          mindeg = ndeg;
        }
      }
    }
    int level_num2;
    rcm_level_set(*root, adj_row, adj, mask, &level_num2, level_row, level);
    if (level_num2 <= *level_num) break;
    *level_num = level_num2;
    if (iccsze <= *level_num) break;
  }
}

static void rcm_rcm(int root, int *adj_row, const int *adj, int *mask, int *perm,
                    int *iccsze, int *deg) {
  rcm_degree(root, adj_row, adj, mask, deg, iccsze, perm);
  mask[root] = 0;
  if (*iccsze <= 1) return;
  int lvlend = 0, lnbr = 1;
  while (lvlend < lnbr) {
    int lbegin = lvlend + 1;
    lvlend = lnbr;
    for (int i = lbegin; i <= lvlend; i++) {
      int node = perm[i];
      int fnbr = lnbr + 1;
      for (int j = adj_row[node]; j <= adj_row[node + 1] - 1; j++) {
        int nbr = adj[j];
        if (mask[nbr] != 0) {
          lnbr++;
          mask[nbr] = 0;
          perm[lnbr] = nbr;
        }
      }
      if (lnbr <= fnbr) continue;
      int k = fnbr;
      while (k < lnbr) {
        int l = k;
        k++;
        int nbr = perm[k];
        while (fnbr < l) {
          int lperm = perm[l];
          if (deg[lperm] <= deg[nbr]) break;
          perm[l + 1] = lperm;
          l--;
        }
        perm[l + 1] = nbr;
      }
    }
  }
  /* ivec_reverse */
  for (int i = 1; i <= *iccsze / 2; i++) {
    int t = perm[i];
    perm[i] = perm[*iccsze + 1 - i];
    perm[*iccsze + 1 - i] = t;
  }
}

/* genrcm (rcm.f90:260-330); perm is 1-based, perm[1..n] = old index */
static void rcm_genrcm(int n, int *adj_row, const int *adj, int *perm) {
  int *mask = xcalloc((size_t)n + 2, sizeof(int));
  int *level_row = xcalloc((size_t)n + 2, sizeof(int));
  int *deg = xcalloc((size_t)n + 2, sizeof(int));
  for (int i = 1; i <= n; i++) mask[i] = 1;
  int num = 1;
  for (int i = 1; i <= n; i++) {
    if (mask[i] != 0) {
      int root = i, level_num, iccsze;
      rcm_root_find(&root, adj_row, adj, mask, &level_num, level_row, perm + num - 1);
      rcm_rcm(root, adj_row, adj, mask, perm + num - 1, &iccsze, deg);
      num += iccsze;
      if (n < num) break;
    }
  }
  free(mask);
  free(level_row);
  free(deg);
}

/* ------------------------------------------------------------------ */
/* stable ascending ranking, as drank (utils.f90:165-330, merge sort) */
static void rank_stable(const double *key, int n, int *idx /* 0-based out */) {
  int *tmp = xcalloc((size_t)n, sizeof(int));
  for (int i = 0; i < n; i++) idx[i] = i;
  for (int w = 1; w < n; w *= 2) {
    for (int lo = 0; lo < n; lo += 2 * w) {
      int mid = lo + w < n ? lo + w : n, hi = lo + 2 * w < n ? lo + 2 * w : n;
      int a = lo, b = mid, k = lo;
      while (a < mid && b < hi) tmp[k++] = (key[idx[a]] <= key[idx[b]]) ? idx[a++] : idx[b++];
      while (a < mid) tmp[k++] = idx[a++];
      while (b < hi) tmp[k++] = idx[b++];
    }
    memcpy(idx, tmp, (size_t)n * sizeof(int));
  }
  free(tmp);
}

/* ------------------------------------------------------------------ */
/* CART_read + CART_build + MESH_STRUCTURED_* (mesh_cartesian.f90:86-314,
 * mesh_structured.f90:12-269)                                          */
/* MESH_LAYERS_build (mesh_layers.f90:331-449): control nodes row by row
 * from zmin, each layer's rows between its bottom and its top boundary
 * (given at the nxp control abscissae), the fault row duplicated; tags by
 * layer, then the fault zone */
static int layered_control(oc_setup *s, const sem2d_deck *dk, int *pnx, int *pnz, int *pezflt, int *pnxp,
                           char *err, int el) {
  int nx = dk->nelem[0], nl = dk->nlayer, ng = 4, nz = 0;
  if (nx <= 0) return seterr(err, el, "MESH_LAYERS_read: nx must be positive"), -1;
  if (nl <= 0 || nl > SEM2D_MAX_LAYERS) return seterr(err, el, "MESH_LAYERS_read: nlayer or file must be set"), -1;
  for (int k = 0; k < nl; k++) {
    if (dk->layer_nz[k] <= 0) return seterr(err, el, "MESH_LAYERS_read: nz null, negative or missing"), -1;
    if (dk->layer_tag[k] < 1) return seterr(err, el, "MESH_LAYERS_read: tag null, negative or missing"), -1;
    if (dk->layer_ngnod[k] != 4 && dk->layer_ngnod[k] != 9)
      return seterr(err, el, "MESH_LAYERS_read: unsupported layer top"), -1;
    if (dk->layer_ngnod[k] > ng) ng = dk->layer_ngnod[k];
    nz += dk->layer_nz[k];
  }
  int ezflt = dk->ezflt;
  if (ezflt == -1) ezflt = nz / 2;
  if (ezflt < -1) return seterr(err, el, "MESH_LAYERS_read: ezflt must be >= -1"), -1;
  if (ezflt >= nz) return seterr(err, el, "MESH_LAYERS_read: ezflt must be < nz"), -1;
  int d = ng == 9 ? 2 : 1, nxp = d * nx + 1, nzp = d * nz + 1 + (ezflt > 0 ? 1 : 0);
  s->ngnod = ng;
  s->flat = 0;
  s->fem_npoin = nxp * nzp;
  s->nelem = nx * nz;
  s->fem_coord = xcalloc(2 * (size_t)s->fem_npoin, sizeof(double));
  s->tag = xcalloc((size_t)s->nelem, sizeof(int));
  double *x = xcalloc((size_t)nxp, sizeof(double)), *bot = xcalloc((size_t)nxp, sizeof(double));
  for (int i = 0; i < nxp; i++) x[i] = dk->xlim[0] + (dk->xlim[1] - dk->xlim[0]) / (double)(nxp - 1) * (double)i;
  for (int k = 0; k < nl; k++) {
    if (!dk->layer_top[k]) {
      free(x); free(bot);
      return seterr(err, el, "MESH_LAYERS_build: layer top missing"), -1;
    }
    for (int i = 0; i < nxp; i++)
      if (dk->layer_top[k][i] < dk->zmin) {
        free(x); free(bot);
        return seterr(err, el, "MESH_LAYERS_build: zmin in MESH_LAYERED should be deeper than all layer interfaces"), -1;
      }
  }
  int row = 0;
  for (int i = 0; i < nxp; i++) {
    s->fem_coord[2 * i] = x[i];
    s->fem_coord[2 * i + 1] = dk->zmin;
    bot[i] = dk->zmin;
  }
  row = 1;
  int jposlast = 1;
  for (int k = 0; k < nl; k++) {
    const double *top = dk->layer_top[k];
    int nj = d * dk->layer_nz[k], jposflt = d * ezflt + 1 - jposlast;
    for (int j = 1; j <= nj; j++) {
      int reps = j == jposflt ? 2 : 1;
      for (int r = 0; r < reps; r++, row++)
        for (int i = 0; i < nxp; i++) {
          double *c = s->fem_coord + 2 * ((size_t)row * nxp + i);
          c[0] = x[i] + (double)j / (double)nj * (x[i] - x[i]);
          c[1] = bot[i] + (double)j / (double)nj * (top[i] - bot[i]);
        }
    }
    jposlast += nj;
    for (int i = 0; i < nxp; i++) bot[i] = top[i];
  }
  free(x);
  free(bot);
  int jl = 0;
  for (int k = 0; k < nl; k++)
    for (int j = 0; j < dk->layer_nz[k]; j++, jl++)
      for (int i = 0; i < nx; i++) s->tag[jl * nx + i] = dk->layer_tag[k];
  if (dk->fztag > 0 && ezflt > 0) {
    int fznz = dk->fznz > 0 ? dk->fznz : 1;
    int j1 = ezflt + 1 - fznz > 1 ? ezflt + 1 - fznz : 1;
    int j2 = ezflt + fznz < nz ? ezflt + fznz : nz;
    for (int j = j1; j <= j2; j++)
      for (int i = 1; i <= nx; i++) s->tag[(j - 1) * nx + (i - 1)] = dk->fztag;
  }
  for (int e = 0; e < s->nelem; e++)
    if (s->tag[e] == 0) return seterr(err, el, "MESH_LAYERS_build: Domain tags not entirely set"), -1;
  *pnx = nx;
  *pnz = nz;
  *pezflt = ezflt;
  *pnxp = nxp;
  return 0;
}

static int build_mesh(oc_setup *s, const sem2d_deck *dk, char *err, int el) {
  int nx, nz, ezflt, nxp;
  s->ngnod = 4;
  s->flat = 1;
  if (dk->mesh_method == 1) {
    if (layered_control(s, dk, &nx, &nz, &ezflt, &nxp, err, el)) return -1;
    s->nx = nx;
    s->nz = nz;
    s->ezflt = ezflt;
  } else {
  nx = dk->nelem[0];
  nz = dk->nelem[1];
  if (nx <= 0 || nz <= 0) return seterr(err, el, "CART_read: nelem must be positive"), -1;
  ezflt = dk->ezflt;
  if (ezflt >= nz) return seterr(err, el, "CART_read: ezflt must be < nelem(2)"), -1;
  if (ezflt == -1) ezflt = nz / 2;
  if (ezflt < -1) return seterr(err, el, "CART_read: ezflt must be >= -1"), -1;
  s->nx = nx;
  s->nz = nz;
  s->ezflt = ezflt;
  nxp = nx + 1;
  int nzp = ezflt > 0 ? nz + 2 : nz + 1;
  s->fem_npoin = nxp * nzp;
  s->nelem = nx * nz;
  s->fem_coord = xcalloc(2 * (size_t)s->fem_npoin, sizeof(double));
  s->tag = xcalloc((size_t)s->nelem, sizeof(int));
  double *x = xcalloc((size_t)nxp, sizeof(double)), *z = xcalloc((size_t)nzp, sizeof(double));
  double hx = (dk->xlim[1] - dk->xlim[0]) / (double)nx;
  double hz = (dk->zlim[1] - dk->zlim[0]) / (double)nz;
  for (int i = 0; i < nxp; i++) x[i] = dk->xlim[0] + hx * (double)i;
  if (ezflt > 0) {
    int k = 0;
    for (int j = 0; j <= ezflt; j++) z[k++] = dk->zlim[0] + hz * (double)j;
    for (int j = ezflt; j <= nz; j++) z[k++] = dk->zlim[0] + hz * (double)j;
  } else {
    for (int j = 0; j <= nz; j++) z[j] = dk->zlim[0] + hz * (double)j;
  }
  for (int j = 0; j < nzp; j++)
    for (int i = 0; i < nxp; i++) {
      s->fem_coord[2 * (j * nxp + i)] = x[i];
      s->fem_coord[2 * (j * nxp + i) + 1] = z[j];
    }
  free(x);
  free(z);
  /* domain tags */
  if (dk->ndomains == 0) {
    for (int e = 0; e < s->nelem; e++) s->tag[e] = 1;
  } else {
    for (int d = 0; d < dk->ndomains; d++) {
      const sem2d_domain *dm = &dk->domains[d];
      if (dm->tag < 1) return seterr(err, el, "CART_read: tag null, negative or missing"), -1;
      if (dm->ex[0] < 1 || dm->ex[0] > nx || dm->ex[1] < 1 || dm->ex[1] > nx ||
          dm->ez[0] < 1 || dm->ez[0] > nz || dm->ez[1] < 1 || dm->ez[1] > nz)
        return seterr(err, el, "CART_read: domain index out of bounds"), -1;
      for (int i = dm->ex[0]; i <= dm->ex[1]; i++)
        for (int j = dm->ez[0]; j <= dm->ez[1]; j++) s->tag[(j - 1) * nx + (i - 1)] = dm->tag;
    }
  }
  if (dk->fztag > 0) {
    int fznz = dk->fznz > 0 ? dk->fznz : 1;
    int j1 = ezflt + 1 - fznz > 1 ? ezflt + 1 - fznz : 1;
    int j2 = ezflt + fznz < nz ? ezflt + fznz : nz;
    for (int j = j1; j <= j2; j++)
      for (int i = 1; i <= nx; i++) s->tag[(j - 1) * nx + (i - 1)] = dk->fztag;
  }
  for (int e = 0; e < s->nelem; e++)
    if (s->tag[e] == 0) return seterr(err, el, "CART_build: Domain tags not entirely set"), -1;
  }
  /* MESH_STRUCTURED_connectivity (mesh_structured.f90:31-99): elements
   * numbered left to right, bottom to top; Q9 nodes on the doubled grid */
  int ng = s->ngnod;
  s->knods = xcalloc((size_t)ng * s->nelem, sizeof(int));
  int k = 0;
  for (int je = 1; je <= nz; je++)
    for (int ie = 1; ie <= nx; ie++, k++) {
      int *kn = s->knods + (size_t)ng * k;
      if (ng == 4) {
        int i = ie, j = je;
        kn[0] = (j - 1) * nxp + i;
        kn[1] = (j - 1) * nxp + i + 1;
        kn[2] = j * nxp + i + 1;
        kn[3] = j * nxp + i;
      } else {
        int i = 2 * (ie - 1) + 1, j = 2 * (je - 1) + 1;
#define SUB2IND(ii, jj) (((jj) - 1) * nxp + (ii))
        kn[0] = SUB2IND(i, j);
        kn[1] = SUB2IND(i + 2, j);
        kn[2] = SUB2IND(i + 2, j + 2);
        kn[3] = SUB2IND(i, j + 2);
        kn[4] = SUB2IND(i + 1, j);
        kn[5] = SUB2IND(i + 2, j + 1);
        kn[6] = SUB2IND(i + 1, j + 2);
        kn[7] = SUB2IND(i, j + 1);
        kn[8] = SUB2IND(i + 1, j + 1);
#undef SUB2IND
      }
    }
  if (ezflt > 0)
    for (int e = nx * ezflt; e < s->nelem; e++)
      for (int c = 0; c < ng; c++) s->knods[(size_t)ng * e + c] += nxp;
  /* boundaries: bnds(1..4) = sides D,R,U,L; 5 = fault down, 6 = fault up */
  s->nbnds = ezflt > 0 ? 6 : 4;
  int cnt[6] = {nx, nz, nx, nz, nx, nx};
  for (int b = 0; b < s->nbnds; b++) {
    oc_bnd *bd = &s->bnds[b];
    bd->tag = b + 1;
    bd->nelem = cnt[b];
    bd->elem = xcalloc((size_t)cnt[b], sizeof(int));
    bd->edge = xcalloc((size_t)cnt[b], sizeof(int));
  }
  for (int i = 1; i <= nx; i++) {
    s->bnds[0].elem[i - 1] = i;                 /* (i,1) edge D */
    s->bnds[0].edge[i - 1] = 1;
    s->bnds[2].elem[i - 1] = (nz - 1) * nx + i; /* (i,nz) edge U */
    s->bnds[2].edge[i - 1] = 3;
  }
  for (int j = 1; j <= nz; j++) {
    s->bnds[1].elem[j - 1] = (j - 1) * nx + nx; /* (nx,j) edge R */
    s->bnds[1].edge[j - 1] = 2;
    s->bnds[3].elem[j - 1] = (j - 1) * nx + 1;  /* (1,j) edge L */
    s->bnds[3].edge[j - 1] = 4;
  }
  if (ezflt > 0)
    for (int i = 1; i <= nx; i++) {
      s->bnds[5].elem[i - 1] = ezflt * nx + i;       /* fault up: (i,ezflt+1) edge D */
      s->bnds[5].edge[i - 1] = 1;
      s->bnds[4].elem[i - 1] = (ezflt - 1) * nx + i; /* fault down: (i,ezflt) edge U */
      s->bnds[4].edge[i - 1] = 3;
    }
  /* RCM renumbering (OPT_RENUMBER, constants.f90:11) */
  int ne = s->nelem;
  int *adj_row = xcalloc((size_t)ne + 2, sizeof(int));
  int *adj = xcalloc(8 * (size_t)ne + 2, sizeof(int));
  int nadj = 0, e = 0;
  for (int j = 1; j <= nz; j++)
    for (int i = 1; i <= nx; i++) {
      e++;
      adj_row[e] = nadj + 1;
      int di[8] = {-1, 0, 1, -1, 1, -1, 0, 1}, dj[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
      for (int q = 0; q < 8; q++) {
        int ii = i + di[q], jj = j + dj[q];
        if (ii >= 1 && ii <= nx && jj >= 1 && jj <= nz) adj[++nadj] = (jj - 1) * nx + ii;
      }
    }
  adj_row[e + 1] = nadj + 1;
  int *perm = xcalloc((size_t)ne + 2, sizeof(int));
  rcm_genrcm(ne, adj_row, adj, perm);
  int *perm_inv = xcalloc((size_t)ne + 2, sizeof(int));
  for (int i = 1; i <= ne; i++) perm_inv[perm[i]] = i;
  /* FE_reorder (fem_grid.f90:505-520) */
  int *kn2 = xcalloc((size_t)ng * ne, sizeof(int)), *tg2 = xcalloc((size_t)ne, sizeof(int));
  for (int i = 1; i <= ne; i++) {
    memcpy(kn2 + (size_t)ng * (i - 1), s->knods + (size_t)ng * (perm[i] - 1), (size_t)ng * sizeof(int));
    tg2[i - 1] = s->tag[perm[i] - 1];
  }
  free(s->knods);
  free(s->tag);
  s->knods = kn2;
  s->tag = tg2;
  for (int b = 0; b < s->nbnds; b++)
    for (int q = 0; q < s->bnds[b].nelem; q++) s->bnds[b].elem[q] = perm_inv[s->bnds[b].elem[q]];
  free(adj_row);
  free(adj);
  free(perm);
  free(perm_inv);
  return 0;
}

/* ------------------------------------------------------------------ */
/* SE_init (spec_grid.f90:121-374, 665-822)                             */
static void edge_ij(int ngll, int edge, int *it, int *jt) {
  for (int k = 0; k < ngll; k++) {
    switch (edge) {
      case 1: it[k] = k; jt[k] = 0; break;
      case 2: it[k] = ngll - 1; jt[k] = k; break;
      case 3: it[k] = ngll - 1 - k; jt[k] = ngll - 1; break;
      default: it[k] = 0; jt[k] = ngll - 1 - k; break;
    }
  }
}

static int build_grid(oc_setup *s, const sem2d_deck *dk, char *err, int el) {
  int n = dk->ngll;
  if (n < 2 || n > 20) return seterr(err, el, "ngll out of range"), -1;
  s->ngll = n;
  s->ndof = dk->ndof;
  s->xgll = xcalloc((size_t)n, sizeof(double));
  s->wgll = xcalloc((size_t)n, sizeof(double));
  s->H = xcalloc((size_t)n * n, sizeof(double));
  oc_gll_info(n, s->xgll, s->wgll, s->H);
  int ng = s->ngnod;
  s->shape = xcalloc((size_t)ng * n * n, sizeof(double));
  s->dshape = xcalloc(2 * (size_t)ng * n * n, sizeof(double));
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) {
      shape_n(ng, s->xgll[i], s->xgll[j], s->shape + ng * (i + n * j));
      dershape_n(ng, s->xgll[i], s->xgll[j], s->dshape + 2 * ng * (i + n * j));
    }
  /* FE_SetConnectivity: vertex lists in head-insertion order */
  int nv = s->fem_npoin, ne = s->nelem;
  int *vcnt = xcalloc((size_t)nv + 1, sizeof(int));
  for (int e = 0; e < ne; e++)
    for (int c = 0; c < 4; c++) vcnt[s->knods[s->ngnod * e + c]]++;
  int *vstart = xcalloc((size_t)nv + 2, sizeof(int));
  for (int k = 1; k <= nv; k++) vstart[k + 1] = vstart[k] + vcnt[k];
  int *velem = xcalloc(4 * (size_t)ne, sizeof(int)), *vnode = xcalloc(4 * (size_t)ne, sizeof(int));
  int *vfill = xcalloc((size_t)nv + 1, sizeof(int));
  for (int e = 0; e < ne; e++)
    for (int c = 0; c < 4; c++) {
      int k = s->knods[s->ngnod * e + c];
      /* head insertion: the last inserted element comes first */
      int pos = vstart[k] + vcnt[k] - 1 - vfill[k]++;
      velem[pos] = e + 1;
      vnode[pos] = c + 1;
    }
  int ek1[4] = {1, 2, 3, 4}, ek2[4] = {2, 3, 4, 1};
  int *econn_e = xcalloc(4 * (size_t)ne, sizeof(int)), *econn_n = xcalloc(4 * (size_t)ne, sizeof(int));
  for (int e = 1; e <= ne; e++)
    for (int nn_ = 1; nn_ <= 4; nn_++) {
      if (econn_e[(nn_ - 1) + 4 * (e - 1)] > 0) continue;
      int k1 = s->knods[(ek1[nn_ - 1] - 1) + s->ngnod * (e - 1)];
      int k2 = s->knods[(ek2[nn_ - 1] - 1) + s->ngnod * (e - 1)];
      int found = 0;
      for (int p1 = vstart[k1]; p1 < vstart[k1 + 1] && !found; p1++) {
        int ee = velem[p1];
        if (ee == e) continue;
        for (int p2 = vstart[k2]; p2 < vstart[k2 + 1]; p2++) {
          if (velem[p2] == ee) {
            int nn2 = vnode[p2];
            econn_e[(nn_ - 1) + 4 * (e - 1)] = ee;
            econn_n[(nn_ - 1) + 4 * (e - 1)] = nn2;
            econn_e[(nn2 - 1) + 4 * (ee - 1)] = e;
            econn_n[(nn2 - 1) + 4 * (ee - 1)] = nn_;
            found = 1;
            break;
          }
        }
      }
    }
  /* SE_init_numbering */
  s->ibool = xcalloc((size_t)n * n * ne, sizeof(int));
  int *iedg = xcalloc(4 * (size_t)n, sizeof(int)), *jedg = xcalloc(4 * (size_t)n, sizeof(int));
  for (int ed = 1; ed <= 4; ed++) edge_ij(n, ed, iedg + n * (ed - 1), jedg + n * (ed - 1));
  int ivtx[4] = {0, n - 1, n - 1, 0}, jvtx[4] = {0, 0, n - 1, n - 1};
  int npoin = 0;
  for (int e = 0; e < ne; e++) {
    for (int j = 1; j < n - 1; j++)
      for (int i = 1; i < n - 1; i++) IB(s, i, j, e) = ++npoin;
    for (int ed = 0; ed < 4; ed++) {
      if (IB(s, iedg[1 + n * ed], jedg[1 + n * ed], e) > 0) continue;
      int ee = econn_e[ed + 4 * e], nn2 = econn_n[ed + 4 * e];
      for (int k = 1; k < n - 1; k++) {
        npoin++;
        IB(s, iedg[k + n * ed], jedg[k + n * ed], e) = npoin;
        if (ee > 0) {
          int kr = n - 1 - k; /* reversed order on the matching edge */
          IB(s, iedg[kr + n * (nn2 - 1)], jedg[kr + n * (nn2 - 1)], ee - 1) = npoin;
        }
      }
    }
    for (int c = 0; c < 4; c++) {
      if (IB(s, ivtx[c], jvtx[c], e) > 0) continue;
      npoin++;
      int k = s->knods[c + s->ngnod * e];
      for (int p = vstart[k]; p < vstart[k + 1]; p++) {
        int c2 = vnode[p] - 1;
        IB(s, ivtx[c2], jvtx[c2], velem[p] - 1) = npoin;
      }
    }
  }
  s->npoin = npoin;
  free(vcnt); free(vstart); free(velem); free(vnode); free(vfill);
  free(econn_e); free(econn_n);
  /* SE_init_coord: coord = matmul(coorg, shape) */
  s->coord = xcalloc(2 * (size_t)npoin, sizeof(double));
  for (int e = 0; e < ne; e++) {
    double c[18];
    elem_coorg(s, e, c);
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        const double *sh = s->shape + ng * (i + n * j);
        int p = IB(s, i, j, e) - 1;
        for (int a = 0; a < 2; a++) {
          double acc = c[a] * sh[0];
          for (int k = 1; k < ng; k++) acc = acc + c[a + 2 * k] * sh[k];
          s->coord[2 * p + a] = acc;
        }
      }
  }
  /* BC_set_bulk_node for each boundary */
  for (int b = 0; b < s->nbnds; b++) {
    oc_bnd *bd = &s->bnds[b];
    bd->ibool = xcalloc((size_t)n * bd->nelem, sizeof(int));
    int *tmpnode = xcalloc((size_t)n * bd->nelem + 1, sizeof(int));
    int *cbulk = xcalloc((size_t)n * bd->nelem + 1, sizeof(int));
    int *cbc = xcalloc((size_t)n * bd->nelem + 1, sizeof(int));
    int ncorner = 0, bnp = 0;
    int it[32], jt[32];
    for (int q = 0; q < bd->nelem; q++) {
      int e = bd->elem[q] - 1;
      edge_ij(n, bd->edge[q], it, jt);
      for (int kl = 0; kl < n; kl++) {
        int bulk = IB(s, it[kl], jt[kl], e), inode = 0, isnew = 1;
        int corner = (kl == 0 || kl == n - 1);
        if (corner)
          for (int c = ncorner - 1; c >= 0; c--)
            if (cbulk[c] == bulk) {
              isnew = 0;
              inode = cbc[c];
              break;
            }
        if (isnew) {
          inode = ++bnp;
          tmpnode[inode] = bulk;
          if (corner) {
            cbulk[ncorner] = bulk;
            cbc[ncorner++] = inode;
          }
        }
        bd->ibool[kl + n * q] = inode;
      }
    }
    bd->npoin = bnp;
    bd->node = xcalloc((size_t)bnp, sizeof(int));
    double *key = xcalloc((size_t)bnp, sizeof(double));
    double xmin = 1e300, xmax = -1e300, zmin = 1e300, zmax = -1e300;
    for (int k = 0; k < bnp; k++) {
      int p = tmpnode[k + 1] - 1;
      double xx = s->coord[2 * p], zz = s->coord[2 * p + 1];
      if (xx < xmin) xmin = xx;
      if (xx > xmax) xmax = xx;
      if (zz < zmin) zmin = zz;
      if (zz > zmax) zmax = zz;
    }
    int use_x = (xmax - xmin) > (zmax - zmin);
    for (int k = 0; k < bnp; k++) key[k] = s->coord[2 * (tmpnode[k + 1] - 1) + (use_x ? 0 : 1)];
    int *isort = xcalloc((size_t)bnp, sizeof(int)), *iback = xcalloc((size_t)bnp + 1, sizeof(int));
    rank_stable(key, bnp, isort);
    for (int k = 0; k < bnp; k++) {
      bd->node[k] = tmpnode[isort[k] + 1];
      iback[isort[k] + 1] = k + 1;
    }
    for (int q = 0; q < n * bd->nelem; q++) bd->ibool[q] = iback[bd->ibool[q]];
    free(key); free(isort); free(iback); free(tmpnode); free(cbulk); free(cbc);
  }
  free(iedg);
  free(jedg);
  return 0;
}

static oc_bnd *find_bnd(oc_setup *s, int tag) {
  for (int b = 0; b < s->nbnds; b++)
    if (s->bnds[b].tag == tag) return &s->bnds[b];
  return NULL;
}

/* BC_get_normal_and_weights (spec_grid.f90:961-1011) */
static void normal_and_weights(oc_setup *s, oc_bnd *bd, double *norm /* (np,2) */, double *w, int periodic) {
  int n = s->ngll, np = bd->npoin;
  int it[32], jt[32];
  for (int k = 0; k < 2 * np; k++) norm[k] = 0.0;
  for (int k = 0; k < np; k++) w[k] = 0.0;
  for (int q = 0; q < bd->nelem; q++) {
    int ed = bd->edge[q], e = bd->elem[q] - 1;
    edge_ij(n, ed, it, jt);
    int ldim = (ed == 1 || ed == 3) ? 0 : 1;
    double sgn = (ed == 3 || ed == 4) ? -1.0 : 1.0;
    double c[18];
    elem_coorg(s, e, c);
    for (int k = 0; k < n; k++) {
      double jac[4];
      jacobian(s, c, it[k], jt[k], jac);
      double dx = jac[0 + 2 * ldim], dz = jac[1 + 2 * ldim];
      double j1 = sqrt(dx * dx + dz * dz);
      double tx = sgn * dx / j1, tz = sgn * dz / j1;
      int bn = bd->ibool[k + n * q] - 1;
      norm[bn] = norm[bn] + tz;
      norm[bn + np] = norm[bn + np] + (-tx);
      w[bn] = w[bn] + s->wgll[k] * j1;
    }
  }
  if (periodic) { /* the two ends are one node (spec_grid.f90:998-1003) */
    for (int c = 0; c < 2; c++) {
      norm[0 + np * c] = norm[0 + np * c] + norm[(np - 1) + np * c];
      norm[(np - 1) + np * c] = norm[0 + np * c];
    }
    w[0] = w[0] + w[np - 1];
    w[np - 1] = w[0];
  }
  for (int q = 0; q < bd->nelem; q++) {
    int ends[2] = {bd->ibool[0 + n * q] - 1, bd->ibool[(n - 1) + n * q] - 1};
    for (int t = 0; t < 2; t++) {
      int bn = ends[t];
      double nrm = sqrt(norm[bn] * norm[bn] + norm[bn + np] * norm[bn + np]);
      norm[bn] = norm[bn] / nrm;
      norm[bn + np] = norm[bn + np] / nrm;
    }
  }
}

/* ------------------------------------------------------------------ */
static const sem2d_material *find_mat(const sem2d_deck *dk, int tag) {
  for (int m = 0; m < dk->nmats; m++)
    if (dk->mats[m].tag == tag) return &dk->mats[m];
  return NULL;
}

/* MAT_init_prop + MAT_ELAST_read/init_elem_prop + MAT_KV (mat_gen.f90:204-303,
 * mat_elastic.f90:69-232, mat_kelvin_voigt.f90:71-134)                */
static int build_materials(oc_setup *s, const sem2d_deck *dk, char *err, int el) {
  size_t np = (size_t)s->ngll * s->ngll * s->nelem, n2 = (size_t)s->ngll * s->ngll;
  s->rho = xcalloc(np, sizeof(double));
  s->cp = xcalloc(np, sizeof(double));
  s->cs = xcalloc(np, sizeof(double));
  s->Kx = xcalloc(np, sizeof(double));
  s->Kz = xcalloc(np, sizeof(double));
  s->la = xcalloc(np, sizeof(double));
  s->mu = xcalloc(np, sizeof(double));
  s->mux = xcalloc(np, sizeof(double));
  s->has_kv = 0;
  for (int m = 0; m < dk->nmats; m++)
    if (dk->mats[m].kv) s->has_kv = 1;
  if (s->has_kv) s->kveta = xcalloc(np, sizeof(double));
  for (int e = 0; e < s->nelem; e++) {
    const sem2d_material *m = find_mat(dk, s->tag[e]);
    if (!m) return seterr(err, el, "element tag %d has no material", s->tag[e]), -1;
    if (!m->hetero && m->rho <= 0.0) return seterr(err, el, "MAT_ELAST_read: undefined density (rho)"), -1;
    if (!m->aniso && !m->hetero && m->cp > 0 && m->cs > 0) {
      double mu = m->rho * m->cs * m->cs, Kmod = m->rho * m->cp * m->cp;
      double lambda = m->rho * (m->cp * m->cp - 2.0 * m->cs * m->cs);
      double poiss = 0.5 * lambda / (Kmod - mu);
      if (poiss < 0.0 || poiss > 0.5) return seterr(err, el, "Poisson's ratio out of range !"), -1;
    }
    for (size_t q = 0; q < n2; q++) {
      size_t p = q + n2 * (size_t)e;
      double rho = m->hetero ? dk->h_rho[p] : m->rho;
      s->rho[p] = rho;
      if (!m->aniso) {
        double cp = m->hetero ? dk->h_cp[p] : m->cp, cs = m->hetero ? dk->h_cs[p] : m->cs;
        double lambda = rho * (cp * cp - 2.0 * cs * cs), mu = rho * cs * cs;
        s->cp[p] = cp;
        s->cs[p] = cs;
        s->la[p] = lambda;
        s->mu[p] = mu;
        s->mux[p] = mu;
        s->Kx[p] = lambda + 2.0 * mu;
        s->Kz[p] = s->Kx[p];
      } else {
        double c11 = m->hetero ? dk->h_c11[p] : m->c11, c13 = m->hetero ? dk->h_c13[p] : m->c13;
        double c33 = m->hetero ? dk->h_c33[p] : m->c33, c55 = m->hetero ? dk->h_c55[p] : m->c55;
        double c66 = m->hetero ? dk->h_c66[p] : m->c66;
        s->la[p] = c13;
        s->mu[p] = c55;
        s->mux[p] = c66;
        s->Kx[p] = c11;
        s->Kz[p] = c33;
        s->cp[p] = sqrt(c11 / rho);
        s->cs[p] = sqrt(c55 / rho);
      }
      if (s->has_kv) s->kveta[p] = m->kv ? (m->hetero && dk->h_kveta ? dk->h_kveta[p] : m->kv_eta) : 0.0;
    }
  }
  return 0;
}

/* CHECK_grid (init.f90:145-289) + TIME_read/TIME_init (time.f90:122-395) */
static int build_time(oc_setup *s, const sem2d_deck *dk, char *err, int el) {
  int n = s->ngll;
  double rlamdamin = 1e308, max_c_dx = 0.0;
  for (int e = 0; e < s->nelem; e++) {
    double c[18];
    elem_coorg(s, e, c);
    double hsq[4];
    hsq[0] = (c[2] - c[0]) * (c[2] - c[0]) + (c[3] - c[1]) * (c[3] - c[1]);
    hsq[1] = (c[4] - c[2]) * (c[4] - c[2]) + (c[5] - c[3]) * (c[5] - c[3]);
    hsq[2] = (c[6] - c[4]) * (c[6] - c[4]) + (c[7] - c[5]) * (c[7] - c[5]);
    hsq[3] = (c[6] - c[0]) * (c[6] - c[0]) + (c[7] - c[1]) * (c[7] - c[1]);
    double mx = hsq[0];
    for (int k = 1; k < 4; k++)
      if (hsq[k] > mx) mx = hsq[k];
    double rdistmax = sqrt(mx);
    const double *cs = s->cs + (size_t)n * n * e, *cp = s->cp + (size_t)n * n * e;
    double csmin = cs[0];
    for (int k = 1; k < n * n; k++)
      if (cs[k] < csmin) csmin = cs[k];
    double rl = csmin / rdistmax;
    if (rl < rlamdamin) rlamdamin = rl;
    const double *cel = s->ndof == 2 ? cp : cs;
    double ratiomax = 0.0;
    for (int j = 0; j < n - 1; j++)
      for (int i = 0; i < n - 1; i++) {
        int p0 = IB(s, i, j, e) - 1, p1 = IB(s, i + 1, j, e) - 1, p2 = IB(s, i, j + 1, e) - 1;
        double x0 = s->coord[2 * p0], z0 = s->coord[2 * p0 + 1];
        double x1 = s->coord[2 * p1], z1 = s->coord[2 * p1 + 1];
        double x2 = s->coord[2 * p2], z2 = s->coord[2 * p2 + 1];
        double r1 = sqrt((x1 - x0) * (x1 - x0) + (z1 - z0) * (z1 - z0));
        double r2 = sqrt((x2 - x0) * (x2 - x0) + (z2 - z0) * (z2 - z0));
        double v = cel[i + n * j] / (r1 < r2 ? r1 : r2);
        if (v > ratiomax) ratiomax = v;
      }
    if (ratiomax > max_c_dx) max_c_dx = ratiomax;
  }
  if ((double)n * rlamdamin / dk->fmax < 5.0)
    return seterr(err, el, "warning: low resolution at fmax (CHECK_grid aborts)"), -1;
  /* TIME_read */
  int nsteps = dk->nsteps;
  double dt = dk->dt, courant = dk->courant, total = dk->total_time;
  if (nsteps < 0 || dt < 0 || total < 0) return seterr(err, el, "TIME: negative setting"), -1;
  if (courant < 0.0 || courant > 0.6) return seterr(err, el, "TIME: Courant out of range [0,0.6]"), -1;
  if ((double)nsteps * total != 0.0)
    return seterr(err, el, "TIME: bad combination of settings, NbSteps or TotalTime"), -1;
  if (dt > 0.0) {
    if (total > 0.0) nsteps = (int)ceil(total / dt);
    total = dt * nsteps;
  }
  s->time_kind = dk->time_kind;
  double omega_max = 2.0;
  s->beta = 0.0;
  s->gamma = 0.5;
  s->alpha = 1.0;
  if (dk->time_kind == SEM2D_TIME_NEWMARK) {
    s->beta = dk->beta;
    s->gamma = dk->gamma;
    if (s->beta < 0 || s->beta > 1 || s->gamma < 0 || s->gamma > 1)
      return seterr(err, el, "TIME_NEWMARK: parameter out of range"), -1;
    omega_max = sqrt(2.0 / s->gamma);
  } else if (dk->time_kind == SEM2D_TIME_HHT) {
    /* TIME_read, case 'HHT-alpha' (time.f90:222-240) */
    double a = dk->hht_alpha, r = dk->hht_rho;
    if (a < 0.0 || a > 1.0) return seterr(err, el, "TIME_HHTA: alpha is out of range [0,1]"), -1;
    if (r < 0.5 || r > 1.0) return seterr(err, el, "TIME_HHTA: rho is out of range [0.5,1]"), -1;
    s->alpha = a;
    s->gamma = 1.5 - a;
    double r2 = r * r, r3 = r2 * r, r4 = r3 * r, r5 = r4 * r, q = 1.0 + r;
    s->beta = (a != 1.0) ? 1.0 - a - r * r * (r - 1.0) / ((1.0 - a) * (q * q * q)) : 0.0;
    omega_max = sqrt(-4.0 * q * q * q * q * q / (r5 + 9.0 * r4 - 34.0 * r3 + 6.0 * r2 - 15.0 * r + 1.0));
  }
  /* TIME_init */
  double grid_cfl = max_c_dx;
  if (dt > 0.0) {
    courant = grid_cfl * dt;
  } else {
    dt = courant / grid_cfl;
    if (total > 0.0) nsteps = (int)ceil(total / dt);
    total = nsteps * dt;
  }
  double critical = omega_max * 3.0 / 7.0 / sqrt(2.0);
  if (courant > critical) return seterr(err, el, "warning: Courant number too high (TIME_init aborts)"), -1;
  s->dt = dt;
  s->courant = courant;
  s->nt = nsteps;
  s->total = total;
  return 0;
}

/* ------------------------------------------------------------------ */
/* TIME_getCoefA2V/A2D/A2Vrhs (time.f90:426-486); alpha = 1 for Newmark */
static int newmark_like(const oc_setup *s) {
  return s->time_kind == SEM2D_TIME_NEWMARK || s->time_kind == SEM2D_TIME_HHT;
}
static double coefA2V(const oc_setup *s) { return newmark_like(s) ? s->gamma * s->dt : s->dt; }
static double coefA2D(const oc_setup *s) { return newmark_like(s) ? s->beta * s->dt * s->dt : 0.0; }
static double coefA2Vrhs(const oc_setup *s) {
  return newmark_like(s) ? s->alpha * coefA2V(s) : 0.5 * coefA2V(s);
}

/* MAT_MASS_init (mat_mass.f90:29-61) */
static void build_mass(oc_setup *s) {
  int n = s->ngll, nd = s->ndof;
  s->rmass = xcalloc((size_t)s->npoin * nd, sizeof(double));
  for (int e = 0; e < s->nelem; e++) {
    double c[18];
    elem_coorg(s, e, c);
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        double jac[4];
        jacobian(s, c, i, j, jac);
        double dvol = jac[0] * jac[3] - jac[2] * jac[1];
        dvol = dvol * (s->wgll[i] * s->wgll[j]);
        double ml = s->rho[i + n * j + (size_t)n * n * e] * dvol;
        int p = IB(s, i, j, e) - 1;
        s->rmass[p] = s->rmass[p] + ml;
      }
  }
  if (nd == 2)
    for (int p = 0; p < s->npoin; p++) s->rmass[p + s->npoin] = s->rmass[p];
}

/* BC_ABSO_init (bc_abso.f90:115-266) */
/* append one Stacey P3 term (BC_ABSO_init, bc_abso.f90:174-218) */
static void st_push(oc_setup *s, int node, int k, const int *edge, double K0, double K1) {
  int n = s->ngll, m = s->nst + 1;
  s->st_node = realloc(s->st_node, (size_t)m * sizeof(int));
  s->st_k = realloc(s->st_k, (size_t)m * sizeof(int));
  s->st_edge = realloc(s->st_edge, (size_t)m * n * sizeof(int));
  s->st_K = realloc(s->st_K, (size_t)m * sizeof(double));
  s->st_K1 = realloc(s->st_K1, (size_t)m * sizeof(double));
  s->st_node[s->nst] = node;
  s->st_k[s->nst] = k;
  memcpy(s->st_edge + (size_t)s->nst * n, edge, (size_t)n * sizeof(int));
  s->st_K[s->nst] = K0;
  s->st_K1[s->nst] = K1;
  s->nst = m;
}

/* SE_InverseJacobian (invert2, utils.f90:88-110) and SE_VolumeWeights
 * (spec_grid.f90:590-602) at every element GLL point of a grid that is not
 * flat */
static int build_general_geometry(oc_setup *s, char *err, int el) {
  int n = s->ngll;
  size_t npt = (size_t)n * n * s->nelem;
  s->xjaci = xcalloc(4 * npt, sizeof(double));
  s->dvol = xcalloc(npt, sizeof(double));
  for (int e = 0; e < s->nelem; e++) {
    double c[18];
    elem_coorg(s, e, c);
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        double jac[4];
        jacobian(s, c, i, j, jac);
        double det = jac[0] * jac[3] - jac[2] * jac[1];
        if (det <= 0.0) return seterr(err, el, "SE_InverseJacobian: undefined Jacobian"), -1;
        size_t q = i + (size_t)n * j + (size_t)n * n * e;
        s->xjaci[4 * q + 0] = jac[3] / det;
        s->xjaci[4 * q + 1] = -jac[1] / det;
        s->xjaci[4 * q + 2] = -jac[2] / det;
        s->xjaci[4 * q + 3] = jac[0] / det;
        s->dvol[q] = det * (s->wgll[i] * s->wgll[j]);
      }
  }
  return 0;
}

/* BC_PERIO_intersects (bc_periodic.f90:108-121) */
static int perio_intersects(const oc_setup *s, const oc_bnd *bd) {
  int first = 0, last = 0;
  for (int k = 0; k < s->nper; k++) {
    if (s->per_m[k] == bd->node[0] || s->per_s[k] == bd->node[0]) first = 1;
    if (s->per_m[k] == bd->node[bd->npoin - 1] || s->per_s[k] == bd->node[bd->npoin - 1]) last = 1;
  }
  return s->nper > 0 && bd->npoin > 0 && first && last;
}

/* BC_PERIO_init (bc_periodic.f90:42-72): pair the two sides' nodes in list
 * order, check the shift, sum the mass on the master and copy it */
static int perio_init(oc_setup *s, const int *tags, char *err, int el) {
  oc_bnd *m = find_bnd(s, tags[0]), *q = find_bnd(s, tags[1]);
  if (!m || !q) return seterr(err, el, "bc_perio_init: boundary tag not found"), -1;
  if (m->nelem != q->nelem) return seterr(err, el, "bc_perio_init: number of boundary elements do not match"), -1;
  if (m->npoin != q->npoin) return seterr(err, el, "bc_perio_init: number of nodes on boundaries do not match"), -1;
  const double *c0m = s->coord + 2 * (size_t)(m->node[0] - 1), *c0s = s->coord + 2 * (size_t)(q->node[0] - 1);
  double sh1 = c0m[0] - c0s[0], sh2 = c0m[1] - c0s[1];
  for (int k = 0; k < m->npoin; k++) {
    const double *cm = s->coord + 2 * (size_t)(m->node[k] - 1), *cs = s->coord + 2 * (size_t)(q->node[k] - 1);
    if (fabs(cm[0] - cs[0] - sh1) > TINY_XABS || fabs(cm[1] - cs[1] - sh2) > TINY_XABS)
      return seterr(err, el, "bc_perio_init: coordinates on boundaries do not match properly"), -1;
  }
  for (int d = 0; d < s->ndof; d++)
    for (int k = 0; k < m->npoin; k++) {
      double *a = &s->rmass[(size_t)(m->node[k] - 1) + (size_t)s->npoin * d];
      double *b = &s->rmass[(size_t)(q->node[k] - 1) + (size_t)s->npoin * d];
      *a = *a + *b;
      *b = *a;
    }
  s->nper = m->npoin;
  s->per_m = xcalloc((size_t)s->nper, sizeof(int));
  s->per_s = xcalloc((size_t)s->nper, sizeof(int));
  memcpy(s->per_m, m->node, (size_t)s->nper * sizeof(int));
  memcpy(s->per_s, q->node, (size_t)s->nper * sizeof(int));
  return 0;
}

/* STF_read (stf_gen.f90:45-97) and the *_read checks; the REAL namelist
 * variables of &STF_RICKER, &STF_GAUSSIAN, &STF_HARMONIC and &STF_USER
 * hold FP32 values (stf_ricker.f90:51, stf_gaussian.f90:44,
 * stf_harmonic.f90:41, stf_user.f90:46) */
static int read_stf(oc_setup *s, const sem2d_stf *in, sem2d_stf *out, char *err, int el) {
  *out = *in;
  switch (in->kind) {
    case SEM2D_STF_RICKER: {
      float f0 = (float)in->f0, onset = (float)in->onset, ampli = (float)in->ampli;
      if (f0 <= 0.0f) return seterr(err, el, "RICKER_read: f0 must be positive"), -1;
      if (onset < 1.0f / f0) return seterr(err, el, "warning: RICKER_read: Onset time too small"), -1;
      out->f0 = (double)f0;
      out->onset = (double)onset;
      out->ampli = (double)ampli;
      return 0;
    }
    case SEM2D_STF_GAUSSIAN: {
      float f0 = (float)in->f0, onset = (float)in->onset, ampli = (float)in->ampli;
      if (f0 < 0.0f) return seterr(err, el, "STF_GAUSSIAN_read: f0 must be positive"), -1;
      out->f0 = (double)f0;
      out->onset = (double)onset;
      out->ampli = (double)ampli;
      return 0;
    }
    case SEM2D_STF_BRUNE:
      if (in->f0 < 0.0) return seterr(err, el, "STF_BRUNE_read: fc must be positive"), -1;
      return 0;
    case SEM2D_STF_HARMONIC: {
      float ampli = (float)in->ampli, f0 = (float)in->f0;
      if (f0 <= 0.0f) return seterr(err, el, "STF_HARMONIC_read: f0 must be positive"), -1;
      if (ampli == 0.0f) return seterr(err, el, "STF_HARMONIC_read: ampli must be non zero"), -1;
      out->ampli = (double)ampli;
      out->f0 = (double)f0;
      return 0;
    }
    case SEM2D_STF_USER:
      out->onset = (double)(float)in->onset;
      out->ampli = (double)(float)in->ampli;
      out->par1 = (double)(float)in->par1;
      out->par2 = (double)(float)in->par2;
      return 0;
    case SEM2D_STF_TAB: {
      int n = in->ntab;
      if (n < 2 || !in->tab_t || !in->tab_v) return seterr(err, el, "STF_TAB_read: the table needs two rows or more"), -1;
      if (s->ntabs + 2 > (int)(sizeof(s->tabs) / sizeof(s->tabs[0]))) return seterr(err, el, "too many tables"), -1;
      double *t = xcalloc((size_t)n, sizeof(double)), *v = xcalloc((size_t)n, sizeof(double));
      memcpy(t, in->tab_t, (size_t)n * sizeof(double));
      memcpy(v, in->tab_v, (size_t)n * sizeof(double));
      s->tabs[s->ntabs++] = t;
      s->tabs[s->ntabs++] = v;
      out->tab_t = t;
      out->tab_v = v;
      for (int k = 1; k < n; k++)
        if (!(t[k] > t[k - 1])) return seterr(err, el, "STF_TAB_read: times must increase"), -1;
      return 0;
    }
    default:
      return seterr(err, el, "STF_read: unknown source time function "), -1;
  }
}

/* BC_DIRNEU_init (bc_dirneu.f90:117-143): the components flagged 'D', and
 * the time functions of the Neumann components (bc_DIRNEU_apply :157-167;
 * a Dirichlet component drops its own, :70-101) */
static int dirneu_init(oc_setup *s, const sem2d_bc *bc, int after, char *err, int el) {
  const int tag = bc->tag[0], mask = bc->dirichlet;
  oc_bnd *bd = find_bnd(s, tag);
  if (!bd) return 0;
  int np = bd->npoin;
  double *norm = xcalloc(2 * (size_t)np, sizeof(double)), *w = xcalloc((size_t)np, sizeof(double));
  normal_and_weights(s, bd, norm, w, perio_intersects(s, bd));
  int horiz = 1, vert = 1;
  for (int k = 0; k < np; k++) {
    if (!(fabs(norm[k]) < TINY_XABS)) horiz = 0;
    if (!(fabs(norm[k + np]) < TINY_XABS)) vert = 0;
  }
  free(norm);
  if (!horiz && !vert) {
    free(w);
    return seterr(err, el, "BC_DIRNEU_init: boundary is not vertical or horizontal"), -1;
  }
  for (int c = 0; c < s->ndof; c++) {
    if (!((mask >> c) & 1)) continue;
    int m = s->ndir + np;
    s->dir_node = realloc(s->dir_node, (size_t)m * sizeof(int));
    s->dir_comp = realloc(s->dir_comp, (size_t)m * sizeof(int));
    s->dir_after = realloc(s->dir_after, (size_t)m * sizeof(int));
    for (int k = 0; k < np; k++) {
      s->dir_node[s->ndir + k] = bd->node[k];
      s->dir_comp[s->ndir + k] = c;
      s->dir_after[s->ndir + k] = after;
    }
    s->ndir = m;
  }
  for (int c = 0; c < s->ndof; c++) {
    const sem2d_stf *in = c == 0 ? &bc->hstf : &bc->vstf;
    if (((mask >> c) & 1) || in->kind == SEM2D_STF_NONE) continue;
    int q = s->nneu_stf;
    if (read_stf(s, in, &s->neu_stfs[q], err, el)) {
      free(w);
      return -1;
    }
    s->nneu_stf = q + 1;
    int m = s->nneu + np;
    s->neu_node = realloc(s->neu_node, (size_t)m * sizeof(int));
    s->neu_comp = realloc(s->neu_comp, (size_t)m * sizeof(int));
    s->neu_stf = realloc(s->neu_stf, (size_t)m * sizeof(int));
    s->neu_B = realloc(s->neu_B, (size_t)m * sizeof(double));
    for (int k = 0; k < np; k++) {
      s->neu_node[s->nneu + k] = bd->node[k];
      s->neu_comp[s->nneu + k] = c;
      s->neu_stf[s->nneu + k] = q;
      s->neu_B[s->nneu + k] = w[k];
    }
    s->nneu = m;
  }
  free(w);
  return 0;
}

static int abso_init(oc_setup *s, int tag, int stacey, int wave, char *err, int el) {
  oc_bnd *bd = find_bnd(s, tag);
  if (!bd) return 0;
  int n = s->ngll, nd = s->ndof, np = bd->npoin;
  const int periodic = perio_intersects(s, bd);
  double *norm = xcalloc(2 * (size_t)np, sizeof(double)), *w = xcalloc((size_t)np, sizeof(double));
  normal_and_weights(s, bd, norm, w, periodic);
  int flat = 1, gtan = 0, gnor = 1;
  int horiz = 1, vert = 1;
  for (int k = 0; k < np; k++) {
    if (!(fabs(norm[k]) < TINY_XABS)) horiz = 0;
    if (!(fabs(norm[k + np]) < TINY_XABS)) vert = 0;
  }
  if (horiz) { gtan = 0; gnor = 1; }
  else if (vert) { gtan = 1; gnor = 0; }
  else { flat = 0; gtan = 1; gnor = 0; }
  if (!flat) {
    free(norm); free(w);
    return seterr(err, el, "absorbing boundary is not flat"), -1;
  }
  double *C = xcalloc((size_t)np * nd, sizeof(double));
  int it[32], jt[32];
  for (int q = 0; q < bd->nelem; q++) {
    int e = bd->elem[q] - 1, ed = bd->edge[q];
    edge_ij(n, ed, it, jt);
    int ldim = (ed == 1 || ed == 3) ? 0 : 1;
    double c8[18];
    elem_coorg(s, e, c8);
    for (int k = 0; k < n; k++) {
      size_t p = it[k] + n * jt[k] + (size_t)n * n * e;
      double rho = s->rho[p], c[2];
      c[gnor] = s->cp[p];
      c[gtan] = s->cs[p];
      double jac[4];
      jacobian(s, c8, it[k], jt[k], jac);
      double ci = s->wgll[k] * sqrt(jac[0 + 2 * ldim] * jac[0 + 2 * ldim] + jac[1 + 2 * ldim] * jac[1 + 2 * ldim]);
      int bk = bd->ibool[k + n * q] - 1;
      if (nd == 1) {
        C[bk] = C[bk] + rho * c[gtan] * ci;
      } else {
        C[bk] = C[bk] + rho * c[0] * ci;
        C[bk + np] = C[bk + np] + rho * c[1] * ci;
      }
      if (stacey && nd == 2) {
        /* K(k,1,e) = CoefIntegr dloc_t/dx_t rho cs (2 cs - cp); K(:,2) = K(:,1);
         * the tangential component negated */
        double det = jac[0] * jac[3] - jac[2] * jac[1];
        double inv[2][2] = {{jac[3] / det, -jac[2] / det}, {-jac[1] / det, jac[0] / det}};
        double K0 = ci * inv[ldim][gtan] * (rho * c[gtan] * (2.0 * c[gtan] - c[gnor]));
        int edge[32];
        for (int l = 0; l < n; l++) edge[l] = bd->node[bd->ibool[l + n * q] - 1];
        st_push(s, bd->node[bk], k, edge, gtan == 0 ? -K0 : K0, gtan == 1 ? -K0 : K0);
      }
    }
  }
  if (periodic) /* the two ends are one node (bc_abso.f90:227-231) */
    for (int d = 0; d < nd; d++) {
      C[0 + np * d] = C[0 + np * d] + C[(np - 1) + np * d];
      C[(np - 1) + np * d] = C[0 + np * d];
    }
  double cf = coefA2Vrhs(s);
  for (int d = 0; d < nd; d++)
    for (int k = 0; k < np; k++) {
      int p = bd->node[k] - 1;
      s->rmass[p + (size_t)s->npoin * d] = s->rmass[p + (size_t)s->npoin * d] + cf * C[k + np * d];
    }
  /* append to the absorbing entry list, with B, the normal and whether the
   * wave source enters (let_wave on a flat side, bc_abso.f90:245-256) */
  int na = s->nabs + np;
  s->abs_node = realloc(s->abs_node, (size_t)na * sizeof(int));
  s->abs_B = realloc(s->abs_B, (size_t)na * sizeof(double));
  s->abs_nx = realloc(s->abs_nx, (size_t)na * sizeof(double));
  s->abs_nz = realloc(s->abs_nz, (size_t)na * sizeof(double));
  s->abs_wave = realloc(s->abs_wave, (size_t)na * sizeof(int));
  for (int k = 0; k < np; k++) {
    s->abs_B[s->nabs + k] = w[k];
    s->abs_nx[s->nabs + k] = norm[k];
    s->abs_nz[s->nabs + k] = norm[k + np];
    s->abs_wave[s->nabs + k] = wave;
  }
  double *nc = xcalloc((size_t)na * nd, sizeof(double));
  for (int d = 0; d < nd; d++)
    for (int k = 0; k < s->nabs; k++) nc[k + (size_t)na * d] = s->abs_C[k + (size_t)s->nabs * d];
  for (int k = 0; k < np; k++) {
    s->abs_node[s->nabs + k] = bd->node[k];
    for (int d = 0; d < nd; d++) nc[s->nabs + k + (size_t)na * d] = C[k + np * d];
  }
  free(s->abs_C);
  s->abs_C = nc;
  s->nabs = na;
  free(norm); free(w); free(C);
  return 0;
}

static double fparam(const sem2d_deck *dk, int which, int k) {
  return dk->flt_array[which] ? dk->flt_array[which][k] : dk->flt_value[which];
}

static long nint_ref(double x) { return (long)(x >= 0 ? floor(x + 0.5) : -floor(-x + 0.5)); }

/* BC_DYNFLT_init (bc_dynflt.f90:231-520) */
static int dynflt_init(oc_setup *s, const sem2d_deck *dk, const int *tags, char *err, int el) {
  if (s->nflt) return seterr(err, el, "only one DYNFLT boundary is supported"), -1;
  oc_bnd *b1 = find_bnd(s, tags[0]), *b2 = tags[1] > 0 ? find_bnd(s, tags[1]) : NULL;
  if (!b1) return 0;
  int nd = s->ndof, two = tags[1] > 0;
  if (two && !b2) return 0;
  if (two && (b1->nelem != b2->nelem || b1->npoin != b2->npoin))
    return seterr(err, el, "bc_dynflt_init: boundaries do not match"), -1;
  int np = b1->npoin;
  if (two)
    for (int k = 0; k < b1->npoin; k++)
      if (b1->node[k] == b2->node[k]) np--;
  s->two_sides = two;
  s->nflt = np;
  s->node1 = xcalloc((size_t)np, sizeof(int));
  s->node2 = xcalloc((size_t)np, sizeof(int));
  double *tn = xcalloc(2 * (size_t)b1->npoin, sizeof(double)), *tb = xcalloc((size_t)b1->npoin, sizeof(double));
  normal_and_weights(s, b1, tn, tb, perio_intersects(s, b1));
  s->n1 = xcalloc(2 * (size_t)np, sizeof(double));
  s->B = xcalloc((size_t)np, sizeof(double));
  int j = 0;
  for (int k = 0; k < b1->npoin; k++) {
    if (two && b1->node[k] == b2->node[k]) continue;
    s->node1[j] = b1->node[k];
    s->node2[j] = two ? b2->node[k] : 0;
    s->B[j] = tb[k];
    s->n1[j] = tn[k];
    s->n1[j + np] = tn[k + b1->npoin];
    j++;
  }
  free(tn); free(tb);
  s->fcoord = xcalloc(2 * (size_t)np, sizeof(double));
  for (int k = 0; k < np; k++) {
    int p = s->node1[k] - 1;
    s->fcoord[2 * k] = s->coord[2 * p];
    s->fcoord[2 * k + 1] = s->coord[2 * p + 1];
    if (two) {
      int q = s->node2[k] - 1;
      if (fabs(s->coord[2 * p] - s->coord[2 * q]) > TINY_XABS ||
          fabs(s->coord[2 * p + 1] - s->coord[2 * q + 1]) > TINY_XABS)
        return seterr(err, el, "bc_dynflt_init: coordinates on boundaries do not match properly"), -1;
    }
  }
  s->coefA2V = coefA2V(s);
  s->coefA2D = coefA2D(s);
  s->invM1 = xcalloc((size_t)np * nd, sizeof(double));
  s->invM2 = xcalloc((size_t)np * nd, sizeof(double));
  s->Z = xcalloc((size_t)np * nd, sizeof(double));
  for (int d = 0; d < nd; d++)
    for (int k = 0; k < np; k++) {
      s->invM1[k + np * d] = 1.0 / s->rmass[(s->node1[k] - 1) + (size_t)s->npoin * d];
      if (two) s->invM2[k + np * d] = 1.0 / s->rmass[(s->node2[k] - 1) + (size_t)s->npoin * d];
      if (two)
        s->Z[k + np * d] = 1.0 / (s->coefA2V * s->B[k] * (s->invM1[k + np * d] + s->invM2[k + np * d]));
      else
        s->Z[k + np * d] = 0.5 / (s->coefA2V * s->B[k] * s->invM1[k + np * d]);
    }
  for (int q = 0; q < SEM2D_FP_NPARAM; q++) {
    s->prm[q] = xcalloc((size_t)np, sizeof(double));
    for (int k = 0; k < np; k++) s->prm[q][k] = fparam(dk, q, k);
  }
  s->T0 = xcalloc(2 * (size_t)np, sizeof(double));
  s->coh = xcalloc((size_t)np, sizeof(double));
  for (int k = 0; k < np; k++) {
    double nx = s->n1[k], nz = s->n1[k + np];
    double Sxx = s->prm[SEM2D_FP_SXX][k], Sxy = s->prm[SEM2D_FP_SXY][k], Sxz = s->prm[SEM2D_FP_SXZ][k];
    double Syz = s->prm[SEM2D_FP_SYZ][k], Szz = s->prm[SEM2D_FP_SZZ][k];
    double Tx = Sxx * nx + Sxz * nz, Ty = Sxy * nx + Syz * nz, Tz = Sxz * nx + Szz * nz;
    if (nd == 1)
      s->T0[k] = s->prm[SEM2D_FP_TT][k] + Ty;
    else
      s->T0[k] = s->prm[SEM2D_FP_TT][k] + Tx * nz - Tz * nx;
    s->T0[k + np] = s->prm[SEM2D_FP_TN][k] + Tx * nx + Tz * nz;
    s->coh[k] = s->prm[SEM2D_FP_COHESION][k];
    if (s->coh[k] < 0.0) return seterr(err, el, "bc_dynflt_init: cohesion must be positive"), -1;
  }
  /* output sampling */
  int oix1 = dk->flt_oxi[0] > 1 ? dk->flt_oxi[0] : 1;
  int oixn = dk->flt_oxi[1] > 0 && dk->flt_oxi[1] < np ? dk->flt_oxi[1] : np;
  int oixd = dk->flt_oxi[2] > 0 ? dk->flt_oxi[2] : 1;
  long oitd = nint_ref(dk->flt_otd / s->dt);
  s->oitd = oitd > 1 ? (int)oitd : 1;
  s->oit = (int)nint_ref(dk->flt_ot1 / s->dt);
  s->oix1 = oix1;
  s->oixn = oixn;
  s->oixd = oixd;
  s->fnsamp = (s->nt - s->oit) / s->oitd + 1;
  return 0;
}

/* SE_find_nearest_node (spec_grid.f90:410-435): the last node at the
 * minimum distance wins ('<=') */
static int nearest_node(const oc_setup *s, const double *xz, double *dist) {
  double d2min = 1.7976931348623157e308;
  int ig = 0;
  for (int p = 0; p < s->npoin; p++) {
    double dx = xz[0] - s->coord[2 * p], dz = xz[1] - s->coord[2 * p + 1];
    double d2 = dx * dx + dz * dz;
    if (d2 <= d2min) {
      d2min = d2;
      ig = p + 1;
    }
  }
  if (dist) *dist = sqrt(d2min);
  return ig;
}

static void invert2(const double *A, double *B) {
  double det = A[0] * A[3] - A[2] * A[1];
  B[0] = A[3] / det;
  B[1] = -A[1] / det;
  B[2] = -A[2] / det;
  B[3] = A[0] / det;
}

/* SE_find_point + FE_find_point (spec_grid.f90:471-497, fem_grid.f90:451-501) */
static int find_point(const oc_setup *s, const double *xz, int *eout, double *xi, double *eta,
                      double *newc) {
  int ig = nearest_node(s, xz, NULL);
  int n = s->ngll;
  for (int e = 0; e < s->nelem; e++)
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) {
        if (IB(s, i, j, e) != ig) continue;
        /* first (e,i,j) holding the node: FE_find_point always reports
         * success because it tests the initial guess (fem_grid.f90:490) */
        double c[18];
        elem_coorg(s, e, c);
        int ng = s->ngnod;
        double x1 = c[0] - c[4], x2 = c[1] - c[5], y1 = c[2] - c[6], y2 = c[3] - c[7];
        double area = 0.5 * fabs(x1 * y2 - x2 * y1);
        double esize = sqrt(area / PI_REF);
        double tolx = TINY_XABS, tolf = TINY_XABS * esize;
        double X[2] = {s->xgll[i], s->xgll[j]};
        int it;
        for (it = 1; it <= 100; it++) {
          double sh[9], ds[18], fv[2], fj[4], fi[4];
          shape_n(ng, X[0], X[1], sh);
          for (int a = 0; a < 2; a++) {
            double acc = c[a] * sh[0];
            for (int k = 1; k < ng; k++) acc = acc + c[a + 2 * k] * sh[k];
            fv[a] = acc - xz[a];
          }
          dershape_n(ng, X[0], X[1], ds);
          for (int b = 0; b < 2; b++)
            for (int a = 0; a < 2; a++) {
              double acc = c[a] * ds[ng * b];
              for (int k = 1; k < ng; k++) acc = acc + c[a + 2 * k] * ds[k + ng * b];
              fj[a + 2 * b] = acc;
            }
          if (fabs(fv[0]) + fabs(fv[1]) <= tolf) break;
          double p0 = -fv[0], p1 = -fv[1];
          invert2(fj, fi);
          double q0 = fi[0] * p0 + fi[2] * p1, q1 = fi[1] * p0 + fi[3] * p1;
          X[0] = X[0] + q0;
          X[1] = X[1] + q1;
          if (fabs(q0) + fabs(q1) <= tolx) break;
        }
        if (it >= 100) return -1;
        *eout = e + 1;
        *xi = X[0];
        *eta = X[1];
        double sh[9];
        shape_n(ng, *xi, *eta, sh);
        for (int a = 0; a < 2; a++) {
          double acc = c[a] * sh[0];
          for (int k = 1; k < ng; k++) acc = acc + c[a + 2 * k] * sh[k];
          newc[a] = acc;
        }
        return 0;
      }
  return -1;
}

/* REC_read + REC_init + REC_posit (receivers.f90:62-303) */
static int rec_init(oc_setup *s, const sem2d_deck *dk, char *err, int el) {
  int nx = dk->rec_number;
  if (nx <= 0) return 0;
  double *rc = xcalloc(2 * (size_t)nx, sizeof(double));
  if (dk->rec_coord) {
    memcpy(rc, dk->rec_coord, 2 * (size_t)nx * sizeof(double));
  } else if (nx > 1) {
    for (int i = 1; i <= nx; i++)
      for (int a = 0; a < 2; a++)
        rc[2 * (i - 1) + a] = dk->rec_first[a] + ((double)(i - 1) / (double)(nx - 1)) *
                                                     (dk->rec_last[a] - dk->rec_first[a]);
  } else {
    rc[0] = dk->rec_first[0];
    rc[1] = dk->rec_first[1];
  }
  s->rec_isamp = dk->rec_isamp > 0 ? dk->rec_isamp : 1;
  s->rec_field = dk->rec_field ? dk->rec_field : 'V';
  s->rec_atnode = dk->rec_atnode;
  int n2 = s->ngll * s->ngll;
  if (dk->rec_atnode) {
    int *ig = xcalloc((size_t)nx, sizeof(int)), irec = 0;
    for (int k = 0; k < nx; k++) {
      int ip = nearest_node(s, rc + 2 * k, NULL), dup = 0;
      if (irec > 1)
        for (int q = 0; q < irec; q++)
          if (ig[q] == ip) dup = 1;
      if (dup) continue;
      ig[irec++] = ip;
    }
    s->nrec = irec;
    s->rec_node = ig;
    s->rec_coord = xcalloc(2 * (size_t)irec, sizeof(double));
    for (int k = 0; k < irec; k++) {
      s->rec_coord[2 * k] = s->coord[2 * (ig[k] - 1)];
      s->rec_coord[2 * k + 1] = s->coord[2 * (ig[k] - 1) + 1];
    }
  } else {
    s->nrec = nx;
    s->rec_elem = xcalloc((size_t)nx, sizeof(int));
    s->rec_interp = xcalloc((size_t)n2 * nx, sizeof(double));
    s->rec_coord = xcalloc(2 * (size_t)nx, sizeof(double));
    for (int k = 0; k < nx; k++) {
      double xi, eta, nc[2];
      int e;
      if (find_point(s, rc + 2 * k, &e, &xi, &eta, nc) != 0) {
        free(rc);
        return seterr(err, el, "SE_find_point: point not found"), -1;
      }
      s->rec_elem[k] = e;
      int q = 0;
      for (int j = 0; j < s->ngll; j++) {
        double fj = oc_hgll(j, eta, s->xgll, s->ngll);
        for (int i = 0; i < s->ngll; i++) {
          double fi = oc_hgll(i, xi, s->xgll, s->ngll);
          s->rec_interp[q++ + (size_t)n2 * k] = fi * fj;
        }
      }
      s->rec_coord[2 * k] = nc[0];
      s->rec_coord[2 * k + 1] = nc[1];
    }
  }
  free(rc);
  s->rec_nsamp = s->nt / s->rec_isamp + 1;
  return 0;
}

/* SO_read + RICKER_read + FORCE_read + SO_init (src_gen.f90:83-262,
 * stf_ricker.f90:46-80, src_force.f90:36-63) */
/* SRC_MOMENT_read / SRC_MOMENT_init / SRC_MOMENT_add (src_moment.f90:27-175):
 * in every element holding the source node (i, j) the row of nodes (:, j)
 * gets G(c,1) h'_l(xi_i) and the column (i, :) gets G(c,2) h'_l(eta_j),
 * G = M jac_inv^T (SH: G = jac_inv M(:,1)); the coefficients are summed per
 * node (in order of first appearance) into point forces */
static int moment_init(oc_setup *s, const sem2d_deck *dk, double f0, double onset, double amp, char *err, int el) {
  int nd = s->ndof, n = s->ngll, ns = dk->nsrc;
  double M[2][2] = {{0, 0}, {0, 0}};
  if (dk->src_mech == 1) {
    if (nd != 2) return seterr(err, el, "SRC_MOMENT_read: explosion only allowed in PSV (ndof=2)"), -1;
    M[0][0] = 1.0;
    M[1][1] = 1.0;
  } else if (dk->src_mech == 2) {
    double dip = dk->src_dip * PI_REF / 180.0, n0 = sin(dip), n1 = cos(dip);
    if (nd == 2) {
      double r0 = -cos(dip), r1 = sin(dip);
      M[0][0] = 2.0 * r0 * n0;
      M[0][1] = r0 * n1 + r1 * n0;
      M[1][0] = M[0][1];
      M[1][1] = 2.0 * r1 * n1;
    } else {
      M[0][0] = n0;
      M[1][0] = n1;
    }
  } else if (dk->src_mech == 3) {
    if (nd == 2) {
      M[0][0] = dk->src_M[0]; M[0][1] = dk->src_M[1]; M[1][0] = dk->src_M[2]; M[1][1] = dk->src_M[3];
    } else {
      M[0][0] = dk->src_M[0];
      M[1][0] = dk->src_M[1];
    }
  } else {
    return seterr(err, el, "unknown source mechanism"), -1;
  }
  int cap = 4 * 2 * n * ns + 1, cnt = 0;
  int *node = xcalloc((size_t)cap, sizeof(int));
  double *F = xcalloc(2 * (size_t)cap, sizeof(double)), *rel = xcalloc((size_t)cap, sizeof(double)),
         *td = xcalloc((size_t)cap, sizeof(double));
  for (int k = 0; k < ns; k++) {
    int src = nearest_node(s, dk->src_coord + 2 * k, NULL), first = cnt;
    for (int e = 0; e < s->nelem; e++)
      for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++) {
          if (s->ibool[i + n * (j + (size_t)n * e)] != src) continue;
          double c8[18], J[4];
          elem_coorg(s, e, c8);
          jacobian(s, c8, i, j, J);
          double det = J[0] * J[3] - J[2] * J[1];
          double inv[2][2] = {{J[3] / det, -J[2] / det}, {-J[1] / det, J[0] / det}};
          double G[2][2];
          if (nd == 2) {
            for (int a = 0; a < 2; a++)
              for (int b = 0; b < 2; b++) G[a][b] = M[a][0] * inv[b][0] + M[a][1] * inv[b][1];
          } else {
            G[0][0] = inv[0][0] * M[0][0] + inv[0][1] * M[1][0];
            G[0][1] = inv[1][0] * M[0][0] + inv[1][1] * M[1][0];
            G[1][0] = G[1][1] = 0.0;
          }
          for (int l = 0; l < n; l++) {
            double hx = s->H[l + n * i], he = s->H[l + n * j];
            int nodes2[2] = {s->ibool[l + n * (j + (size_t)n * e)], s->ibool[i + n * (l + (size_t)n * e)]};
            double fx[2] = {G[0][0] * hx, G[0][1] * he}, fz[2] = {G[1][0] * hx, G[1][1] * he};
            for (int t = 0; t < 2; t++) {
              int q = first;
              while (q < cnt && node[q] != nodes2[t]) q++;
              if (q == cnt) {
                node[cnt] = nodes2[t];
                F[2 * cnt] = 0.0;
                F[2 * cnt + 1] = 0.0;
                rel[cnt] = dk->src_ampli ? dk->src_ampli[k] : 1.0;
                td[cnt] = dk->src_tdelay ? dk->src_tdelay[k] : 0.0;
                cnt++;
              }
              F[2 * q] += fx[t];
              F[2 * q + 1] += fz[t];
            }
          }
        }
  }
  s->nsrc = cnt;
  s->src_node = node;
  s->src_dir = xcalloc(2 * (size_t)cnt, sizeof(double));
  s->src_f0 = xcalloc((size_t)cnt, sizeof(double));
  s->src_t0 = xcalloc((size_t)cnt, sizeof(double));
  s->src_amp = xcalloc((size_t)cnt, sizeof(double));
  s->src_rel = rel;
  s->src_tdelay = td;
  for (int q = 0; q < cnt; q++) {
    if (nd == 2) {
      s->src_dir[2 * q] = F[2 * q];
      s->src_dir[2 * q + 1] = F[2 * q + 1];
    } else { /* SH: the force is the amplitude itself */
      s->src_dir[2 * q] = 1.0;
      s->src_rel[q] = s->src_rel[q] * F[2 * q];
    }
    s->src_f0[q] = (double)f0;
    s->src_t0[q] = (double)onset;
    s->src_amp[q] = (double)amp;
  }
  free(F);
  return 0;
}

/* WAVE_read + WAVE_init (src_wave.f90:78-180): the angle brought into
 * [-180, 180], the reference point at the node nearest the domain corner
 * the wave enters first, the material at the first element point of that
 * node (SE_node_belongs_to, spec_grid.f90:441-456).  The reference
 * computes that corner and then searches from wave%coord, which it never
 * sets; the corner is what its comments and input documentation describe. */
static int wave_init(oc_setup *s, const sem2d_deck *dk, const sem2d_stf *stf, char *err, int el) {
  double angle = dk->wave_angle + 180.0;
  angle = angle - floor(angle / 360.0) * 360.0 - 180.0;
  if (dk->wave_phase != SEM2D_WAVE_P && dk->wave_phase != SEM2D_WAVE_S)
    return seterr(err, el, "WAVE_read: phase must be S or P"), -1;
  double xmin = s->coord[0], xmax = s->coord[0], zmin = s->coord[1], zmax = s->coord[1];
  for (int p = 0; p < s->npoin; p++) {
    double x = s->coord[2 * p], z = s->coord[2 * p + 1];
    if (x < xmin) xmin = x;
    if (x > xmax) xmax = x;
    if (z < zmin) zmin = z;
    if (z > zmax) zmax = z;
  }
  double corner[2];
  corner[0] = angle >= 0.0 ? xmax : xmin;
  corner[1] = fabs(angle) < 90.0 ? zmin : zmax;
  int ig = nearest_node(s, corner, NULL), n = s->ngll;
  size_t at = 0;
  int found = 0;
  for (int e = 0; e < s->nelem && !found; e++)
    for (int j = 0; j < n && !found; j++)
      for (int i = 0; i < n && !found; i++)
        if (IB(s, i, j, e) == ig) {
          at = i + n * (j + (size_t)n * e);
          found = 1;
        }
  const sem2d_material *m = find_mat(dk, s->tag[at / ((size_t)n * n)]);
  if (m && m->aniso) return seterr(err, el, "MAT_getProp: the incident wave needs mu and lambda of an isotropic material"), -1;
  double rho = s->rho[at], cp = s->cp[at], cs = s->cs[at];
  s->wave_phase = dk->wave_phase;
  s->wave_angle = angle;
  s->wave_ref[0] = s->coord[2 * (size_t)(ig - 1)];
  s->wave_ref[1] = s->coord[2 * (size_t)(ig - 1) + 1];
  s->wave_cp = cp;
  s->wave_cs = cs;
  s->wave_mu = rho * cs * cs;
  s->wave_lambda = rho * (cp * cp - 2.0 * cs * cs);
  s->wave_tdelay = dk->src_tdelay ? dk->src_tdelay[0] : 0.0;
  s->wave_stf = *stf;
  return 0;
}

static int src_init(oc_setup *s, const sem2d_deck *dk, char *err, int el) {
  int ns = dk->nsrc;
  if (ns <= 0) return 0;
  /* the time function all sources share (src_gen.f90:150-158) */
  sem2d_stf in = dk->stf, stf;
  if (in.kind == SEM2D_STF_NONE) {
    in.kind = SEM2D_STF_RICKER;
    in.f0 = dk->ricker_f0;
    in.onset = dk->ricker_onset;
    in.ampli = dk->ricker_ampli;
  }
  if (read_stf(s, &in, &stf, err, el)) return -1;
  if (dk->src_mech == 4) return wave_init(s, dk, &stf, err, el);
  if (stf.kind != SEM2D_STF_RICKER) {
    s->has_src_stf = 1;
    s->src_stf = stf;
  }
  /* the values of the time function as read (Ricker: already FP32) */
  double f0 = stf.f0, onset = stf.onset, amp = stf.ampli;
  double ang = dk->force_angle * PI_REF / 180.0;
  if (dk->src_mech != 0) return moment_init(s, dk, f0, onset, amp, err, el);
  s->nsrc = ns;
  s->src_node = xcalloc((size_t)ns, sizeof(int));
  s->src_dir = xcalloc(2 * (size_t)ns, sizeof(double));
  s->src_f0 = xcalloc((size_t)ns, sizeof(double));
  s->src_t0 = xcalloc((size_t)ns, sizeof(double));
  s->src_amp = xcalloc((size_t)ns, sizeof(double));
  s->src_rel = xcalloc((size_t)ns, sizeof(double));
  s->src_tdelay = xcalloc((size_t)ns, sizeof(double));
  for (int k = 0; k < ns; k++) {
    s->src_node[k] = nearest_node(s, dk->src_coord + 2 * k, NULL);
    s->src_dir[2 * k] = -sin(ang);
    s->src_dir[2 * k + 1] = cos(ang);
    s->src_f0[k] = (double)f0;
    s->src_t0[k] = (double)onset;
    s->src_amp[k] = (double)amp;
    s->src_rel[k] = dk->src_ampli ? dk->src_ampli[k] : 1.0;
    s->src_tdelay[k] = dk->src_tdelay ? dk->src_tdelay[k] : 0.0;
  }
  return 0;
}

/* ------------------------------------------------------------------ */
oc_setup *oc_grid_build(const sem2d_deck *dk, char *err, int el) {
  oc_setup *s = xcalloc(1, sizeof(oc_setup));
  s->deck = dk;
  if (dk->ndof != 1 && dk->ndof != 2) {
    seterr(err, el, "ndof must be 1 or 2");
    oc_setup_free(s);
    return NULL;
  }
  s->ndof = dk->ndof;
  if (build_mesh(s, dk, err, el) || build_grid(s, dk, err, el)) {
    oc_setup_free(s);
    return NULL;
  }
  return s;
}

oc_setup *oc_setup_build(const sem2d_deck *dk, char *err, int el) {
  oc_setup *s = oc_grid_build(dk, err, el);
  if (!s) return NULL;
  if (build_materials(s, dk, err, el) || build_time(s, dk, err, el)) goto fail;
  if (s->has_kv) {
    /* MAT_KV_init_elem_work: eta*dt when ETAxDT */
    int n2 = s->ngll * s->ngll;
    for (int e = 0; e < s->nelem; e++) {
      const sem2d_material *m = find_mat(dk, s->tag[e]);
      if (m->kv && m->kv_etaxdt)
        for (int q = 0; q < n2; q++) s->kveta[q + (size_t)n2 * e] = s->dt * s->kveta[q + (size_t)n2 * e];
    }
  }
  build_mass(s);
  if (!s->flat && build_general_geometry(s, err, el)) goto fail;
  /* BC_init: periodic sides first (bc_gen.f90:221-228), then the &BC_DEF
   * order, which decides the mass snapshot of the fault */
  for (int b = 0; b < dk->nbcs; b++)
    if (dk->bcs[b].kind == SEM2D_BC_PERIOD) {
      if (s->nper) {
        seterr(err, el, "more than one pair of periodic sides");
        goto fail;
      }
      if (perio_init(s, dk->bcs[b].tag, err, el)) goto fail;
    }
  int fault_seen = 0;
  for (int b = 0; b < dk->nbcs; b++) {
    const sem2d_bc *bc = &dk->bcs[b];
    if (bc->kind == SEM2D_BC_ABSORB) {
      if (abso_init(s, bc->tag[0], bc->stacey, !bc->no_wave && dk->nsrc > 0 && dk->src_mech == 4, err, el))
        goto fail;
    } else if (bc->kind == SEM2D_BC_DYNFLT) {
      if (dynflt_init(s, dk, bc->tag, err, el)) goto fail;
      fault_seen = 1;
    } else if (bc->kind == SEM2D_BC_DIRNEU) {
      if (dirneu_init(s, bc, fault_seen, err, el)) goto fail;
    }
  }
  if (rec_init(s, dk, err, el) || src_init(s, dk, err, el)) goto fail;
  if (s->nst) {  /* Stacey K(nst,2): the first components, then the second */
    s->st_K = realloc(s->st_K, 2 * (size_t)s->nst * sizeof(double));
    memcpy(s->st_K + s->nst, s->st_K1, (size_t)s->nst * sizeof(double));
  }
  if (s->nabs) {
    s->abs_n = xcalloc(2 * (size_t)s->nabs, sizeof(double));
    memcpy(s->abs_n, s->abs_nx, (size_t)s->nabs * sizeof(double));
    memcpy(s->abs_n + s->nabs, s->abs_nz, (size_t)s->nabs * sizeof(double));
  }
  /* invert the mass matrix (init.f90:112-116) */
  for (size_t q = 0; q < (size_t)s->npoin * s->ndof; q++) s->rmass[q] = 1.0 / s->rmass[q];
  return s;
fail:
  oc_setup_free(s);
  return NULL;
}

void oc_setup_free(oc_setup *s) {
  if (!s) return;
  free(s->fem_coord); free(s->knods); free(s->tag);
  for (int b = 0; b < s->nbnds; b++) {
    free(s->bnds[b].elem); free(s->bnds[b].edge); free(s->bnds[b].node); free(s->bnds[b].ibool);
  }
  free(s->xgll); free(s->wgll); free(s->H); free(s->shape); free(s->dshape);
  free(s->ibool); free(s->coord);
  free(s->rho); free(s->cp); free(s->cs); free(s->Kx); free(s->Kz); free(s->la); free(s->mu);
  free(s->mux); free(s->kveta); free(s->rmass); free(s->abs_node); free(s->abs_C);
  free(s->st_node); free(s->st_k); free(s->st_edge); free(s->st_K); free(s->st_K1);
  free(s->per_m); free(s->per_s); free(s->dir_node); free(s->dir_comp); free(s->dir_after);
  free(s->node1); free(s->node2); free(s->fcoord); free(s->n1); free(s->B); free(s->invM1);
  free(s->invM2); free(s->Z); free(s->T0); free(s->coh);
  for (int q = 0; q < SEM2D_FP_NPARAM; q++) free(s->prm[q]);
  free(s->src_node); free(s->src_dir); free(s->src_f0); free(s->src_t0); free(s->src_amp);
  free(s->src_rel); free(s->src_tdelay); free(s->rec_node); free(s->rec_elem); free(s->rec_interp);
  free(s->rec_coord);
  free(s->abs_B); free(s->abs_nx); free(s->abs_nz); free(s->abs_n); free(s->abs_wave);
  free(s->neu_node); free(s->neu_comp); free(s->neu_stf); free(s->neu_B);
  for (int q = 0; q < s->ntabs; q++) free(s->tabs[q]);
  free(s->xjaci); free(s->dvol);
  free(s);
}

void oc_setup_sizes(const oc_setup *s, int *nelem, int *npoin, int *ngll) {
  if (nelem) *nelem = s->nelem;
  if (npoin) *npoin = s->npoin;
  if (ngll) *ngll = s->ngll;
}
void oc_setup_ibool(const oc_setup *s, int *ib) {
  memcpy(ib, s->ibool, (size_t)s->ngll * s->ngll * s->nelem * sizeof(int));
}
void oc_setup_coord(const oc_setup *s, double *c) { memcpy(c, s->coord, 2 * (size_t)s->npoin * sizeof(double)); }
void oc_setup_tags(const oc_setup *s, int *t) { memcpy(t, s->tag, (size_t)s->nelem * sizeof(int)); }
void oc_setup_knods(const oc_setup *s, int *k) {
  for (int e = 0; e < s->nelem; e++) memcpy(k + 4 * (size_t)e, s->knods + (size_t)s->ngnod * e, 4 * sizeof(int));
}
int oc_setup_boundary(const oc_setup *s, int tag, int *nodes) {
  for (int b = 0; b < s->nbnds; b++)
    if (s->bnds[b].tag == tag) {
      if (nodes) memcpy(nodes, s->bnds[b].node, (size_t)s->bnds[b].npoin * sizeof(int));
      return s->bnds[b].npoin;
    }
  return 0;
}
void oc_setup_time(const oc_setup *s, double *dt, int *nt, double *courant) {
  if (dt) *dt = s->dt;
  if (nt) *nt = s->nt;
  if (courant) *courant = s->courant;
}
int oc_setup_rec_coord(const oc_setup *s, double *c) {
  if (c && s->nrec) memcpy(c, s->rec_coord, 2 * (size_t)s->nrec * sizeof(double));
  return s->nrec;
}
int oc_setup_fault_coord(const oc_setup *s, double *c) {
  if (c && s->nflt) memcpy(c, s->fcoord, 2 * (size_t)s->nflt * sizeof(double));
  return s->nflt;
}

int oc_setup_desc(const oc_setup *s, sem2d_problem_desc *d) {
  memset(d, 0, sizeof(*d));
  const sem2d_deck *dk = s->deck;
  d->ngll = s->ngll;
  d->ndof = s->ndof;
  d->nelem = s->nelem;
  d->npoin = s->npoin;
  d->ibool = s->ibool;
  d->coord = s->coord;
  d->hprime = s->H;
  d->wgll = s->wgll;
  d->Kx = s->Kx;
  d->Kz = s->Kz;
  d->la = s->la;
  d->mu = s->mu;
  d->mux = s->mux;
  d->kv_eta = s->has_kv ? s->kveta : NULL;
  d->kd2_form = dk->kd2_form >= 0 ? dk->kd2_form : (s->ngll == 5);
  d->rmass = s->rmass;
  d->nabs = s->nabs;
  d->abs_node = s->abs_node;
  d->abs_C = s->abs_C;
  d->nstacey = s->nst;
  d->stacey_node = s->st_node;
  d->stacey_k = s->st_k;
  d->stacey_edge = s->st_edge;
  d->stacey_K = s->st_K;
  d->nperio = s->nper;
  d->perio_master = s->per_m;
  d->perio_slave = s->per_s;
  d->ndir = s->ndir;
  d->dir_node = s->dir_node;
  d->dir_comp = s->dir_comp;
  d->dir_after_fault = s->dir_after;
  d->time_scheme = s->time_kind;
  d->dt = s->dt;
  d->beta = s->beta;
  d->gamma = s->gamma;
  d->alpha = s->alpha;
  d->nt = s->nt;
  d->nsrc = s->nsrc;
  d->src_node = s->src_node;
  d->src_dir = s->src_dir;
  d->src_f0 = s->src_f0;
  d->src_t0 = s->src_t0;
  d->src_ampli = s->src_amp;
  d->src_relamp = s->src_rel;
  d->src_tdelay = s->src_tdelay;
  d->nrec = s->nrec;
  d->rec_field = s->rec_field;
  d->rec_isamp = s->rec_isamp > 0 ? s->rec_isamp : 1;
  d->rec_nsamp = s->rec_nsamp;
  d->rec_node = s->rec_node;
  d->rec_elem = s->rec_elem;
  d->rec_interp = s->rec_interp;
  d->nflt = s->nflt;
  if (s->nflt) {
    d->flt_node1 = s->node1;
    d->flt_node2 = s->two_sides ? s->node2 : NULL;
    d->flt_n1 = s->n1;
    d->flt_B = s->B;
    d->flt_invM1 = s->invM1;
    d->flt_invM2 = s->two_sides ? s->invM2 : NULL;
    d->flt_Z = s->Z;
    d->flt_T0 = s->T0;
    d->flt_cohesion = s->coh;
    d->flt_coefA2V = s->coefA2V;
    d->flt_coefA2D = s->coefA2D;
    d->flt_opening = dk->flt_opening;
    d->flt_friction = dk->flt_friction;
    d->swf_kind = dk->swf_kind;
    d->swf_healing = dk->swf_healing;
    d->swf_dc = s->prm[SEM2D_FP_SWF_DC];
    d->swf_mus = s->prm[SEM2D_FP_SWF_MUS];
    d->swf_mud = s->prm[SEM2D_FP_SWF_MUD];
    d->swf_p = s->prm[SEM2D_FP_SWF_P];
    d->swf_alpha = s->prm[SEM2D_FP_SWF_ALPHA];
    d->rsf_kind = dk->rsf_kind;
    d->rsf_dc = s->prm[SEM2D_FP_RSF_DC];
    d->rsf_mus = s->prm[SEM2D_FP_RSF_MUS];
    d->rsf_a = s->prm[SEM2D_FP_RSF_A];
    d->rsf_b = s->prm[SEM2D_FP_RSF_B];
    d->rsf_vstar = s->prm[SEM2D_FP_RSF_VSTAR];
    d->rsf_vc = s->prm[SEM2D_FP_RSF_VC];
    d->rsf_theta = s->prm[SEM2D_FP_RSF_THETA];
    d->flt_V0 = s->prm[SEM2D_FP_V0];
    d->normal_kind = dk->normal_kind;
    d->normal_T = dk->normal_T;
    d->normal_L = dk->normal_L;
    d->normal_V = dk->normal_V;
    d->flt_oit = s->oit;
    d->flt_oitd = s->oitd;
    d->flt_oix1 = s->oix1;
    d->flt_oixn = s->oixn;
    d->flt_oixd = s->oixd;
    d->flt_nsamp = s->fnsamp;
  }
  d->precision = dk->precision;
  d->width = dk->width;
  d->rho = s->rho;
  if (s->nflt) {
    d->twf_kind = dk->flt_friction == SEM2D_FRICTION_TWF && dk->twf_kind == 0 ? 1 : dk->twf_kind;
    d->twf_mus = dk->twf_mus;
    d->twf_mud = dk->twf_mud;
    d->twf_mu0 = dk->twf_mu0;
    d->twf_X = dk->twf_X;
    d->twf_Z = dk->twf_Z;
    d->twf_V = dk->twf_V;
    d->twf_L = dk->twf_L;
    d->twf_T = dk->twf_T;
    d->twf_Dc = dk->twf_Dc;
    d->flt_potency = dk->flt_potency;
  }
  d->src_stf = s->has_src_stf ? &s->src_stf : NULL;
  d->wave_phase = s->wave_phase;
  if (s->wave_phase) {
    d->wave_angle = s->wave_angle;
    d->wave_ref[0] = s->wave_ref[0];
    d->wave_ref[1] = s->wave_ref[1];
    d->wave_cp = s->wave_cp;
    d->wave_cs = s->wave_cs;
    d->wave_mu = s->wave_mu;
    d->wave_lambda = s->wave_lambda;
    d->wave_tdelay = s->wave_tdelay;
    d->wave_stf = &s->wave_stf;
    d->abs_wave = s->abs_wave;
  }
  d->abs_B = s->abs_B;
  d->abs_n = s->abs_n;
  d->nneu = s->nneu;
  d->neu_node = s->neu_node;
  d->neu_comp = s->neu_comp;
  d->neu_B = s->neu_B;
  d->neu_stf = s->neu_stf;
  d->nneu_stf = s->nneu_stf;
  d->neu_stfs = s->nneu_stf ? s->neu_stfs : NULL;
  d->xjaci = s->xjaci;
  d->dvol = s->dvol;
  return 0;
}

/*
 * ORACLE (test infrastructure only -- never part of the product path).
 *
 * Gauss-Lobatto-Legendre points, weights and Lagrange derivative matrix,
 * restating SRC/gll.f90 of SEM2DPACK step by step (same recurrences and
 * operation order, FP64, no FMA contraction):
 *   get_GLL_info  gll.f90:19-36     jacobf  gll.f90:386-438
 *   endw1/endw2   gll.f90:87-197    pndleg  gll.f90:442-474
 *   gammaf        gll.f90:199-228   pnleg   gll.f90:478-504
 *   hdgll         gll.f90:230-265   pnormj  gll.f90:508-547
 *   hgll          gll.f90:269-296   zwgjd   gll.f90:551-618
 *   jacg          gll.f90:300-382   zwgljd  gll.f90:622-684
 */
#include <math.h>
#include "sem2d_oracle.h"

static double gammaf(double x) {
  const double pi = 3.141592653589793;
  double g = 1.0;
  if (x == -0.5) g = -2.0 * sqrt(pi);
  if (x == 0.5) g = sqrt(pi);
  if (x == 1.0) g = 1.0;
  if (x == 2.0) g = 1.0;
  if (x == 1.5) g = sqrt(pi) / 2.0;
  if (x == 2.5) g = 1.5 * sqrt(pi) / 2.0;
  if (x == 3.5) g = 2.5 * 1.5 * sqrt(pi) / 2.0;
  if (x == 3.0) g = 2.0;
  if (x == 4.0) g = 6.0;
  if (x == 5.0) g = 24.0;
  if (x == 6.0) g = 120.0;
  return g;
}

static double endw1(int n, double alpha, double beta) {
  double apb = alpha + beta, f1, fint1, fint2, f2, f3 = 0.0;
  if (n == 0) return 0.0;
  f1 = gammaf(alpha + 2.0) * gammaf(beta + 1.0) / gammaf(apb + 3.0);
  f1 = f1 * (apb + 2.0) * pow(2.0, apb + 2.0) / 2.0;
  if (n == 1) return f1;
  fint1 = gammaf(alpha + 2.0) * gammaf(beta + 1.0) / gammaf(apb + 3.0);
  fint1 = fint1 * pow(2.0, apb + 2.0);
  fint2 = gammaf(alpha + 2.0) * gammaf(beta + 2.0) / gammaf(apb + 4.0);
  fint2 = fint2 * pow(2.0, apb + 3.0);
  f2 = (-2.0 * (beta + 2.0) * fint1 + (apb + 4.0) * fint2) * (apb + 3.0) / 4.0;
  if (n == 2) return f2;
  for (int i = 3; i <= n; i++) {
    double di = (double)(i - 1), abn = alpha + beta + di, abnn = abn + di;
    double a1 = -(2.0 * (di + alpha) * (di + beta)) / (abn * abnn * (abnn + 1.0));
    double a2 = (2.0 * (alpha - beta)) / (abnn * (abnn + 2.0));
    double a3 = (2.0 * (abn + 1.0)) / ((abnn + 2.0) * (abnn + 1.0));
    f3 = -(a2 * f2 + a1 * f1) / a3;
    f1 = f2;
    f2 = f3;
  }
  return f3;
}

static double endw2(int n, double alpha, double beta) {
  double apb = alpha + beta, f1, fint1, fint2, f2, f3 = 0.0;
  if (n == 0) return 0.0;
  f1 = gammaf(alpha + 1.0) * gammaf(beta + 2.0) / gammaf(apb + 3.0);
  f1 = f1 * (apb + 2.0) * pow(2.0, apb + 2.0) / 2.0;
  if (n == 1) return f1;
  fint1 = gammaf(alpha + 1.0) * gammaf(beta + 2.0) / gammaf(apb + 3.0);
  fint1 = fint1 * pow(2.0, apb + 2.0);
  fint2 = gammaf(alpha + 2.0) * gammaf(beta + 2.0) / gammaf(apb + 4.0);
  fint2 = fint2 * pow(2.0, apb + 3.0);
  f2 = (2.0 * (alpha + 2.0) * fint1 - (apb + 4.0) * fint2) * (apb + 3.0) / 4.0;
  if (n == 2) return f2;
  for (int i = 3; i <= n; i++) {
    double di = (double)(i - 1), abn = alpha + beta + di, abnn = abn + di;
    double a1 = -(2.0 * (di + alpha) * (di + beta)) / (abn * abnn * (abnn + 1.0));
    double a2 = (2.0 * (alpha - beta)) / (abnn * (abnn + 2.0));
    double a3 = (2.0 * (abn + 1.0)) / ((abnn + 2.0) * (abnn + 1.0));
    f3 = -(a2 * f2 + a1 * f1) / a3;
    f1 = f2;
    f2 = f3;
  }
  return f3;
}

/* Jacobi polynomial of degree n and its derivative at x, plus the two
 * previous degrees (gll.f90:386-438). */
static void jacobf(double *poly, double *pder, double *polym1, double *pderm1,
                   double *polym2, double *pderm2, int n, double alp,
                   double bet, double x) {
  double apb = alp + bet, polyl, pderl, psave = 0.0, pdsave = 0.0;
  *poly = 1.0;
  *pder = 0.0;
  if (n == 0) return;
  polyl = *poly;
  pderl = *pder;
  *poly = (alp - bet + (apb + 2.0) * x) / 2.0;
  *pder = (apb + 2.0) / 2.0;
  if (n == 1) return;
  for (int k = 2; k <= n; k++) {
    double dk = (double)k;
    double a1 = 2.0 * dk * (dk + apb) * (2.0 * dk + apb - 2.0);
    double a2 = (2.0 * dk + apb - 1.0) * (alp * alp - bet * bet);
    double b3 = (2.0 * dk + apb - 2.0);
    double a3 = b3 * (b3 + 1.0) * (b3 + 2.0);
    double a4 = 2.0 * (dk + alp - 1.0) * (dk + bet - 1.0) * (2.0 * dk + apb);
    double polyn = ((a2 + a3 * x) * (*poly) - a4 * polyl) / a1;
    double pdern = ((a2 + a3 * x) * (*pder) - a4 * pderl + a3 * (*poly)) / a1;
    psave = polyl;
    pdsave = pderl;
    polyl = *poly;
    *poly = polyn;
    pderl = *pder;
    *pder = pdern;
  }
  *polym1 = polyl;
  *pderm1 = pderl;
  *polym2 = psave;
  *pderm2 = pdsave;
}

/* np Gauss-Jacobi points by Newton with deflation (gll.f90:300-382). */
static void jacg(double *xjac, int np, double alpha, double beta) {
  const int kstop = 10;
  const double eps = 1.0e-12;
  double p = 0, pd = 0, pm1 = 0, pdm1 = 0, pm2 = 0, pdm2 = 0, xlast = 0.0;
  int n = np - 1, jmin = 0;
  double dth = 4.0 * atan(1.0) / (2.0 * (double)n + 2.0);
  for (int j = 1; j <= np; j++) {
    double x;
    if (j == 1) {
      x = cos((2.0 * ((double)j - 1.0) + 1.0) * dth);
    } else {
      double x1 = cos((2.0 * ((double)j - 1.0) + 1.0) * dth);
      double x2 = xlast;
      x = (x1 + x2) / 2.0;
    }
    for (int k = 1; k <= kstop; k++) {
      jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, np, alpha, beta, x);
      double recsum = 0.0;
      for (int i = 1; i <= j - 1; i++) recsum = recsum + 1.0 / (x - xjac[np - i]);
      double delx = -p / (pd - recsum * p);
      x = x + delx;
      if (fabs(delx) < eps) break;
    }
    xjac[np - j] = x;
    xlast = x;
  }
  for (int i = 1; i <= np; i++) {
    double xmin = 2.0;
    for (int j = i; j <= np; j++) {
      if (xjac[j - 1] < xmin) {
        xmin = xjac[j - 1];
        jmin = j;
      }
    }
    if (jmin != i) {
      double swap = xjac[i - 1];
      xjac[i - 1] = xjac[jmin - 1];
      xjac[jmin - 1] = swap;
    }
  }
}

static double pnormj(int n, double alpha, double beta) {
  double dn = (double)n, cst = alpha + beta + 1.0, prod;
  if (n <= 1) {
    prod = gammaf(dn + alpha) * gammaf(dn + beta);
    prod = prod / (gammaf(dn) * gammaf(dn + alpha + beta));
    return prod * pow(2.0, cst) / (2.0 * dn + cst);
  }
  prod = gammaf(alpha + 1.0) * gammaf(beta + 1.0);
  prod = prod / (2.0 * (1.0 + cst) * gammaf(cst + 1.0));
  prod = prod * (1.0 + alpha) * (2.0 + alpha);
  prod = prod * (1.0 + beta) * (2.0 + beta);
  for (int i = 3; i <= n; i++) {
    double dindx = (double)i;
    double frac = (dindx + alpha) * (dindx + beta) / (dindx * (dindx + alpha + beta));
    prod = prod * frac;
  }
  return prod * pow(2.0, cst) / (2.0 * dn + cst);
}

static void zwgjd(double *z, double *w, int np, double alpha, double beta) {
  double p = 0, pd = 0, pm1 = 0, pdm1 = 0, pm2 = 0, pdm2 = 0;
  int n = np - 1;
  double apb = alpha + beta;
  if (np == 1) {
    z[0] = (beta - alpha) / (apb + 2.0);
    w[0] = gammaf(alpha + 1.0) * gammaf(beta + 1.0) / gammaf(apb + 2.0) *
           pow(2.0, apb + 1.0);
    return;
  }
  jacg(z, np, alpha, beta);
  int np1 = n + 1, np2 = n + 2;
  double dnp1 = (double)np1, dnp2 = (double)np2;
  double fac1 = dnp1 + alpha + beta + 1.0;
  double fac2 = fac1 + dnp1;
  double fac3 = fac2 + 1.0;
  double fnorm = pnormj(np1, alpha, beta);
  double rcoef = (fnorm * fac2 * fac3) / (2.0 * fac1 * dnp2);
  for (int i = 0; i < np; i++) {
    jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, np2, alpha, beta, z[i]);
    w[i] = -rcoef / (p * pdm1);
  }
}

static void zwgljd(double *z, double *w, int np, double alpha, double beta) {
  double p = 0, pd = 0, pm1 = 0, pdm1 = 0, pm2 = 0, pdm2 = 0;
  int n = np - 1, nm1 = n - 1;
  if (nm1 > 0) zwgjd(z + 1, w + 1, nm1, alpha + 1.0, beta + 1.0);
  z[0] = -1.0;
  z[np - 1] = 1.0;
  for (int i = 2; i <= np - 1; i++) w[i - 1] = w[i - 1] / (1.0 - z[i - 1] * z[i - 1]);
  jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, n, alpha, beta, z[0]);
  w[0] = endw1(n, alpha, beta) / (2.0 * pd);
  jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, n, alpha, beta, z[np - 1]);
  w[np - 1] = endw2(n, alpha, beta) / (2.0 * pd);
}

double oc_pnleg(double z, int n) {
  double p1 = 1.0, p2 = z, p3 = p2;
  for (int k = 1; k <= n - 1; k++) {
    double fk = (double)k;
    p3 = ((2.0 * fk + 1.0) * z * p2 - fk * p1) / (fk + 1.0);
    p1 = p2;
    p2 = p3;
  }
  return p3;
}

double oc_pndleg(double z, int n) {
  double p1 = 1.0, p2 = z, p1d = 0.0, p2d = 1.0, p3d = 1.0;
  for (int k = 1; k <= n - 1; k++) {
    double fk = (double)k;
    double p3 = ((2.0 * fk + 1.0) * z * p2 - fk * p1) / (fk + 1.0);
    p3d = ((2.0 * fk + 1.0) * p2 + (2.0 * fk + 1.0) * z * p2d - fk * p1d) / (fk + 1.0);
    p1 = p2;
    p2 = p3;
    p1d = p2d;
    p2d = p3d;
  }
  return p3d;
}

/* derivative of the i-th Lagrange interpolant at zgll[j] (0-based) */
static double hdgll(int i, int j, const double *zgll, int nz) {
  int idegpoly = nz - 1;
  if (i == 0 && j == 0) return -(double)idegpoly * ((double)idegpoly + 1.0) / 4.0;
  if (i == idegpoly && j == idegpoly) return (double)idegpoly * ((double)idegpoly + 1.0) / 4.0;
  if (i == j) return 0.0;
  double r1 = oc_pnleg(zgll[j], idegpoly);
  double r2 = oc_pndleg(zgll[j], idegpoly);
  double r3 = oc_pnleg(zgll[i], idegpoly);
  return r1 / (r3 * (zgll[j] - zgll[i])) +
         (1.0 - zgll[j] * zgll[j]) * r2 /
             ((double)idegpoly * ((double)idegpoly + 1.0) * r3 * (zgll[j] - zgll[i]) *
              (zgll[j] - zgll[i]));
}

double oc_hgll(int i, double z, const double *zgll, int nz) {
  const double eps = 1.0e-5;
  double dz = z - zgll[i];
  if (fabs(dz) < eps) return 1.0;
  int n = nz - 1;
  double alfan = (double)n * ((double)n + 1.0);
  return -(1.0 - z * z) * oc_pndleg(z, n) / (alfan * oc_pnleg(zgll[i], n) * (z - zgll[i]));
}

void oc_gll_info(int n, double *x, double *w, double *H) {
  zwgljd(x, w, n, 0.0, 0.0);
  if (n % 2 != 0) x[(n - 1) / 2] = 0.0;
  for (int ix = 0; ix < n; ix++)
    for (int ip = 0; ip < n; ip++) H[ip + n * ix] = hdgll(ip, ix, x, n);
}

// stf.cuh -- source time functions of the GPU library (STF_get,
// stf_gen.f90:99-121), evaluated on the host for the per-step tables of
// the point sources and on the device for the boundary forces whose phase
// differs from node to node (the incident plane wave).
#pragma once

#include <cmath>
#include <vector>

#include "../../include/sem2d_gpu.h"

struct StfDev {
  int kind, ntab;
  double f0, onset, ampli, par1, par2;
  const double *t, *v, *v2;  // TAB rows and spline second derivatives
};

// The products are grouped as the reference writes them (Fortran evaluates
// a*b*c as (a*b)*c and -a*b as -(a*b)).
__host__ __device__ inline double stf_value(const StfDev &s, double t) {
  const double kPi = 3.141592653589793;
  switch (s.kind) {
    case SEM2D_STF_RICKER: {  // stf_ricker.f90:89-103
      double a = kPi * s.f0 * (t - s.onset);
      a = a * a;
      return -((s.ampli * (1.0 - 2.0 * a)) * exp(-a));
    }
    case SEM2D_STF_GAUSSIAN: {  // stf_gaussian.f90:76-86
      double a = kPi * s.f0 * (t - s.onset);
      a = a * a;
      return s.ampli * exp(-a);
    }
    case SEM2D_STF_BRUNE: {  // stf_brune.f90:73-83
      const double a = 2.0 * kPi * s.f0 * (t > 0.0 ? t : 0.0);
      return s.ampli * (1.0 - (1.0 + a) * exp(-a));
    }
    case SEM2D_STF_HARMONIC:  // stf_harmonic.f90:68-77
      return s.ampli * sin(2.0 * kPi * t * s.f0);
    case SEM2D_STF_USER: {  // stf_user.f90:110-122
      const double a = t - s.onset;
      return s.ampli * sin(a) + s.par1 * (a * a);
    }
    case SEM2D_STF_TAB: {  // stf_tabulated.f90:83-95, splint utils.f90:697-734
      const int n = s.ntab;
      double x = t < s.t[0] ? s.t[0] : t;
      x = x > s.t[n - 1] ? s.t[n - 1] : x;
      // the row before x: largest k with t[k] < x, within [0, n-2]
      int lo = 0, hi = n - 1;
      while (hi - lo > 1) {
        const int m = (lo + hi) >> 1;
        if (x > s.t[m]) lo = m; else hi = m;
      }
      const double h = s.t[hi] - s.t[lo];
      const double a = (s.t[hi] - x) / h, b = (x - s.t[lo]) / h;
      return a * s.v[lo] + b * s.v[hi] + ((a * a * a - a) * s.v2[lo] + (b * b * b - b) * s.v2[hi]) * (h * h) / 6.0;
    }
    default:
      return 0.0;
  }
}

// Second derivatives of the cubic spline through (t, v) with zero slope at
// both ends (spline, utils.f90:652-691, called with yp1 = ypn = 0 by
// STF_TAB_read, stf_tabulated.f90:66).
inline std::vector<double> stf_spline_d2(const double *x, const double *y, int n) {
  std::vector<double> y2(n, 0.0), u(n, 0.0);
  y2[0] = -0.5;
  u[0] = (3.0 / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - 0.0);
  for (int i = 1; i < n - 1; ++i) {
    const double sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1]);
    const double p = sig * y2[i - 1] + 2.0;
    y2[i] = (sig - 1.0) / p;
    u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1])) /
                (x[i + 1] - x[i - 1]) -
            sig * u[i - 1]) /
           p;
  }
  const double qn = 0.5;
  const double un = (3.0 / (x[n - 1] - x[n - 2])) * (0.0 - (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]));
  y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.0);
  for (int k = n - 2; k >= 0; --k) y2[k] = y2[k] * y2[k + 1] + u[k];
  return y2;
}

// Checks a caller's description; returns nullptr or a message.
inline const char *stf_check(const sem2d_stf &s) {
  switch (s.kind) {
    case SEM2D_STF_RICKER:
    case SEM2D_STF_GAUSSIAN:
    case SEM2D_STF_BRUNE:
    case SEM2D_STF_HARMONIC:
    case SEM2D_STF_USER:
      return nullptr;
    case SEM2D_STF_TAB:
      if (s.ntab < 2 || !s.tab_t || !s.tab_v) return "tabulated time function needs two rows or more";
      for (int k = 1; k < s.ntab; ++k)
        if (!(s.tab_t[k] > s.tab_t[k - 1])) return "tabulated time function: times must increase";
      return nullptr;
    default:
      return "unknown source time function";
  }
}

// Boundary forces with a time function of their own, evaluated every step
// on the perimeter nodes: the incident plane wave across the absorbing
// sides (BC_ABSO_apply, bc_abso.f90:299-306) and the time-dependent
// tractions of &BC_DIRNEU (bc_DIRNEU_apply, bc_dirneu.f90:157-167).
// Entry k (0, 1) of perimeter slot s adds to force component c
//     W[(k*ndof + c)*nslot + s] * stf[q](t - phi[k*nslot + s]),
// q = fn[(k*ndof + c)*nslot + s] (-1: nothing), t = it dt + tshift.
struct BoundaryForces {
  const double *W = nullptr;  // null: no boundary forces
  const signed char *fn = nullptr;
  const double *phi = nullptr;
  const StfDev *stf = nullptr;
  double dt = 0, tshift = 0;
};

__device__ __forceinline__ double boundary_force(const BoundaryForces &b, int ndof, int nslot, int s, int c,
                                                 int it) {
  const double t = it * b.dt + b.tshift;
  double f = 0.0;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int e = (k * ndof + c) * nslot + s;
    const int q = b.fn[e];
    if (q >= 0) f = f + b.W[e] * stf_value(b.stf[q], t - b.phi[k * nslot + s]);
  }
  return f;
}

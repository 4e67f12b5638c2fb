// fault_kernel.cuh -- split-node dynamic fault, one thread per fault node
// pair, entirely in FP64 (called from the bulk kernel by the CTA that owns
// the fault rows).
//
// Restates BC_DYNFLT_apply (bc_dynflt.f90:569-739): traction that keeps
// the fault stuck (T = Z (dV + coefA2V dA)), rotation to the fault frame,
// opening, normal-stress law (bc_dynflt_normal.f90:118-133), friction
// (slip weakening bc_dynflt_swf.f90:142-183; rate and state
// bc_dynflt_rsf.f90:165-568 with the bracketed Newton solver), boundary
// term B T added to both sides, slip and slip-rate update; then finishes
// the time update of the two split nodes (which the bulk kernel skipped)
// and records the fault time series (bc_dynflt.f90:751-778).
//
// Each thread keeps FP64 copies of displacement, velocity and
// acceleration of its two nodes, so slip, slip rate and the state
// variable are accumulated in FP64 whatever the precision of the bulk.
#pragma once

#include "sem2d_common.cuh"

namespace sem2d {

constexpr int kNrMaxIt = 200;       // bc_dynflt_rsf.f90:372 (default of FaultParams::nr_maxit)
constexpr int kNrMaxBracket = 200;  // bound for the loop at bc_dynflt_rsf.f90:393-398
constexpr int kErrNR = -4;          // SEM2D_E_NR

// slip-weakening parameters of one node (read together, before any store)
struct SwfNode {
  double dc, mus, mud, p, alpha;
};

template <typename real>
__device__ __forceinline__ SwfNode swf_node(const FaultParams<real> &p, int k) {
  return SwfNode{p.swf_dc[k], p.swf_mus[k], p.swf_mud[k], p.swf_kind == 3 ? p.swf_p[k] : 0.0, p.swf_alpha[k]};
}

__device__ __forceinline__ double swf_mu_of(int kind, const SwfNode &w, double th) {
  double mu;
  if (kind == 1) {
    const double r = th / w.dc;
    mu = w.mus - (w.mus - w.mud) * (r < 1.0 ? r : 1.0);
  } else if (kind == 2) {
    mu = w.mud - (w.mud - w.mus) * exp(-th / w.dc);
  } else {
    mu = w.mud + (w.mus - w.mud) / pow(1.0 + th / w.dc, w.p);
  }
  return mu + w.alpha * th;
}

template <typename real>
__device__ double swf_mu(const FaultParams<real> &p, int k, double th) {
  return swf_mu_of(p.swf_kind, swf_node(p, k), th);
}

template <typename real>
__device__ double rsf_mu(const FaultParams<real> &p, int k, double v, double th) {
  const double av = fabs(v), a = p.rsf_a[k], b = p.rsf_b[k];
  if (p.rsf_kind == 1)
    return p.rsf_mus[k] + a * av / (av + p.rsf_vstar[k]) - b * th / (th + p.rsf_dc[k]);
  const double lg = p.rsf_kind == 4 ? log(p.rsf_vc[k] * th / p.rsf_dc[k] + 1.0)
                                    : log(p.rsf_vstar[k] * th / p.rsf_dc[k]);
  return a * asinh(av / (2.0 * p.rsf_vstar[k]) * exp((p.rsf_mus[k] + b * lg) / a));
}

template <typename real>
__device__ double rsf_theta(const FaultParams<real> &p, int k, double th, double v) {
  if (p.rsf_kind == 1) {
    double r = th * p.rsf_coeft[k] + p.rsf_Tc[k] * fabs(v) * (1.0 - p.rsf_coeft[k]);
    return r < 1.0e-12 ? 0.0 : r;
  }
  if (p.rsf_kind == 3) {
    const double r = p.rsf_dc[k] / fabs(v);
    return r * pow(th / r, exp(-p.dt / r));
  }
  const double x = fabs(v) / p.rsf_dc[k];
  const double ex = exp(-(p.dt * x));
  if (p.dt * x > 1.0e-8) return th * ex + (1.0 - ex) / x;
  return th * ex + p.dt * (1.0 - 0.5 * p.dt * x);
}

// the factor 2 V* exp(-(f0 + b ln(V* theta/Dc))/a) of the slip-rate law,
// fixed during one solve (theta does not change)
template <typename real>
__device__ double nr_rate_factor(const FaultParams<real> &p, int k, double th) {
  double tmp = p.rsf_kind == 4
                   ? p.rsf_mus[k] + p.rsf_b[k] * log(p.rsf_vc[k] * th / p.rsf_dc[k] + 1.0)
                   : p.rsf_mus[k] + p.rsf_b[k] * log(p.rsf_vstar[k] * th / p.rsf_dc[k]);
  return 2.0 * p.rsf_vstar[k] * exp(-tmp / p.rsf_a[k]);
}

// tau_stick - Z v(tau) - tau and its derivative (nr_fric_func_tau,
// bc_dynflt_rsf.f90:533-568); rf = nr_rate_factor, sa = -sigma a
__device__ __forceinline__ void nr_func(double rf, double sa, double tau, double ts, double Z, double &fn,
                                        double &dfn, double &v) {
  v = sinh(tau / sa) * rf;
  fn = ts - Z * v - tau;
  dfn = -Z * (cosh(tau / sa) * rf / sa) - 1.0;
}

// bracketed Newton-Raphson with bisection (bc_dynflt_rsf.f90:369-468);
// returns the slip rate of its last function evaluation, as the reference
template <typename real>
__device__ double nr_solve(const FaultParams<real> &p, int k, double xL, double xR, double xacc,
                           double th, double ts, double sig, double Z, bool &fail) {
  const double rf = nr_rate_factor(p, k, th), sa = -sig * p.rsf_a[k];
  double flo, fhi, dfn, v, xl = xL, xr = xR;
  nr_func(rf, sa, xL, ts, Z, flo, dfn, v);
  nr_func(rf, sa, xR, ts, Z, fhi, dfn, v);
  int guard = 0;
  while (flo * fhi > 0) {
    if (++guard > kNrMaxBracket) {
      fail = true;
      return v;
    }
    xl = xl / 2.0;
    xr = xr * 2.0;
    nr_func(rf, sa, xl, ts, Z, flo, dfn, v);
    nr_func(rf, sa, xr, ts, Z, fhi, dfn, v);
  }
  if (flo == 0 || fhi == 0) return v;
  double xlow = flo < 0 ? xl : xr, xhigh = flo < 0 ? xr : xl;
  double xest = 0.5 * (xl + xr), dxold = fabs(xr - xl), dx = dxold, fx;
  nr_func(rf, sa, xest, ts, Z, fx, dfn, v);
  for (int is = 0; is < p.nr_maxit; ++is) {
    if (((xest - xhigh) * dfn - fx) * ((xest - xlow) * dfn - fx) > 0 ||
        fabs(2 * fx) > fabs(dxold * dfn)) {
      dxold = dx;
      dx = 0.5 * (xhigh - xlow);
      xest = xlow + dx;
      if (xlow == xest) return v;
    } else {
      dxold = dx;
      dx = fx / dfn;
      const double tmp = xest;
      xest = xest - dx;
      if (tmp == xest) return v;
    }
    if (fabs(dx) < fabs(xacc)) {
      nr_func(rf, sa, xest, ts, Z, fx, dfn, v);
      return v;
    }
    nr_func(rf, sa, xest, ts, Z, fx, dfn, v);
    if (fx < 0) xlow = xest;
    else xhigh = xest;
  }
  fail = true;
  return v;
}

template <typename real>
__device__ double rsf_V(const FaultParams<real> &p, int k, double ts, double sig, double th,
                        double th_old, double Z, bool &fail) {
  if (p.rsf_kind == 1) {
    // rsf_mu_no_direct uses the state stored before this step
    const double mnd = p.rsf_mus[k] - p.rsf_b[k] * th_old / (th_old + p.rsf_dc[k]);
    double v = (ts + sig * mnd) / Z;
    const double tmp = v - p.rsf_vstar[k] + sig * p.rsf_a[k] / Z;
    v = 0.5 * (tmp + sqrt(tmp * tmp + 4.0 * v * p.rsf_vstar[k]));
    v = v > 0.0 ? v : 0.0;
    return v < 1.0e-12 ? 0.0 : v;
  }
  const double tol = -0.001 * p.rsf_a[k] * sig;
  const double lo = ts < 0.0 ? ts : 0.0, hi = ts > 0.0 ? ts : 0.0;
  return nr_solve(p, k, lo, hi, tol, th, ts, sig, Z, fail);
}

template <typename real>
__device__ void fault_record(const FaultParams<real> &p, int k, int it) {
  if (it < p.oit || (it - p.oit) % p.oitd != 0) return;
  const int s = (it - p.oit) / p.oitd;
  const int k1 = k + 1;
  if (s >= p.nsamp || k1 < p.oix1 || (k1 - p.oix1) % p.oixd != 0) return;
  const int q = (k1 - p.oix1) / p.oixd;
  if (q >= p.onx) return;
  const int nf = p.nflt;
  double *o = p.series + (size_t)p.onx * 6 * s;
  o[q] = p.D[k];
  o[q + p.onx] = p.V[k];
  o[q + 2 * p.onx] = p.T[k];
  o[q + 3 * p.onx] = p.T[k + nf];
  o[q + 4 * p.onx] = p.MU[k];
  o[q + 5 * p.onx] = p.Tstick[k];
}

// time-weakening friction coefficient (twf_mu, bc_dynflt_twf.f90:117-184)
// of node k at time `time` with slip d.  Kind 3 leaves mu undefined for
// r > V T in the reference; the large value is returned there, so the
// other law (or sticking) decides.
template <typename real>
__device__ double twf_mu(const FaultParams<real> &p, int k, double time, double d) {
  const double big = 1.7976931348623157e308;  // huge(1d0)
  const double x = p.fxz[2 * k] - p.twf_X, z = p.fxz[2 * k + 1] - p.twf_Z;
  const double dist = sqrt(x * x + z * z);
  if (p.twf_kind == 1 || p.twf_kind == 2) {
    double t, r;
    if (p.twf_kind == 1) {
      t = time + ((p.twf_mus - p.twf_mu0) * p.twf_L) / ((p.twf_mus - p.twf_mud) * p.twf_V);
      if (t > p.twf_T) t = 0.0;
      r = p.twf_V * t;
    } else {
      t = time + (0.5 * p.twf_T) *
                     (1.0 - sqrt(1.0 - ((4.0 * (p.twf_mus - p.twf_mu0)) * p.twf_L) /
                                           (((p.twf_mus - p.twf_mud) * p.twf_T) * p.twf_V)));
      if (t > p.twf_T) t = p.twf_T;
      r = (p.twf_V * t) * (1.0 - t / p.twf_T);
    }
    r = dist - r;
    if (r < -p.twf_L) return p.twf_mud;
    if (r <= p.twf_L) return p.twf_mus + ((p.twf_mus - p.twf_mud) / p.twf_L) * r;
    return big;
  }
  const double vt = p.twf_V * time;
  if (dist <= p.twf_V * p.twf_T && d <= p.twf_Dc) {
    if (dist < vt - p.twf_L) return p.twf_mud;
    if (dist <= vt) return p.twf_mus + ((p.twf_mus - p.twf_mud) / p.twf_L) * (dist - vt);
  }
  return big;
}

// initial friction and the step-0 record (bc_dynflt.f90:401-415, 247)
template <typename real>
__global__ void fault_init_kernel(FaultParams<real> p) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= p.nflt) return;
  p.sigma[k] = p.T0[k + p.nflt];
  if (p.friction == 2) p.MU[k] = rsf_mu(p, k, p.V[k], p.theta[k]);
  else if (p.friction == 1) p.MU[k] = swf_mu(p, k, p.theta[k]);
  if (p.twf_kind) {
    const double mt = twf_mu(p, k, 0.0, 0.0);
    if (p.friction == 3 || mt < p.MU[k]) p.MU[k] = mt;
  }
  fault_record(p, k, 0);
}

// One fault node pair k at step it, given the raw nodal forces f1, f2 of
// both sides (internal + sources + absorbing terms).  Finishes the time
// update of the two split nodes, which the bulk update skips.
template <typename real>
__device__ void fault_node_update(const FaultParams<real> &p, int k, int it, const double *f1in,
                                  const double *f2in) {
  const int nd = p.ndof, nf = p.nflt;
  double f1[2] = {0, 0}, f2[2] = {0, 0}, d1[2] = {0, 0}, d2[2] = {0, 0};
  double v1[2] = {0, 0}, v2[2] = {0, 0}, dD[2] = {0, 0}, dV[2] = {0, 0}, dA[2] = {0, 0};
  double T[2] = {0, 0}, Ts[2] = {0, 0};
  for (int c = 0; c < nd; ++c) {
    const int o1 = (0 * nd + c) * nf + k, o2 = (1 * nd + c) * nf + k;
    f1[c] = f1in[c];
    d1[c] = p.d64[o1];
    v1[c] = p.v64[o1];
    if (p.scheme == 1) v1[c] = v1[c] + p.cpred * p.a64[o1];
    if (p.two) {
      f2[c] = f2in[c];
      d2[c] = p.d64[o2];
      v2[c] = p.v64[o2];
      if (p.scheme == 1) v2[c] = v2[c] + p.cpred * p.a64[o2];
      dD[c] = d2[c] - d1[c];
      dV[c] = v2[c] - v1[c];
      dA[c] = p.invM2[k + nf * c] * f2[c] - p.invM1[k + nf * c] * f1[c];
    } else {
      dD[c] = -2.0 * d1[c];
      dV[c] = -2.0 * v1[c];
      dA[c] = -2.0 * p.invM1[k + nf * c] * f1[c];
    }
    T[c] = p.Z[k + nf * c] * (dV[c] + p.coefA2V * dA[c]);
  }
  const double nx = p.n1[k], nz = p.n1[k + nf];
  // the node's other inputs, read before any of its stores so that their
  // latencies overlap
  const double T00 = p.T0[k], T01 = p.T0[k + nf], sig_old = p.sigma[k], th_old = p.theta[k];
  const double Dk = p.D[k], Vk = p.V[k], cohk = p.coh[k], Zk = p.Z[k];
  SwfNode swn{0, 0, 0, 0, 0};
  if (p.friction == 1) swn = swf_node(p, k);
  if (nd == 2) {
    double r0, r1;
    r0 = nz * dD[0] - nx * dD[1]; r1 = nx * dD[0] + nz * dD[1]; dD[0] = r0; dD[1] = r1;
    r0 = nz * dV[0] - nx * dV[1]; r1 = nx * dV[0] + nz * dV[1]; dV[0] = r0; dV[1] = r1;
    r0 = nz * dA[0] - nx * dA[1]; r1 = nx * dA[0] + nz * dA[1]; dA[0] = r0; dA[1] = r1;
    r0 = nz * T[0] - nx * T[1];   r1 = nx * T[0] + nz * T[1];   T[0] = r0;  T[1] = r1;
  }
  if (!p.two || nd == 1) T[1] = 0.0;
  T[0] = T[0] + T00;
  T[1] = T[1] + T01;
  if (p.opening) T[1] = T[1] < 0.0 ? T[1] : 0.0;
  double sig = sig_old;
  if (p.normal_kind == 1) sig = T[1];
  else if (p.normal_kind == 2) sig = T[1] + p.normal_coef * (sig - T[1]);
  else if (p.normal_kind == 3)
    sig = T[1] + exp(-(fabs(dV[0]) + p.normal_V) * p.normal_coef) * (sig - T[1]);
  double mu, th_new = th_old;
  if (p.friction == 2) {
    bool fail = false;
    const double vold = Vk, th0 = th_old;
    const double th1 = rsf_theta(p, k, th0, vold);
    double vnew = rsf_V(p, k, T[0], sig, th1, th0, Zk, fail);
    const double th2 = rsf_theta(p, k, th0, 0.5 * (vold + vnew));
    vnew = rsf_V(p, k, T[0], sig, th2, th0, Zk, fail);
    if (fail) atomicExch(p.error, kErrNR);
    th_new = th2;
    mu = rsf_mu(p, k, vnew, th2);
    if (p.twf_kind) {
      const double mt = twf_mu(p, k, it * p.dt + p.tshift, Dk);
      if (mt < mu) mu = mt;
    }
    T[0] = copysign(fabs(-mu * sig), T[0]);
    // T_stick is undefined on this branch of the reference (bc_dynflt.f90:581)
    Ts[0] = 0.0;
    Ts[1] = 0.0;
  } else {
    if (p.friction == 1) {
      double th = th_old;
      if (p.coefA2D == 0.0) {
        if (p.swf_healing) {
          th = th + fabs(dV[0]) * p.dt;
          if (fabs(dV[0]) < 1.0e-14) th = 0.0;
        } else {
          th = fabs(dD[0]);
        }
      } else {
        th = fabs(Dk);
      }
      th_new = th;
      mu = swf_mu_of(p.swf_kind, swn, th);
      if (p.twf_kind) {
        const double mt = twf_mu(p, k, it * p.dt + p.tshift, Dk);
        if (mt < mu) mu = mt;
      }
    } else {  // time weakening alone
      mu = twf_mu(p, k, it * p.dt + p.tshift, Dk);
    }
    const double strength = cohk - mu * sig;
    Ts[0] = T[0];
    Ts[1] = T[1];
    const double at = fabs(T[0]);
    T[0] = copysign(fabs(at < strength ? at : strength), T[0]);
  }
  p.sigma[k] = sig;
  if (p.friction == 1 || p.friction == 2) p.theta[k] = th_new;
  p.MU[k] = mu;
  T[0] = T[0] - T00;
  T[1] = T[1] - T01;
  p.T[k] = T[0];
  p.T[k + nf] = T[1];
  p.Tstick[k] = Ts[0] - T00;
  p.Tstick[k + nf] = Ts[1] - T01;
  double Tx[2] = {T[0], T[1]};
  if (nd == 2) {
    Tx[0] = nz * T[0] + nx * T[1];
    Tx[1] = -nx * T[0] + nz * T[1];
  }
  for (int c = 0; c < nd; ++c) {
    const double dAc = dA[c] - T[c] / (p.Z[k + nf * c] * p.coefA2V);
    p.D[k + nf * c] = dD[c] + p.coefA2D * dAc;
    p.V[k + nf * c] = dV[c] + p.coefA2V * dAc;
  }
  double vnew[2][2] = {{0, 0}, {0, 0}}, dcor[2][2] = {{0, 0}, {0, 0}};
  for (int side = 0; side < 1 + p.two; ++side) {
    const int J = side == 0 ? p.jf1 : p.jf2;
    for (int c = 0; c < nd; ++c) {
      const int o = (side * nd + c) * nf + k;
      double f = side == 0 ? f1[c] + p.B[k] * Tx[c] : f2[c] - p.B[k] * Tx[c];
      // a zero-Dirichlet side after the fault in &BC_DEF order (bc_gen.f90:279-281)
      if (p.dir_zero && ((p.dir_zero[k] >> (side * 2 + c)) & 1)) f = 0.0;
      const double vp = side == 0 ? v1[c] : v2[c];
      double dc = side == 0 ? d1[c] : d2[c];
      const double a = p.rm[o] * f;
      const double vn = vp + p.cv * a;
      // Newmark corrector d += beta dt^2 a (solver.f90:82) before the next
      // step's predictor
      if (p.scheme == 1 && p.cb != 0.0) dc = dc + p.cb * a;
      const double dn = p.scheme == 1 ? (dc + p.dt * vn) + p.cd2 * a : dc + p.dt * vn;
      p.d64[o] = dn;
      p.v64[o] = vn;
      p.a64[o] = a;
      vnew[side][c] = vn;
      dcor[side][c] = dc;
      const long long g = c * p.plane + (long long)J * p.pitch + k;
      p.Dnext[g] = real(dn);
      p.Vnext[g] = real(vn);
      if (p.Anext) p.Anext[g] = real(a);
    }
  }
  if (p.pot) {
    // this pair's terms of BC_DYNFLT_potency (bc_dynflt.f90:832-855) for
    // the displacement d^n and the velocity v^n of the step (get_jump,
    // bc_dynflt.f90:692-704): P-SV p11, p22, p12; SH p13, p23
    const double b = p.B[k];
    for (int f = 0; f < 2; ++f) {
      double dl[2] = {0, 0};
      for (int c = 0; c < nd; ++c) {
        const double x1 = f == 0 ? dcor[0][c] : vnew[0][c];
        dl[c] = p.two ? (f == 0 ? dcor[1][c] : vnew[1][c]) - x1 : -2.0 * x1;
      }
      double t0, t1, t2;
      if (nd == 2) {
        t0 = nx * dl[0] * b;
        t1 = nz * dl[1] * b;
        t2 = 0.5 * ((nx * dl[1] + nz * dl[0]) * b);
      } else {
        t0 = 0.5 * (nx * dl[0] * b);
        t1 = 0.5 * (nz * dl[0] * b);
        t2 = 0.0;
      }
      p.pot[(3 * f) * nf + k] = t0;
      p.pot[(3 * f + 1) * nf + k] = t1;
      p.pot[(3 * f + 2) * nf + k] = t2;
    }
  }
  fault_record(p, k, it);
}

// interpolated seismograms of velocity or acceleration, and of displacement
// under the Newmark corrector (REC_store,
// receivers.f90:309-344), after the bulk kernel moved the step counter
template <typename real>
__global__ void receiver_kernel(RecParams<real> p) {
  const int it = *p.step;
  if (it % p.isamp != 0) return;
  const int s = it / p.isamp;
  if (s >= p.nsamp) return;
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= p.nrec * p.ndof) return;
  const int r = q % p.nrec, c = q / p.nrec;
  const real *f = p.field + c * p.plane;
  const real *ac = p.acc ? p.acc + c * p.plane : nullptr;
  auto at = [&](int l) { return ac ? double(f[l] + p.cb * ac[l]) : double(f[l]); };
  double val;
  if (p.npts == 1) {
    val = at(p.lat[r]);
  } else {
    const int *L = p.lat + (size_t)r * p.npts;
    const double *W = p.w + (size_t)r * p.npts;
    val = W[0] * at(L[0]);
    for (int k = 1; k < p.npts; ++k) val = val + W[k] * at(L[k]);
  }
  p.sis[s + (size_t)p.nsamp * (r + (size_t)p.nrec * c)] = val;
}

}  // namespace sem2d

namespace sem2d {

// Periodic columns (bc_perio_apply = BC_PERIO_set_field, bc_periodic.f90:
// 77-88, applied first of the boundary terms, bc_gen.f90:271-275): the
// raw forces the step kernel left for the nodes (0, J) and (LX-1, J) are
// summed, each copy takes its dashpot, boundary-force, Stacey and Dirichlet
// terms and is updated as the step kernel updates a node; on the fault rows
// the sums go to the fault node update of k = 0 and k = LX-1.  One thread
// per lattice row; with tb the rows J = 0 and LZ-1 instead, one thread per
// lattice column (no fault).
template <typename real>
struct PerioParams {
  int LX, LZ, ndof, nslot, scheme;
  long long plane, pitch;
  const real *pf;
  const real *Dcur, *Vcur, *Acur;
  real *Dnext, *Vnext, *Anext;
  const real *per_rm, *per_Ca, *per_Cb;
  const int *per_dir;
  const real *per_bf;  // incident wave and Neumann tractions of this step, or null
  const real *per_kd;  // Stacey forces of this step, or null
  int tb;              // bottom/top rows instead of left/right columns
  real dt, cv, cpred, cpa, cd2, cb;
  int jf1, jf2, has_fault, two;
  const int *step;
};

template <typename real>
__device__ __forceinline__ real perio_boundary(const PerioParams<real> &p, int I, int J, int c, real fc, real *vpred,
                                               real *rm) {
  const long long g = c * p.plane + (long long)J * p.pitch + I;
  real vp = p.Vcur[g], vd = vp;
  if (p.scheme != 0) {
    const real an = p.Acur[g];
    vd = vp + (p.scheme == 2 ? p.cpa : p.cpred) * an;
    vp = vp + p.cpred * an;
  }
  const int sp = perimeter_slot(I, J, p.LX, p.LZ), so = c * p.nslot + sp;
  fc = fc - p.per_Ca[so] * vd;
  fc = fc - p.per_Cb[so] * vd;
  if (p.per_bf) fc = fc + p.per_bf[so];
  if (p.per_kd) fc = fc - p.per_kd[so];
  if (p.per_dir && ((p.per_dir[sp] >> c) & 1)) fc = real(0);
  *vpred = vp;
  *rm = p.per_rm[so];
  return fc;
}

template <typename real>
__global__ void perio_kernel(const PerioParams<real> p, FaultParams<real> flt) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (p.tb) {  // the pair (I, 0), (I, LZ-1)
    if (q >= p.LX) return;
    for (int e = 0; e < 2; ++e) {
      const int J = e ? p.LZ - 1 : 0;
      for (int c = 0; c < p.ndof; ++c) {
        const long long g = c * p.plane + (long long)J * p.pitch + q;
        real vp, rm;
        const real s = p.pf[(size_t(c) * p.LX + q) * 2] + p.pf[(size_t(c) * p.LX + q) * 2 + 1];
        const real fc = perio_boundary(p, q, J, c, s, &vp, &rm);
        const real a = rm * fc;
        const real vnew = vp + p.cv * a;
        real dcur = p.Dcur[g];
        if (p.scheme != 0 && p.cb != real(0)) dcur = dcur + p.cb * a;
        const real dnext = p.scheme != 0 ? (dcur + p.dt * vnew) + p.cd2 * a : dcur + p.dt * vnew;
        p.Vnext[g] = vnew;
        p.Dnext[g] = dnext;
        if (p.Anext) p.Anext[g] = a;
      }
    }
    return;
  }
  const int J = q;
  if (J >= p.LZ) return;
  const int it = *p.step;
  if (p.has_fault && p.two && J == p.jf2) return;  // with the row jf1
  if (p.has_fault && J == p.jf1) {
    for (int e = 0; e < 2; ++e) {
      const int I = e ? p.LX - 1 : 0;
      double f1[2] = {0, 0}, f2[2] = {0, 0};
      for (int c = 0; c < p.ndof; ++c) {
        real vp, rm;
        const real s1 = p.pf[(size_t(c) * p.LZ + p.jf1) * 2] + p.pf[(size_t(c) * p.LZ + p.jf1) * 2 + 1];
        f1[c] = double(perio_boundary(p, I, p.jf1, c, s1, &vp, &rm));
        if (p.two) {
          const real s2 = p.pf[(size_t(c) * p.LZ + p.jf2) * 2] + p.pf[(size_t(c) * p.LZ + p.jf2) * 2 + 1];
          f2[c] = double(perio_boundary(p, I, p.jf2, c, s2, &vp, &rm));
        }
      }
      fault_node_update(flt, I, it, f1, f2);
    }
    return;
  }
  for (int e = 0; e < 2; ++e) {
    const int I = e ? p.LX - 1 : 0;
    for (int c = 0; c < p.ndof; ++c) {
      const long long g = c * p.plane + (long long)J * p.pitch + I;
      real vp, rm;
      const real s = p.pf[(size_t(c) * p.LZ + J) * 2] + p.pf[(size_t(c) * p.LZ + J) * 2 + 1];
      const real fc = perio_boundary(p, I, J, c, s, &vp, &rm);
      const real a = rm * fc;
      const real vnew = vp + p.cv * a;
      real dcur = p.Dcur[g];
      if (p.scheme != 0 && p.cb != real(0)) dcur = dcur + p.cb * a;
      const real dnext = p.scheme != 0 ? (dcur + p.dt * vnew) + p.cd2 * a : dcur + p.dt * vnew;
      p.Vnext[g] = vnew;
      p.Dnext[g] = dnext;
      if (p.Anext) p.Anext[g] = a;
    }
  }
}

}  // namespace sem2d

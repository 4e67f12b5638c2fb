// host_builder.cpp -- Par.inp-level problem builder for the Cartesian path.
//
// Implements include/sem2d_host.h.  The reference builds a generic FEM
// database (vertex/edge connectivity lists, fem_grid.f90:103-205) and then
// numbers GLL nodes element by element (spec_grid.f90:198-314).  Here the
// mesh is known to be a structured lattice of GLL nodes, possibly with one
// duplicated row at a fault (mesh_structured.f90:78-80), so numbering,
// coordinates and boundary tables are produced directly on that lattice.
// The results are bit-identical to the reference's:
//   * elements are visited in reverse Cuthill-McKee order (rcm.f90), and a
//     node gets its number the first time an element in that order reaches
//     it: interior nodes, then the unnumbered edges D,R,U,L in
//     counterclockwise order, then the unnumbered vertices;
//   * a node shared by several elements takes the coordinate computed by
//     the last of them (spec_grid.f90:321-374);
//   * boundary node tables are the lattice lines, i.e. the order of the
//     stable coordinate sort of BC_set_bulk_node (spec_grid.f90:780-800).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/sem2d_host.h"

namespace {

thread_local std::string g_err;

struct BuildError : std::runtime_error {
  explicit BuildError(const std::string &m) : std::runtime_error(m) {}
};

constexpr double kPi = 3.141592653589793;  // constants.f90:34
constexpr double kTinyXabs = 1.0e-3;       // constants.f90:30

// --------------------------------------------------------------------
// Gauss-Lobatto-Legendre quadrature: Gauss-Jacobi interior points by
// Newton iteration with deflation, weights from the Jacobi recurrences
// (the algorithm of gll.f90:300-684), derivative matrix from the Legendre
// recurrence (gll.f90:230-265).  Same recurrences and operation order.
struct Jacobi {
  double p, pd, pm1, pdm1, pm2, pdm2;
};

Jacobi jacobi_eval(int n, double a, double b, double x) {
  Jacobi r{1.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  if (n == 0) return r;
  const double apb = a + b;
  double pl = r.p, pdl = r.pd, ps = 0.0, pds = 0.0;
  r.p = (a - b + (apb + 2.0) * x) / 2.0;
  r.pd = (apb + 2.0) / 2.0;
  if (n == 1) return r;
  for (int k = 2; k <= n; ++k) {
    const double dk = k;
    const double a1 = 2.0 * dk * (dk + apb) * (2.0 * dk + apb - 2.0);
    const double a2 = (2.0 * dk + apb - 1.0) * (a * a - b * b);
    const double b3 = (2.0 * dk + apb - 2.0);
    const double a3 = b3 * (b3 + 1.0) * (b3 + 2.0);
    const double a4 = 2.0 * (dk + a - 1.0) * (dk + b - 1.0) * (2.0 * dk + apb);
    const double pn = ((a2 + a3 * x) * r.p - a4 * pl) / a1;
    const double pdn = ((a2 + a3 * x) * r.pd - a4 * pdl + a3 * r.p) / a1;
    ps = pl;
    pds = pdl;
    pl = r.p;
    r.p = pn;
    pdl = r.pd;
    r.pd = pdn;
  }
  r.pm1 = pl;
  r.pdm1 = pdl;
  r.pm2 = ps;
  r.pdm2 = pds;
  return r;
}

double gamma_small(double x) {  // exact values used by the GLL weights
  const double sp = std::sqrt(kPi);
  if (x == -0.5) return -2.0 * sp;
  if (x == 0.5) return sp;
  if (x == 1.5) return sp / 2.0;
  if (x == 2.5) return 1.5 * sp / 2.0;
  if (x == 3.5) return 2.5 * 1.5 * sp / 2.0;
  if (x == 3.0) return 2.0;
  if (x == 4.0) return 6.0;
  if (x == 5.0) return 24.0;
  if (x == 6.0) return 120.0;
  return 1.0;
}

double end_weight(int n, double a, double b, bool right) {
  const double apb = a + b;
  if (n == 0) return 0.0;
  double f1 = right ? gamma_small(a + 1.0) * gamma_small(b + 2.0) / gamma_small(apb + 3.0)
                    : gamma_small(a + 2.0) * gamma_small(b + 1.0) / gamma_small(apb + 3.0);
  f1 = f1 * (apb + 2.0) * std::pow(2.0, apb + 2.0) / 2.0;
  if (n == 1) return f1;
  double fint1 = right ? gamma_small(a + 1.0) * gamma_small(b + 2.0) / gamma_small(apb + 3.0)
                       : gamma_small(a + 2.0) * gamma_small(b + 1.0) / gamma_small(apb + 3.0);
  fint1 = fint1 * std::pow(2.0, apb + 2.0);
  double fint2 = gamma_small(a + 2.0) * gamma_small(b + 2.0) / gamma_small(apb + 4.0);
  fint2 = fint2 * std::pow(2.0, apb + 3.0);
  double f2 = right ? (2.0 * (a + 2.0) * fint1 - (apb + 4.0) * fint2) * (apb + 3.0) / 4.0
                    : (-2.0 * (b + 2.0) * fint1 + (apb + 4.0) * fint2) * (apb + 3.0) / 4.0;
  if (n == 2) return f2;
  double f3 = 0.0;
  for (int i = 3; i <= n; ++i) {
    const double di = i - 1, abn = a + b + di, abnn = abn + di;
    const double a1 = -(2.0 * (di + a) * (di + b)) / (abn * abnn * (abnn + 1.0));
    const double a2 = (2.0 * (a - b)) / (abnn * (abnn + 2.0));
    const double a3 = (2.0 * (abn + 1.0)) / ((abnn + 2.0) * (abnn + 1.0));
    f3 = -(a2 * f2 + a1 * f1) / a3;
    f1 = f2;
    f2 = f3;
  }
  return f3;
}

double jacobi_norm(int n, double a, double b) {
  const double dn = n, c = a + b + 1.0;
  double prod;
  if (n <= 1) {
    prod = gamma_small(dn + a) * gamma_small(dn + b);
    prod = prod / (gamma_small(dn) * gamma_small(dn + a + b));
    return prod * std::pow(2.0, c) / (2.0 * dn + c);
  }
  prod = gamma_small(a + 1.0) * gamma_small(b + 1.0);
  prod = prod / (2.0 * (1.0 + c) * gamma_small(c + 1.0));
  prod = prod * (1.0 + a) * (2.0 + a);
  prod = prod * (1.0 + b) * (2.0 + b);
  for (int i = 3; i <= n; ++i) {
    const double di = i;
    prod = prod * ((di + a) * (di + b) / (di * (di + a + b)));
  }
  return prod * std::pow(2.0, c) / (2.0 * dn + c);
}

void gauss_jacobi(double *z, double *w, int np, double a, double b) {
  const double apb = a + b;
  if (np == 1) {
    z[0] = (b - a) / (apb + 2.0);
    w[0] = gamma_small(a + 1.0) * gamma_small(b + 1.0) / gamma_small(apb + 2.0) *
           std::pow(2.0, apb + 1.0);
    return;
  }
  // roots, largest first, Newton with deflation of the roots already found
  const int n = np - 1;
  const double dth = 4.0 * std::atan(1.0) / (2.0 * n + 2.0);
  double xlast = 0.0;
  for (int j = 1; j <= np; ++j) {
    double x = std::cos((2.0 * (j - 1.0) + 1.0) * dth);
    if (j > 1) x = (x + xlast) / 2.0;
    for (int k = 0; k < 10; ++k) {
      const Jacobi J = jacobi_eval(np, a, b, x);
      double rs = 0.0;
      for (int i = 1; i <= j - 1; ++i) rs = rs + 1.0 / (x - z[np - i]);
      const double dx = -J.p / (J.pd - rs * J.p);
      x = x + dx;
      if (std::fabs(dx) < 1.0e-12) break;
    }
    z[np - j] = x;
    xlast = x;
  }
  // selection sort to ascending order (as gll.f90:370-381)
  int jmin = 0;
  for (int i = 0; i < np; ++i) {
    double xm = 2.0;
    for (int j = i; j < np; ++j)
      if (z[j] < xm) {
        xm = z[j];
        jmin = j;
      }
    if (jmin != i) std::swap(z[i], z[jmin]);
  }
  const int np1 = n + 1, np2 = n + 2;
  const double fac1 = np1 + a + b + 1.0, fac2 = fac1 + np1, fac3 = fac2 + 1.0;
  const double rcoef = (jacobi_norm(np1, a, b) * fac2 * fac3) / (2.0 * fac1 * double(np2));
  for (int i = 0; i < np; ++i) {
    const Jacobi J = jacobi_eval(np2, a, b, z[i]);
    w[i] = -rcoef / (J.p * J.pdm1);
  }
}

double legendre(double z, int n) {
  double p1 = 1.0, p2 = z, p3 = p2;
  for (int k = 1; k <= n - 1; ++k) {
    const double fk = k;
    p3 = ((2.0 * fk + 1.0) * z * p2 - fk * p1) / (fk + 1.0);
    p1 = p2;
    p2 = p3;
  }
  return p3;
}

double legendre_deriv(double z, int n) {
  double p1 = 1.0, p2 = z, p1d = 0.0, p2d = 1.0, p3d = 1.0;
  for (int k = 1; k <= n - 1; ++k) {
    const double fk = k;
    const double p3 = ((2.0 * fk + 1.0) * z * p2 - fk * p1) / (fk + 1.0);
    p3d = ((2.0 * fk + 1.0) * p2 + (2.0 * fk + 1.0) * z * p2d - fk * p1d) / (fk + 1.0);
    p1 = p2;
    p2 = p3;
    p1d = p2d;
    p2d = p3d;
  }
  return p3d;
}

struct Gll {
  int n;
  std::vector<double> x, w, H;  // H(i,j) = h'_i(x_j), column-major
};

Gll make_gll(int n) {
  Gll g{n, std::vector<double>(n), std::vector<double>(n), std::vector<double>(n * n)};
  if (n > 2) gauss_jacobi(&g.x[1], &g.w[1], n - 2, 1.0, 1.0);
  g.x[0] = -1.0;
  g.x[n - 1] = 1.0;
  for (int i = 1; i < n - 1; ++i) g.w[i] = g.w[i] / (1.0 - g.x[i] * g.x[i]);
  const int deg = n - 1;
  g.w[0] = end_weight(deg, 0.0, 0.0, false) / (2.0 * jacobi_eval(deg, 0, 0, g.x[0]).pd);
  g.w[n - 1] = end_weight(deg, 0.0, 0.0, true) / (2.0 * jacobi_eval(deg, 0, 0, g.x[n - 1]).pd);
  if (n % 2) g.x[(n - 1) / 2] = 0.0;
  const double dd = deg, al = dd * (dd + 1.0);
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) {
      double h;
      if (i == 0 && j == 0) h = -dd * (dd + 1.0) / 4.0;
      else if (i == deg && j == deg) h = dd * (dd + 1.0) / 4.0;
      else if (i == j) h = 0.0;
      else {
        const double l1 = legendre(g.x[j], deg), l2 = legendre_deriv(g.x[j], deg);
        const double l3 = legendre(g.x[i], deg), dz = g.x[j] - g.x[i];
        h = l1 / (l3 * dz) + (1.0 - g.x[j] * g.x[j]) * l2 / (dd * (dd + 1.0) * l3 * dz * dz);
      }
      g.H[i + n * j] = h;
    }
  (void)al;
  return g;
}

// Lagrange interpolant through the GLL points (gll.f90:269-296)
double lagrange(int i, double z, const Gll &g) {
  if (std::fabs(z - g.x[i]) < 1.0e-5) return 1.0;
  const int n = g.n - 1;
  const double al = double(n) * (double(n) + 1.0);
  return -(1.0 - z * z) * legendre_deriv(z, n) / (al * legendre(g.x[i], n) * (z - g.x[i]));
}

// --------------------------------------------------------------------
// Reverse Cuthill-McKee ordering of the 8-neighbour element graph of an
// nx x nz box (mesh_structured.f90:204-269 with rcm.f90: root_find by
// pseudo-peripheral search, level-by-level ordering with neighbours sorted
// by increasing degree, then reversal).  Returns perm[new] = old (0-based).
class ElementGraph {
 public:
  ElementGraph(int nx, int nz) : nx_(nx), nz_(nz), row_(size_t(nx) * nz + 1) {
    static const int di[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
    static const int dj[8] = {-1, -1, -1, 0, 0, 1, 1, 1};
    adj_.reserve(size_t(nx) * nz * 8);
    for (int j = 0; j < nz; ++j)
      for (int i = 0; i < nx; ++i) {
        row_[size_t(j) * nx + i] = int(adj_.size());
        for (int q = 0; q < 8; ++q) {
          const int ii = i + di[q], jj = j + dj[q];
          if (ii >= 0 && ii < nx && jj >= 0 && jj < nz) adj_.push_back(jj * nx + ii);
        }
      }
    row_[size_t(nx) * nz] = int(adj_.size());
  }
  int size() const { return nx_ * nz_; }
  int begin(int v) const { return row_[v]; }
  int end(int v) const { return row_[v + 1]; }
  int at(int k) const { return adj_[k]; }

 private:
  int nx_, nz_;
  std::vector<int> row_, adj_;
};

// breadth-first level structure from root among unmasked vertices
int level_structure(const ElementGraph &G, int root, std::vector<char> &mask,
                    std::vector<int> &level, std::vector<int> &level_start) {
  level.clear();
  level_start.clear();
  mask[root] = 0;
  level.push_back(root);
  size_t lbegin = 0;
  while (true) {
    const size_t lend = level.size();
    level_start.push_back(int(lbegin));
    for (size_t i = lbegin; i < lend; ++i) {
      const int v = level[i];
      for (int k = G.begin(v); k < G.end(v); ++k) {
        const int u = G.at(k);
        if (mask[u]) {
          mask[u] = 0;
          level.push_back(u);
        }
      }
    }
    if (level.size() == lend) break;
    lbegin = lend;
  }
  for (int v : level) mask[v] = 1;
  level_start.push_back(int(level.size()));
  return int(level_start.size()) - 1;  // number of levels
}

std::vector<int> rcm_order(int nx, int nz) {
  ElementGraph G(nx, nz);
  const int n = G.size();
  std::vector<char> mask(n, 1);
  std::vector<int> perm;
  perm.reserve(n);
  std::vector<int> level, lstart, deg(n, 0);
  for (int start = 0; start < n; ++start) {
    if (!mask[start]) continue;
    // pseudo-peripheral root
    int root = start;
    int nlev = level_structure(G, root, mask, level, lstart);
    const int ncomp = int(level.size());
    if (nlev != 1 && nlev != ncomp) {
      while (true) {
        int mindeg = ncomp;
        const int last = lstart[nlev - 1];
        root = level[last];
        if (last < ncomp - 1) {
          for (int j = last; j < ncomp; ++j) {
            const int v = level[j];
            int d = 0;
            for (int k = G.begin(v); k < G.end(v); ++k) d += mask[G.at(k)] > 0;
            if (d < mindeg) {
              root = v;
              mindeg = d;
            }
          }
        }
        const int nlev2 = level_structure(G, root, mask, level, lstart);
        if (nlev2 <= nlev) break;
        nlev = nlev2;
        if (ncomp <= nlev) break;
      }
    }
    // degrees within the component (counted over unmasked neighbours)
    const size_t base = perm.size();
    {
      std::vector<char> seen(n, 0);
      std::vector<int> q{root};
      seen[root] = 1;
      for (size_t i = 0; i < q.size(); ++i) {
        const int v = q[i];
        int d = 0;
        for (int k = G.begin(v); k < G.end(v); ++k) {
          const int u = G.at(k);
          if (mask[u]) {
            ++d;
            if (!seen[u]) {
              seen[u] = 1;
              q.push_back(u);
            }
          }
        }
        deg[v] = d;
      }
    }
    // Cuthill-McKee: children of each vertex, sorted by increasing degree
    mask[root] = 0;
    perm.push_back(root);
    size_t lvl_end = base, lnbr = base + 1;
    while (lvl_end < lnbr) {
      const size_t lbegin = lvl_end;
      lvl_end = lnbr;
      for (size_t i = lbegin; i < lvl_end; ++i) {
        const int v = perm[i];
        const size_t first = lnbr;
        for (int k = G.begin(v); k < G.end(v); ++k) {
          const int u = G.at(k);
          if (mask[u]) {
            mask[u] = 0;
            perm.push_back(u);
            ++lnbr;
          }
        }
        // stable insertion sort by degree of perm[first+1, lnbr); as in
        // rcm.f90:571-590 the first child is never compared and stays first
        for (size_t a = first + 2; a < lnbr; ++a) {
          const int u = perm[a];
          size_t b = a;
          while (b > first + 1 && deg[perm[b - 1]] > deg[u]) {
            perm[b] = perm[b - 1];
            --b;
          }
          perm[b] = u;
        }
      }
    }
    std::reverse(perm.begin() + long(base), perm.end());
  }
  return perm;
}

}  // namespace

// ----------------------------------------------------------------------
// Grid: control mesh, lattice, numbering, coordinates, boundary tables.
struct sem2d_grid {
  int ngll = 0, ndof = 0, nx = 0, nz = 0, ezflt = 0, npoin = 0, nelem = 0;
  Gll gll;
  // control nodes on a structured grid of nxp columns (row by row, the split
  // row of a fault duplicated): ngnod 4 (Q4) or 9 (Q9, every other control
  // node a vertex); flat: rectangles, MESH_CART (grid%flat,
  // mesh_cartesian.f90:238) -- MESH_LAYERS_build sets it false
  int ngnod = 4, nxp = 0;
  bool flat = true;
  std::vector<double> cx, cz;
  std::vector<int> elem_ex, elem_ez;  // structured position of element e (RCM order)
  std::vector<int> tag;
  std::vector<int> ibool;         // (ngll,ngll,nelem), 1-based
  std::vector<double> coord;      // (2,npoin)
  int LX = 0, LZ = 0;             // lattice size
  std::vector<int> lattice;       // node number at lattice (I,J), 1-based
  std::vector<int> row0;          // lattice row of local j=0 for element row ez
  struct Boundary {
    int tag;
    std::vector<int> elem, edge;  // 1-based element, edge 1..4
    std::vector<int> node;        // 1-based bulk nodes in boundary order
    std::vector<int> ib;          // (ngll, nelem_b) boundary-node index, 1-based
  };
  std::vector<Boundary> bnds;
  const Boundary *find(int t) const {
    for (auto &b : bnds)
      if (b.tag == t) return &b;
    return nullptr;
  }
  // lattice index of GLL point (i,j) of element e
  size_t lat(int e, int i, int j) const {
    const int I = elem_ex[e] * (ngll - 1) + i;
    const int J = row0[elem_ez[e]] + j;
    return size_t(J) * LX + I;
  }
  // control nodes of element e in the order of knods
  // (MESH_STRUCTURED_connectivity, mesh_structured.f90:31-99):
  // (x1,z1,...), the four vertices counterclockwise first
  void control(int e, double *c) const {
    const int d = ngnod == 9 ? 2 : 1;
    const int i = d * elem_ex[e];
    const int j = d * elem_ez[e] + (ezflt > 0 && elem_ez[e] >= ezflt ? 1 : 0);  // control row, split shift
    static const int di9[9] = {0, 2, 2, 0, 1, 2, 1, 0, 1}, dj9[9] = {0, 0, 2, 2, 0, 1, 2, 1, 1};
    static const int di4[4] = {0, 1, 1, 0}, dj4[4] = {0, 0, 1, 1};
    for (int k = 0; k < ngnod; ++k) {
      const size_t q = size_t(j + (ngnod == 9 ? dj9[k] : dj4[k])) * nxp + (i + (ngnod == 9 ? di9[k] : di4[k]));
      c[2 * k] = cx[q];
      c[2 * k + 1] = cz[q];
    }
  }
  // the four vertices
  void corners(int e, double *c) const {
    double a[18];
    control(e, a);
    std::copy(a, a + 8, c);
  }
};

namespace {

// Q4 shape functions (elem_q4.f90:43-95)
inline void q4_shape(double s, double t, double *sh) {
  const double sp = s + 1.0, sm = s - 1.0, tp = t + 1.0, tm = t - 1.0;
  sh[0] = 0.25 * sm * tm;
  sh[1] = -(0.25 * sp * tm);
  sh[2] = 0.25 * sp * tp;
  sh[3] = -(0.25 * sm * tp);
}
inline void q4_dshape(double s, double t, double *d) {
  const double sp = s + 1.0, sm = s - 1.0, tp = t + 1.0, tm = t - 1.0;
  d[0] = 0.25 * tm; d[1] = -(0.25 * tm); d[2] = 0.25 * tp; d[3] = -(0.25 * tp);
  d[4] = 0.25 * sm; d[5] = -(0.25 * sp); d[6] = 0.25 * sp; d[7] = -(0.25 * sm);
}
// Q9 shape functions and derivatives (elem_q9.f90:40-110)
inline void q9_shape(double s, double t, double *sh) {
  const double sp = s + 1.0, sm = s - 1.0, tp = t + 1.0, tm = t - 1.0, ss = s * s, tt = t * t, st = s * t;
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
inline void q9_dshape(double s, double t, double *d) {  // d[k] d/ds, d[9 + k] d/dt
  const double sp = s + 1.0, sm = s - 1.0, tp = t + 1.0, tm = t - 1.0, ss = s * s, tt = t * t, st = s * t;
  const double s2 = s * 2.0, t2 = t * 2.0;
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
inline void shape(int ngnod, double s, double t, double *sh) {
  if (ngnod == 9) q9_shape(s, t, sh);
  else q4_shape(s, t, sh);
}
// sum_k c(a,k) w(k) in increasing k (matmul(coorg, shape))
inline double interp(const double *c, int ngnod, int a, const double *w) {
  double acc = c[a] * w[0];
  for (int k = 1; k < ngnod; ++k) acc = acc + c[a + 2 * k] * w[k];
  return acc;
}
inline double interp4(const double *c, int a, const double *w) { return interp(c, 4, a, w); }
// Jacobian [dx/dxi dx/deta; dz/dxi dz/deta] at (s,t), column-major
// (SE_Jacobian: matmul(coorg, dshape), spec_grid.f90:551-583)
inline void jacobian(int ngnod, const double *c, double s, double t, double *J) {
  double d[18];
  if (ngnod == 9) {
    q9_dshape(s, t, d);
  } else {
    double d4[8];
    q4_dshape(s, t, d4);
    for (int k = 0; k < 4; ++k) {
      d[k] = d4[k];
      d[9 + k] = d4[4 + k];
    }
  }
  for (int b = 0; b < 2; ++b)
    for (int a = 0; a < 2; ++a) J[a + 2 * b] = interp(c, ngnod, a, d + 9 * b);
}
inline void jacobian(const double *c, double s, double t, double *J) { jacobian(4, c, s, t, J); }

void edge_ij(int n, int edge, int k, int &i, int &j) {
  switch (edge) {
    case 1: i = k; j = 0; break;
    case 2: i = n - 1; j = k; break;
    case 3: i = n - 1 - k; j = n - 1; break;
    default: i = 0; j = n - 1 - k; break;
  }
}

void build_lattice(sem2d_grid &g, int ezflt, const std::vector<int> &tag_s);

// MESH_CART_build (mesh_cartesian.f90:238-314)
void build_cartesian(sem2d_grid &g, const sem2d_deck &dk) {
  const int nx = dk.nelem[0], nz = dk.nelem[1];
  if (nx <= 0 || nz <= 0) throw BuildError("CART_read: nelem must be positive");
  if (dk.ngll < 2 || dk.ngll > 20) throw BuildError("ngll out of range");
  if (dk.ndof != 1 && dk.ndof != 2) throw BuildError("ndof must be 1 or 2");
  int ezflt = dk.ezflt;
  if (ezflt >= nz) throw BuildError("CART_read: ezflt must be < nelem(2)");
  if (ezflt == -1) ezflt = nz / 2;
  if (ezflt < -1) throw BuildError("CART_read: ezflt must be >= -1");
  g.ngll = dk.ngll;
  g.ndof = dk.ndof;
  g.nx = nx;
  g.nz = nz;
  g.ezflt = ezflt;
  g.nelem = nx * nz;
  g.gll = make_gll(dk.ngll);
  // control-node coordinates (mesh_cartesian.f90:248-263); the fault row is
  // duplicated in zc
  const double hx = (dk.xlim[1] - dk.xlim[0]) / double(nx);
  const double hz = (dk.zlim[1] - dk.zlim[0]) / double(nz);
  std::vector<double> xc(nx + 1), zc;
  for (int i = 0; i <= nx; ++i) xc[i] = dk.xlim[0] + hx * double(i);
  for (int j = 0; j <= nz; ++j) {
    zc.push_back(dk.zlim[0] + hz * double(j));
    if (ezflt > 0 && j == ezflt) zc.push_back(dk.zlim[0] + hz * double(j));
  }
  g.ngnod = 4;
  g.nxp = nx + 1;
  for (double z : zc)
    for (double x : xc) {
      g.cx.push_back(x);
      g.cz.push_back(z);
    }
  // domain tags in structured order
  std::vector<int> tag_s(size_t(nx) * nz, dk.ndomains == 0 ? 1 : 0);
  for (int d = 0; d < dk.ndomains; ++d) {
    const sem2d_domain &dm = dk.domains[d];
    if (dm.tag < 1) throw BuildError("CART_read: tag null, negative or missing");
    if (dm.ex[0] < 1 || dm.ex[0] > nx || dm.ex[1] < 1 || dm.ex[1] > nx || dm.ez[0] < 1 ||
        dm.ez[0] > nz || dm.ez[1] < 1 || dm.ez[1] > nz)
      throw BuildError("CART_read: domain index out of bounds");
    for (int i = dm.ex[0]; i <= dm.ex[1]; ++i)
      for (int j = dm.ez[0]; j <= dm.ez[1]; ++j) tag_s[size_t(j - 1) * nx + (i - 1)] = dm.tag;
  }
  if (dk.fztag > 0) {
    const int fznz = dk.fznz > 0 ? dk.fznz : 1;
    const int j1 = std::max(ezflt + 1 - fznz, 1), j2 = std::min(ezflt + fznz, nz);
    for (int j = j1; j <= j2; ++j)
      for (int i = 1; i <= nx; ++i) tag_s[size_t(j - 1) * nx + (i - 1)] = dk.fztag;
  }
  for (int t : tag_s)
    if (t == 0) throw BuildError("CART_build: Domain tags not entirely set");
  build_lattice(g, ezflt, tag_s);
}

// MESH_LAYERS_build (mesh_layers.f90:331-449): control rows from zmin up,
// each layer's rows interpolated between its bottom and its top boundary
// (layer_top at the nxp control abscissae), the row of the fault split
// duplicated; Q4 when every top is flat or piecewise linear, Q9 otherwise
void build_layered(sem2d_grid &g, const sem2d_deck &dk) {
  const int nx = dk.nelem[0], nl = dk.nlayer;
  if (nx <= 0) throw BuildError("MESH_LAYERS_read: nx must be positive");
  if (nl <= 0 || nl > SEM2D_MAX_LAYERS) throw BuildError("MESH_LAYERS_read: nlayer or file must be set");
  if (dk.ngll < 2 || dk.ngll > 20) throw BuildError("ngll out of range");
  if (dk.ndof != 1 && dk.ndof != 2) throw BuildError("ndof must be 1 or 2");
  int ngnod = 4, nz = 0;
  for (int k = 0; k < nl; ++k) {
    if (dk.layer_nz[k] <= 0) throw BuildError("MESH_LAYERS_read: nz null, negative or missing");
    if (dk.layer_tag[k] < 1) throw BuildError("MESH_LAYERS_read: tag null, negative or missing");
    if (dk.layer_ngnod[k] != 4 && dk.layer_ngnod[k] != 9) throw BuildError("MESH_LAYERS_read: unsupported layer top");
    ngnod = std::max(ngnod, dk.layer_ngnod[k]);
    nz += dk.layer_nz[k];
  }
  int ezflt = dk.ezflt;
  if (ezflt == -1) ezflt = nz / 2;
  if (ezflt < -1) throw BuildError("MESH_LAYERS_read: ezflt must be >= -1");
  if (ezflt >= nz) throw BuildError("MESH_LAYERS_read: ezflt must be < nz");
  const int d = ngnod == 9 ? 2 : 1, nxp = d * nx + 1;
  g.ngll = dk.ngll;
  g.ndof = dk.ndof;
  g.nx = nx;
  g.nz = nz;
  g.ezflt = ezflt;
  g.nelem = nx * nz;
  g.gll = make_gll(dk.ngll);
  g.ngnod = ngnod;
  g.nxp = nxp;
  g.flat = false;
  std::vector<double> x(nxp);
  for (int i = 0; i < nxp; ++i) x[i] = dk.xlim[0] + (dk.xlim[1] - dk.xlim[0]) / double(nxp - 1) * double(i);
  for (int k = 0; k < nl; ++k) {
    if (!dk.layer_top[k]) throw BuildError("MESH_LAYERS_build: layer top missing");
    for (int i = 0; i < nxp; ++i)
      if (dk.layer_top[k][i] < dk.zmin)
        throw BuildError("MESH_LAYERS_build: zmin in MESH_LAYERED should be deeper than all layer interfaces");
  }
  auto row = [&](const std::vector<double> &zr) {
    g.cx.insert(g.cx.end(), x.begin(), x.end());
    g.cz.insert(g.cz.end(), zr.begin(), zr.end());
  };
  std::vector<double> bot(nxp, dk.zmin), xbot = x;
  row(bot);
  int jposlast = 1;
  for (int k = 0; k < nl; ++k) {  // bottom to top
    const double *top = dk.layer_top[k];
    const int nj = d * dk.layer_nz[k];
    const int jposflt = d * ezflt + 1 - jposlast;
    for (int j = 1; j <= nj; ++j) {
      std::vector<double> zr(nxp), xr(nxp);
      for (int i = 0; i < nxp; ++i) {
        xr[i] = xbot[i] + double(j) / double(nj) * (x[i] - xbot[i]);
        zr[i] = bot[i] + double(j) / double(nj) * (top[i] - bot[i]);
      }
      const int reps = j == jposflt ? 2 : 1;
      for (int r = 0; r < reps; ++r) {
        g.cx.insert(g.cx.end(), xr.begin(), xr.end());
        g.cz.insert(g.cz.end(), zr.begin(), zr.end());
      }
    }
    jposlast += nj;
    bot.assign(top, top + nxp);  // the next layer starts from this top (bot => top)
    xbot = x;
  }
  // tags: layer tags, then the fault zone
  std::vector<int> tag_s(size_t(nx) * nz, 0);
  int jl = 0;
  for (int k = 0; k < nl; ++k)
    for (int j = 0; j < dk.layer_nz[k]; ++j, ++jl)
      for (int i = 0; i < nx; ++i) tag_s[size_t(jl) * nx + i] = dk.layer_tag[k];
  if (dk.fztag > 0 && ezflt > 0) {
    const int fznz = dk.fznz > 0 ? dk.fznz : 1;
    const int j1 = std::max(ezflt + 1 - fznz, 1), j2 = std::min(ezflt + fznz, nz);
    for (int j = j1; j <= j2; ++j)
      for (int i = 1; i <= nx; ++i) tag_s[size_t(j - 1) * nx + (i - 1)] = dk.fztag;
  }
  for (int t : tag_s)
    if (t == 0) throw BuildError("MESH_LAYERS_build: Domain tags not entirely set");
  build_lattice(g, ezflt, tag_s);
}

void build_lattice(sem2d_grid &g, int ezflt, const std::vector<int> &tag_s) {
  const int nx = g.nx, nz = g.nz, N = g.ngll;
  // element order
  const std::vector<int> perm = rcm_order(nx, nz);
  std::vector<int> inv(perm.size());
  for (size_t k = 0; k < perm.size(); ++k) inv[perm[k]] = int(k);
  g.elem_ex.resize(g.nelem);
  g.elem_ez.resize(g.nelem);
  g.tag.resize(g.nelem);
  for (int e = 0; e < g.nelem; ++e) {
    g.elem_ex[e] = perm[e] % nx;
    g.elem_ez[e] = perm[e] / nx;
    g.tag[e] = tag_s[perm[e]];
  }
  // GLL lattice with one extra row at the fault
  g.LX = nx * (N - 1) + 1;
  g.row0.resize(nz);
  for (int j = 0; j < nz; ++j) g.row0[j] = j * (N - 1) + (ezflt > 0 && j >= ezflt ? 1 : 0);
  g.LZ = g.row0[nz - 1] + N;
  g.lattice.assign(size_t(g.LX) * g.LZ, 0);
  // numbering (spec_grid.f90:198-314) on the lattice
  int np = 0;
  for (int e = 0; e < g.nelem; ++e) {
    for (int j = 1; j < N - 1; ++j)
      for (int i = 1; i < N - 1; ++i) g.lattice[g.lat(e, i, j)] = ++np;
    for (int ed = 1; ed <= 4; ++ed) {
      int i, j;
      edge_ij(N, ed, 1, i, j);
      if (g.lattice[g.lat(e, i, j)] > 0) continue;
      for (int k = 1; k < N - 1; ++k) {
        edge_ij(N, ed, k, i, j);
        g.lattice[g.lat(e, i, j)] = ++np;
      }
    }
    static const int vi[4] = {0, 1, 1, 0}, vj[4] = {0, 0, 1, 1};
    for (int c = 0; c < 4; ++c) {
      const size_t L = g.lat(e, vi[c] * (N - 1), vj[c] * (N - 1));
      if (g.lattice[L] == 0) g.lattice[L] = ++np;
    }
  }
  g.npoin = np;
  g.ibool.resize(size_t(N) * N * g.nelem);
  for (int e = 0; e < g.nelem; ++e)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) g.ibool[i + N * (j + size_t(N) * e)] = g.lattice[g.lat(e, i, j)];
  // coordinates: the last element (in element order) writes a shared node
  g.coord.assign(2 * size_t(np), 0.0);
  const int ng = g.ngnod;
  std::vector<double> shp(size_t(ng) * N * N);
  for (int j = 0; j < N; ++j)
    for (int i = 0; i < N; ++i) shape(ng, g.gll.x[i], g.gll.x[j], &shp[ng * (i + N * j)]);
  for (int e = 0; e < g.nelem; ++e) {
    double c[18];
    g.control(e, c);
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        const int p = g.ibool[i + N * (j + size_t(N) * e)] - 1;
        g.coord[2 * p] = interp(c, ng, 0, &shp[ng * (i + N * j)]);
        g.coord[2 * p + 1] = interp(c, ng, 1, &shp[ng * (i + N * j)]);
      }
  }
  // boundaries: tags 1..4 = bottom, right, top, left; 5/6 = fault sides
  auto add_bnd = [&](int t, int edge, auto elem_of, int count, bool horizontal_line, int line) {
    sem2d_grid::Boundary b;
    b.tag = t;
    for (int q = 0; q < count; ++q) {
      b.elem.push_back(inv[elem_of(q)] + 1);
      b.edge.push_back(edge);
    }
    // lattice line in increasing coordinate
    if (horizontal_line)
      for (int I = 0; I < g.LX; ++I) b.node.push_back(g.lattice[size_t(line) * g.LX + I]);
    else
      for (int J = 0; J < g.LZ; ++J) b.node.push_back(g.lattice[size_t(J) * g.LX + line]);
    // position of each node of each boundary element in b.node
    b.ib.resize(size_t(N) * count);
    for (int q = 0; q < count; ++q) {
      const int e = b.elem[q] - 1;
      for (int k = 0; k < N; ++k) {
        int i, j;
        edge_ij(N, edge, k, i, j);
        const size_t L = g.lat(e, i, j);
        const int pos = horizontal_line ? int(L % g.LX) : int(L / g.LX);
        b.ib[k + size_t(N) * q] = pos + 1;
      }
    }
    g.bnds.push_back(std::move(b));
  };
  add_bnd(1, 1, [&](int q) { return q; }, nx, true, 0);
  add_bnd(2, 2, [&](int q) { return q * nx + nx - 1; }, nz, false, g.LX - 1);
  add_bnd(3, 3, [&](int q) { return (nz - 1) * nx + q; }, nx, true, g.LZ - 1);
  add_bnd(4, 4, [&](int q) { return q * nx; }, nz, false, 0);
  if (ezflt > 0) {
    add_bnd(5, 3, [&](int q) { return (ezflt - 1) * nx + q; }, nx, true, g.row0[ezflt - 1] + N - 1);
    add_bnd(6, 1, [&](int q) { return ezflt * nx + q; }, nx, true, g.row0[ezflt]);
  }
}

void build_grid(sem2d_grid &g, const sem2d_deck &dk) {
  if (dk.mesh_method == 1) build_layered(g, dk);
  else build_cartesian(g, dk);
}

}  // namespace

// ----------------------------------------------------------------------
struct sem2d_problem {
  const sem2d_grid *g = nullptr;
  int ndof = 0, time_kind = 0, nt = 0;
  double dt = 0, courant = 0, beta = 0, gamma = 0.5, alpha = 1.0;
  std::vector<double> Kx, Kz, la, mu, mux, rho, cp, cs, kveta;
  bool has_kv = false;
  std::vector<double> mass;  // becomes rmass
  std::vector<int> abs_node;
  std::vector<double> abs_C;  // built per dof then transposed at export
  std::vector<std::vector<double>> abs_Cd;
  // per absorbing entry: boundary weight, outward normal (n0 then n1 at
  // export) and whether the incident wave enters there
  std::vector<double> abs_B, abs_n0, abs_n1, abs_n;
  std::vector<int> abs_wave;
  // time-dependent Neumann tractions of &BC_DIRNEU
  std::vector<int> neu_node, neu_comp, neu_stf;
  std::vector<double> neu_B;
  std::vector<sem2d_stf> neu_stfs;
  // source time function other than Ricker and the incident plane wave;
  // TAB rows are copied (tabs) so the descriptor outlives the deck
  bool has_src_stf = false;
  sem2d_stf src_stf{};
  int wave_phase = 0;
  double wave_angle = 0, wave_ref[2] = {0, 0}, wave_cp = 0, wave_cs = 0, wave_mu = 0, wave_lambda = 0,
         wave_tdelay = 0;
  sem2d_stf wave_stf{};
  std::vector<std::unique_ptr<std::vector<double>>> tabs;
  // Stacey P3 terms, one per (boundary element, edge point)
  std::vector<int> st_node, st_k, st_edge;
  std::vector<double> st_K0, st_K1;
  // zero-Dirichlet components
  std::vector<int> dir_node, dir_comp, dir_after;
  // periodic node pairs
  std::vector<int> per_master, per_slave;
  // fault
  int nflt = 0;
  bool two = false;
  std::vector<int> node1, node2;
  std::vector<double> fcoord, n1, B, invM1, invM2, Z, T0, coh;
  double coefA2V = 0, coefA2D = 0;
  std::vector<double> prm[SEM2D_FP_NPARAM];
  int oit = 0, oitd = 1, oix1 = 1, oixn = 1, oixd = 1, fnsamp = 0;
  // sources, receivers
  std::vector<int> src_node;
  std::vector<double> src_dir, src_f0, src_t0, src_amp, src_rel, src_tdelay;
  int nrec = 0, rec_isamp = 1, rec_nsamp = 0;
  char rec_field = 'V';
  std::vector<int> rec_node, rec_elem;
  std::vector<double> rec_interp, rec_coord;
  std::vector<double> H, w;
  // a grid that is not flat: inverse Jacobian and weights at every element
  // GLL point (SE_InverseJacobian, SE_VolumeWeights)
  std::vector<double> xjaci, dvol;
  sem2d_deck deck{};
};

namespace {

const sem2d_material *find_mat(const sem2d_deck &dk, int tag) {
  for (int m = 0; m < dk.nmats; ++m)
    if (dk.mats[m].tag == tag) return &dk.mats[m];
  return nullptr;
}

void build_materials(sem2d_problem &P, const sem2d_deck &dk) {
  const sem2d_grid &g = *P.g;
  const size_t n2 = size_t(g.ngll) * g.ngll, np = n2 * g.nelem;
  for (auto *v : {&P.Kx, &P.Kz, &P.la, &P.mu, &P.mux, &P.rho, &P.cp, &P.cs}) v->assign(np, 0.0);
  for (int m = 0; m < dk.nmats; ++m) P.has_kv |= dk.mats[m].kv != 0;
  if (P.has_kv) P.kveta.assign(np, 0.0);
  for (int e = 0; e < g.nelem; ++e) {
    const sem2d_material *m = find_mat(dk, g.tag[e]);
    if (!m) throw BuildError("element tag " + std::to_string(g.tag[e]) + " has no material");
    if (!m->hetero && m->rho <= 0.0) throw BuildError("MAT_ELAST_read: undefined density (rho)");
    if (m->hetero && (!dk.h_rho || (!m->aniso && (!dk.h_cp || !dk.h_cs)) ||
                      (m->aniso && (!dk.h_c11 || !dk.h_c13 || !dk.h_c33 || !dk.h_c55 || !dk.h_c66))))
      throw BuildError("heterogeneous material without per-point arrays");
    if (!m->aniso && !m->hetero && m->cp > 0 && m->cs > 0) {
      const double mu = m->rho * m->cs * m->cs, K = m->rho * m->cp * m->cp;
      const double lam = m->rho * (m->cp * m->cp - 2.0 * m->cs * m->cs);
      const double poiss = 0.5 * lam / (K - mu);
      if (poiss < 0.0 || poiss > 0.5) throw BuildError("Poisson's ratio out of range !");
    }
    for (size_t q = 0; q < n2; ++q) {
      const size_t p = q + n2 * e;
      const double rho = m->hetero ? dk.h_rho[p] : m->rho;
      P.rho[p] = rho;
      if (!m->aniso) {
        const double cp = m->hetero ? dk.h_cp[p] : m->cp, cs = m->hetero ? dk.h_cs[p] : m->cs;
        const double lam = rho * (cp * cp - 2.0 * cs * cs), mu = rho * cs * cs;
        P.cp[p] = cp;
        P.cs[p] = cs;
        P.la[p] = lam;
        P.mu[p] = mu;
        P.mux[p] = mu;
        P.Kx[p] = lam + 2.0 * mu;
        P.Kz[p] = P.Kx[p];
      } else {
        auto val = [&](double c, const double *h) { return m->hetero ? h[p] : c; };
        const double c11 = val(m->c11, dk.h_c11), c13 = val(m->c13, dk.h_c13);
        const double c33 = val(m->c33, dk.h_c33), c55 = val(m->c55, dk.h_c55);
        const double c66 = val(m->c66, dk.h_c66);
        P.la[p] = c13;
        P.mu[p] = c55;
        P.mux[p] = c66;
        P.Kx[p] = c11;
        P.Kz[p] = c33;
        P.cp[p] = std::sqrt(c11 / rho);
        P.cs[p] = std::sqrt(c55 / rho);
      }
      if (P.has_kv) P.kveta[p] = m->kv ? ((m->hetero && dk.h_kveta) ? dk.h_kveta[p] : m->kv_eta) : 0.0;
    }
  }
}

// CHECK_grid (init.f90:145-289) and TIME_read/TIME_init (time.f90:122-395)
void build_time(sem2d_problem &P, const sem2d_deck &dk) {
  const sem2d_grid &g = *P.g;
  const int N = g.ngll;
  const size_t n2 = size_t(N) * N;
  double lam_min = 1e308, max_c_dx = 0.0;
  for (int e = 0; e < g.nelem; ++e) {
    double c[8];
    g.corners(e, c);
    double hsq[4] = {(c[2] - c[0]) * (c[2] - c[0]) + (c[3] - c[1]) * (c[3] - c[1]),
                     (c[4] - c[2]) * (c[4] - c[2]) + (c[5] - c[3]) * (c[5] - c[3]),
                     (c[6] - c[4]) * (c[6] - c[4]) + (c[7] - c[5]) * (c[7] - c[5]),
                     (c[6] - c[0]) * (c[6] - c[0]) + (c[7] - c[1]) * (c[7] - c[1])};
    const double hmax = std::sqrt(*std::max_element(hsq, hsq + 4));
    const double *cs = &P.cs[n2 * e], *cp = &P.cp[n2 * e];
    lam_min = std::min(lam_min, *std::min_element(cs, cs + n2) / hmax);
    const double *cel = g.ndof == 2 ? cp : cs;
    double rmax = 0.0;
    for (int j = 0; j < N - 1; ++j)
      for (int i = 0; i < N - 1; ++i) {
        const int p0 = g.ibool[i + N * (j + size_t(N) * e)] - 1;
        const int p1 = g.ibool[(i + 1) + N * (j + size_t(N) * e)] - 1;
        const int p2 = g.ibool[i + N * ((j + 1) + size_t(N) * e)] - 1;
        const double *c0 = &g.coord[2 * p0], *c1 = &g.coord[2 * p1], *c2 = &g.coord[2 * p2];
        const double r1 = std::sqrt((c1[0] - c0[0]) * (c1[0] - c0[0]) + (c1[1] - c0[1]) * (c1[1] - c0[1]));
        const double r2 = std::sqrt((c2[0] - c0[0]) * (c2[0] - c0[0]) + (c2[1] - c0[1]) * (c2[1] - c0[1]));
        rmax = std::max(rmax, cel[i + N * j] / std::min(r1, r2));
      }
    max_c_dx = std::max(max_c_dx, rmax);
  }
  if (double(N) * lam_min / dk.fmax < 5.0)
    throw BuildError("warning: low resolution at fmax (the reference aborts on warnings)");
  int nsteps = dk.nsteps;
  double dt = dk.dt, courant = dk.courant, total = dk.total_time;
  if (nsteps < 0 || dt < 0 || total < 0) throw BuildError("TIME: negative setting");
  if (courant < 0.0 || courant > 0.6) throw BuildError("TIME: Courant out of range [0,0.6]");
  if (double(nsteps) * total != 0.0)
    throw BuildError("TIME: bad combination of settings, NbSteps or TotalTime");
  if (dt > 0.0) {
    if (total > 0.0) nsteps = int(std::ceil(total / dt));
    total = dt * nsteps;
  }
  P.time_kind = dk.time_kind;
  double omega = 2.0;
  if (dk.time_kind == SEM2D_TIME_NEWMARK) {
    P.beta = dk.beta;
    P.gamma = dk.gamma;
    if (P.beta < 0 || P.beta > 1 || P.gamma < 0 || P.gamma > 1)
      throw BuildError("TIME_NEWMARK: parameter out of range");
    omega = std::sqrt(2.0 / P.gamma);
  } else if (dk.time_kind == SEM2D_TIME_HHT) {
    // TIME_read 'HHT-alpha' (time.f90:222-240): second order, gamma = 3/2 -
    // alpha, beta from alpha and the spectral radius rho
    const double a = dk.hht_alpha, r = dk.hht_rho;
    if (a < 0.0 || a > 1.0) throw BuildError("TIME_HHTA: alpha is out of range [0,1]");
    if (r < 0.5 || r > 1.0) throw BuildError("TIME_HHTA: rho is out of range [0.5,1]");
    P.alpha = a;
    P.gamma = 1.5 - a;
    const double q = 1.0 + r, r2 = r * r, r3 = r2 * r, r4 = r3 * r, r5 = r4 * r;
    P.beta = a != 1.0 ? 1.0 - a - r * r * (r - 1.0) / ((1.0 - a) * (q * q * q)) : 0.0;
    omega = std::sqrt(-4.0 * (q * q * q * q * q) / (r5 + 9.0 * r4 - 34.0 * r3 + 6.0 * r2 - 15.0 * r + 1.0));
  } else if (dk.time_kind != SEM2D_TIME_LEAPFROG) {
    throw BuildError("TIME: unknown time scheme");
  }
  if (dt > 0.0) {
    courant = max_c_dx * dt;
  } else {
    dt = courant / max_c_dx;
    if (total > 0.0) nsteps = int(std::ceil(total / dt));
  }
  if (courant > omega * 3.0 / 7.0 / std::sqrt(2.0))
    throw BuildError("warning: Courant number too high (the reference aborts on warnings)");
  P.dt = dt;
  P.courant = courant;
  P.nt = nsteps;
}

// TIME_getCoefA2V, TIME_getCoefA2D, TIME_getCoefA2Vrhs (time.f90:426-486);
// alpha is 1 for Newmark
bool newmark_like(const sem2d_problem &P) { return P.time_kind == SEM2D_TIME_NEWMARK || P.time_kind == SEM2D_TIME_HHT; }
double coefA2V(const sem2d_problem &P) { return newmark_like(P) ? P.gamma * P.dt : P.dt; }
double coefA2D(const sem2d_problem &P) { return newmark_like(P) ? P.beta * P.dt * P.dt : 0.0; }
double coefA2Vrhs(const sem2d_problem &P) {
  return newmark_like(P) ? P.alpha * coefA2V(P) : 0.5 * coefA2V(P);
}

// SE_InverseJacobian (invert2, utils.f90:88-110) and SE_VolumeWeights
// (spec_grid.f90:590-602) at every element GLL point
void build_general_geometry(sem2d_problem &P) {
  const sem2d_grid &g = *P.g;
  const int N = g.ngll;
  const size_t npt = size_t(N) * N * g.nelem;
  P.xjaci.assign(4 * npt, 0.0);
  P.dvol.assign(npt, 0.0);
  for (int e = 0; e < g.nelem; ++e) {
    double c[18];
    g.control(e, c);
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        double J[4];
        jacobian(g.ngnod, c, g.gll.x[i], g.gll.x[j], J);
        const double det = J[0] * J[3] - J[2] * J[1];
        if (det <= 0.0) throw BuildError("SE_InverseJacobian: undefined Jacobian");
        const size_t q = i + N * (j + size_t(N) * e);
        P.xjaci[4 * q + 0] = J[3] / det;
        P.xjaci[4 * q + 1] = -J[1] / det;
        P.xjaci[4 * q + 2] = -J[2] / det;
        P.xjaci[4 * q + 3] = J[0] / det;
        P.dvol[q] = det * (g.gll.w[i] * g.gll.w[j]);
      }
  }
}

// MAT_MASS_init (mat_mass.f90:29-61)
void build_mass(sem2d_problem &P) {
  const sem2d_grid &g = *P.g;
  const int N = g.ngll;
  P.mass.assign(size_t(g.npoin) * P.ndof, 0.0);
  for (int e = 0; e < g.nelem; ++e) {
    double c[18];
    g.control(e, c);
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        double J[4];
        jacobian(g.ngnod, c, g.gll.x[i], g.gll.x[j], J);
        double dvol = J[0] * J[3] - J[2] * J[1];
        dvol = dvol * (g.gll.w[i] * g.gll.w[j]);
        const size_t q = i + N * (j + size_t(N) * e);
        const int p = g.ibool[q] - 1;
        P.mass[p] = P.mass[p] + P.rho[q] * dvol;
      }
  }
  if (P.ndof == 2) std::copy(P.mass.begin(), P.mass.begin() + g.npoin, P.mass.begin() + g.npoin);
}

// BC_get_normal_and_weights (spec_grid.f90:961-1011)
void normals(const sem2d_grid &g, const sem2d_grid::Boundary &b, std::vector<double> &nrm,
             std::vector<double> &w, bool periodic = false) {
  const int N = g.ngll, np = int(b.node.size());
  nrm.assign(2 * size_t(np), 0.0);
  w.assign(np, 0.0);
  for (size_t q = 0; q < b.elem.size(); ++q) {
    const int e = b.elem[q] - 1, ed = b.edge[q];
    const int ld = (ed == 1 || ed == 3) ? 0 : 1;
    const double sg = (ed == 3 || ed == 4) ? -1.0 : 1.0;
    double c[18];
    g.control(e, c);
    for (int k = 0; k < N; ++k) {
      int i, j;
      edge_ij(N, ed, k, i, j);
      double J[4];
      jacobian(g.ngnod, c, g.gll.x[i], g.gll.x[j], J);
      const double dx = J[0 + 2 * ld], dz = J[1 + 2 * ld];
      const double j1 = std::sqrt(dx * dx + dz * dz);
      const double tx = sg * dx / j1, tz = sg * dz / j1;
      const int bn = b.ib[k + size_t(N) * q] - 1;
      nrm[bn] = nrm[bn] + tz;
      nrm[bn + np] = nrm[bn + np] + (-tx);
      w[bn] = w[bn] + g.gll.w[k] * j1;
    }
  }
  if (periodic) {  // the two ends are one node (spec_grid.f90:998-1003)
    for (int c = 0; c < 2; ++c) {
      nrm[0 + size_t(np) * c] = nrm[0 + size_t(np) * c] + nrm[(np - 1) + size_t(np) * c];
      nrm[(np - 1) + size_t(np) * c] = nrm[0 + size_t(np) * c];
    }
    w[0] = w[0] + w[np - 1];
    w[np - 1] = w[0];
  }
  for (size_t q = 0; q < b.elem.size(); ++q)
    for (int k : {0, N - 1}) {
      const int bn = b.ib[k + size_t(N) * q] - 1;
      const double r = std::sqrt(nrm[bn] * nrm[bn] + nrm[bn + np] * nrm[bn + np]);
      nrm[bn] = nrm[bn] / r;
      nrm[bn + np] = nrm[bn + np] / r;
    }
}

// BC_PERIO_intersects (bc_periodic.f90:108-121): both ends of the boundary
// are periodic nodes
bool perio_intersects(const sem2d_problem &P, const sem2d_grid::Boundary &b) {
  if (P.per_master.empty() || b.node.empty()) return false;
  auto on = [&](int n) {
    for (size_t k = 0; k < P.per_master.size(); ++k)
      if (P.per_master[k] == n || P.per_slave[k] == n) return true;
    return false;
  };
  return on(b.node.front()) && on(b.node.back());
}

// BC_PERIO_init (bc_periodic.f90:42-72): pair the nodes of the two sides in
// list order after checking they differ by one shift, then assemble the
// mass on the master nodes and copy it to the slaves (BC_PERIO_set_field)
void perio_init(sem2d_problem &P, const int tags[2]) {
  const sem2d_grid &g = *P.g;
  const sem2d_grid::Boundary *m = g.find(tags[0]), *s = g.find(tags[1]);
  if (!m || !s) throw BuildError("bc_perio_init: boundary tag not found");
  if (m->elem.size() != s->elem.size()) throw BuildError("bc_perio_init: number of boundary elements do not match");
  if (m->node.size() != s->node.size()) throw BuildError("bc_perio_init: number of nodes on boundaries do not match");
  const double *c0m = &g.coord[2 * size_t(m->node[0] - 1)], *c0s = &g.coord[2 * size_t(s->node[0] - 1)];
  const double sh1 = c0m[0] - c0s[0], sh2 = c0m[1] - c0s[1];
  for (size_t k = 0; k < m->node.size(); ++k) {
    const double *cm = &g.coord[2 * size_t(m->node[k] - 1)], *cs = &g.coord[2 * size_t(s->node[k] - 1)];
    if (std::fabs(cm[0] - cs[0] - sh1) > kTinyXabs || std::fabs(cm[1] - cs[1] - sh2) > kTinyXabs)
      throw BuildError("bc_perio_init: coordinates on boundaries do not match properly");
  }
  for (int d = 0; d < P.ndof; ++d)
    for (size_t k = 0; k < m->node.size(); ++k) {
      double &a = P.mass[size_t(m->node[k] - 1) + size_t(g.npoin) * d];
      double &b = P.mass[size_t(s->node[k] - 1) + size_t(g.npoin) * d];
      a = a + b;
      b = a;
    }
  P.per_master.insert(P.per_master.end(), m->node.begin(), m->node.end());
  P.per_slave.insert(P.per_slave.end(), s->node.begin(), s->node.end());
}

// STF_read (stf_gen.f90:45-97) of a deck value: the checks of the *_read
// routines, the parameters that &STF_RICKER, &STF_GAUSSIAN, &STF_HARMONIC
// and &STF_USER read into REAL variables rounded to FP32, the TAB rows
// copied into the problem.  A deck kind NONE with ricker_* values is the
// Ricker of &STF_RICKER.
sem2d_stf read_stf(sem2d_problem &P, const sem2d_stf &in) {
  sem2d_stf s = in;
  auto r32 = [](double x) { return double(float(x)); };
  switch (in.kind) {
    case SEM2D_STF_RICKER:  // stf_ricker.f90:46-78
      s.f0 = r32(in.f0);
      s.onset = r32(in.onset);
      s.ampli = r32(in.ampli);
      if (s.f0 <= 0.0) throw BuildError("RICKER_read: f0 must be positive");
      // a severe warning, fatal under the default abort_on_warnings (stdio.f90:13,218-227)
      if (float(s.onset) < 1.0f / float(s.f0)) throw BuildError("warning: RICKER_read: Onset time too small");
      break;
    case SEM2D_STF_GAUSSIAN:  // stf_gaussian.f90:36-60
      s.f0 = r32(in.f0);
      s.onset = r32(in.onset);
      s.ampli = r32(in.ampli);
      if (s.f0 < 0.0) throw BuildError("STF_GAUSSIAN_read: f0 must be positive");
      break;
    case SEM2D_STF_BRUNE:  // stf_brune.f90:36-60 (double precision)
      if (in.f0 < 0.0) throw BuildError("STF_BRUNE_read: fc must be positive");
      break;
    case SEM2D_STF_HARMONIC:  // stf_harmonic.f90:33-58
      s.ampli = r32(in.ampli);
      s.f0 = r32(in.f0);
      if (s.f0 <= 0.0) throw BuildError("STF_HARMONIC_read: f0 must be positive");
      if (s.ampli == 0.0) throw BuildError("STF_HARMONIC_read: ampli must be non zero");
      break;
    case SEM2D_STF_USER:  // stf_user.f90:38-80
      s.onset = r32(in.onset);
      s.ampli = r32(in.ampli);
      s.par1 = r32(in.par1);
      s.par2 = r32(in.par2);
      break;
    case SEM2D_STF_TAB: {  // stf_tabulated.f90:37-71
      if (in.ntab < 2 || !in.tab_t || !in.tab_v) throw BuildError("STF_TAB_read: the table needs two rows or more");
      P.tabs.emplace_back(new std::vector<double>(in.tab_t, in.tab_t + in.ntab));
      s.tab_t = P.tabs.back()->data();
      P.tabs.emplace_back(new std::vector<double>(in.tab_v, in.tab_v + in.ntab));
      s.tab_v = P.tabs.back()->data();
      for (int k = 1; k < in.ntab; ++k)
        if (!(in.tab_t[k] > in.tab_t[k - 1])) throw BuildError("STF_TAB_read: times must increase");
      break;
    }
    default:
      throw BuildError("STF_read: unknown source time function ");
  }
  return s;
}

// BC_ABSO_init (bc_abso.f90:115-266), Clayton-Engquist on flat sides, and
// the Stacey P3 coefficients of a P-SV side with stacey=T
// (bc_abso.f90:174-218): K(k,c,e) = w_k |dx/dloc_t| dloc_t/dx_t
// rho cs (2 cs - cp), negated for the tangential component
void abso_init(sem2d_problem &P, int tag, int stacey, int let_wave, bool wave_source) {
  const sem2d_grid &g = *P.g;
  const sem2d_grid::Boundary *b = g.find(tag);
  if (!b) return;  // the reference ignores a BC whose tag is absent (bc_gen.f90:214-219)
  const int N = g.ngll, np = int(b->node.size()), nd = P.ndof;
  const bool periodic = perio_intersects(P, *b);
  std::vector<double> nrm, w;
  normals(g, *b, nrm, w, periodic);
  bool horiz = true, vert = true;
  for (int k = 0; k < np; ++k) {
    horiz &= std::fabs(nrm[k]) < kTinyXabs;
    vert &= std::fabs(nrm[k + np]) < kTinyXabs;
  }
  if (!horiz && !vert) throw BuildError("absorbing boundary is not flat");
  const int gtan = horiz ? 0 : 1, gnor = horiz ? 1 : 0;
  std::vector<double> Cb(size_t(np) * nd, 0.0);
  for (size_t q = 0; q < b->elem.size(); ++q) {
    const int e = b->elem[q] - 1, ed = b->edge[q];
    const int ld = (ed == 1 || ed == 3) ? 0 : 1;
    double c8[18];
    g.control(e, c8);
    for (int k = 0; k < N; ++k) {
      int i, j;
      edge_ij(N, ed, k, i, j);
      const size_t p = i + N * (j + size_t(N) * e);
      double cv[2];
      cv[gnor] = P.cp[p];
      cv[gtan] = P.cs[p];
      double J[4];
      jacobian(g.ngnod, c8, g.gll.x[i], g.gll.x[j], J);
      const double ci = g.gll.w[k] * std::sqrt(J[0 + 2 * ld] * J[0 + 2 * ld] + J[1 + 2 * ld] * J[1 + 2 * ld]);
      const int bk = b->ib[k + size_t(N) * q] - 1;
      if (nd == 1) {
        Cb[bk] = Cb[bk] + P.rho[p] * cv[gtan] * ci;
      } else {
        Cb[bk] = Cb[bk] + P.rho[p] * cv[0] * ci;
        Cb[bk + np] = Cb[bk + np] + P.rho[p] * cv[1] * ci;
      }
      if (stacey && nd == 2) {
        const double det = J[0] * J[3] - J[2] * J[1];
        const double inv[2][2] = {{J[3] / det, -J[2] / det}, {-J[1] / det, J[0] / det}};
        const double K0 = ci * inv[ld][gtan] * (P.rho[p] * cv[gtan] * (2.0 * cv[gtan] - cv[gnor]));
        P.st_node.push_back(b->node[bk]);
        P.st_k.push_back(k);
        for (int l = 0; l < N; ++l) P.st_edge.push_back(b->node[b->ib[l + size_t(N) * q] - 1]);
        P.st_K0.push_back(gtan == 0 ? -K0 : K0);
        P.st_K1.push_back(gtan == 1 ? -K0 : K0);
      }
    }
  }
  if (periodic)  // the two ends are one node (bc_abso.f90:227-231)
    for (int d = 0; d < nd; ++d) {
      Cb[0 + size_t(np) * d] = Cb[0 + size_t(np) * d] + Cb[(np - 1) + size_t(np) * d];
      Cb[(np - 1) + size_t(np) * d] = Cb[0 + size_t(np) * d];
    }
  const double cf = coefA2Vrhs(P);
  for (int d = 0; d < nd; ++d)
    for (int k = 0; k < np; ++k) {
      const size_t p = size_t(b->node[k] - 1) + size_t(g.npoin) * d;
      P.mass[p] = P.mass[p] + cf * Cb[k + size_t(np) * d];
    }
  if (P.abs_Cd.empty()) P.abs_Cd.resize(nd);
  // the first wave source found enters across a flat side with let_wave
  // (bc_abso.f90:245-256); every side here is flat
  const int wave = let_wave && wave_source ? 1 : 0;
  for (int k = 0; k < np; ++k) {
    P.abs_node.push_back(b->node[k]);
    for (int d = 0; d < nd; ++d) P.abs_Cd[d].push_back(Cb[k + size_t(np) * d]);
    P.abs_B.push_back(w[k]);
    P.abs_n0.push_back(nrm[k]);
    P.abs_n1.push_back(nrm[k + np]);
    P.abs_wave.push_back(wave);
  }
}

// BC_DIRNEU_init (bc_dirneu.f90:117-143): a flat side whose components
// flagged 'D' have their force set to zero (bc_DIRNEU_apply, :148-169)
void dirneu_init(sem2d_problem &P, const sem2d_bc &bc, int after_fault) {
  const int tag = bc.tag[0], mask = bc.dirichlet;
  const sem2d_grid &g = *P.g;
  const sem2d_grid::Boundary *b = g.find(tag);
  if (!b) return;
  const int np = int(b->node.size());
  std::vector<double> nrm, w;
  normals(g, *b, nrm, w, perio_intersects(P, *b));
  bool horiz = true, vert = true;
  for (int k = 0; k < np; ++k) {
    horiz &= std::fabs(nrm[k]) < kTinyXabs;
    vert &= std::fabs(nrm[k + np]) < kTinyXabs;
  }
  if (!horiz && !vert) throw BuildError("BC_DIRNEU_init: boundary is not vertical or horizontal");
  for (int c = 0; c < P.ndof; ++c) {
    if (!((mask >> c) & 1)) continue;
    for (int k = 0; k < np; ++k) {
      P.dir_node.push_back(b->node[k]);
      P.dir_comp.push_back(c);
      P.dir_after.push_back(after_fault);
    }
  }
  // a Neumann component with a time function: field += STF(t) B
  // (bc_DIRNEU_apply, bc_dirneu.f90:157-167; a Dirichlet component's
  // function is dropped, :70-101; SH has only the horizontal one)
  for (int c = 0; c < P.ndof; ++c) {
    const sem2d_stf &in = c == 0 ? bc.hstf : bc.vstf;
    if (((mask >> c) & 1) || in.kind == SEM2D_STF_NONE) continue;
    const int q = int(P.neu_stfs.size());
    P.neu_stfs.push_back(read_stf(P, in));
    for (int k = 0; k < np; ++k) {
      P.neu_node.push_back(b->node[k]);
      P.neu_comp.push_back(c);
      P.neu_B.push_back(w[k]);
      P.neu_stf.push_back(q);
    }
  }
}

long nint_ref(double x) { return long(x >= 0 ? std::floor(x + 0.5) : -std::floor(-x + 0.5)); }

// BC_DYNFLT_init (bc_dynflt.f90:231-520)
void dynflt_init(sem2d_problem &P, const sem2d_deck &dk, const int *tags) {
  const sem2d_grid &g = *P.g;
  if (P.nflt) throw BuildError("only one DYNFLT boundary is supported");
  const sem2d_grid::Boundary *b1 = g.find(tags[0]);
  const sem2d_grid::Boundary *b2 = tags[1] > 0 ? g.find(tags[1]) : nullptr;
  if (!b1 || (tags[1] > 0 && !b2)) return;
  const int nd = P.ndof, nb = int(b1->node.size());
  P.two = tags[1] > 0;
  if (P.two && (b1->elem.size() != b2->elem.size() || b2->node.size() != b1->node.size()))
    throw BuildError("bc_dynflt_init: boundaries do not match");
  std::vector<double> nrm, w;
  normals(g, *b1, nrm, w, perio_intersects(P, *b1));
  for (int k = 0; k < nb; ++k) {
    if (P.two && b1->node[k] == b2->node[k]) continue;  // non-split nodes are dropped
    P.node1.push_back(b1->node[k]);
    P.node2.push_back(P.two ? b2->node[k] : 0);
    P.B.push_back(w[k]);
    P.n1.push_back(nrm[k]);
  }
  const int nf = int(P.node1.size());
  P.nflt = nf;
  {
    std::vector<double> nz;
    int q = 0;
    for (int k = 0; k < nb; ++k) {
      if (P.two && b1->node[k] == b2->node[k]) continue;
      nz.push_back(nrm[k + nb]);
      ++q;
    }
    P.n1.insert(P.n1.end(), nz.begin(), nz.end());
  }
  for (int k = 0; k < nf; ++k) {
    const double *c1 = &g.coord[2 * size_t(P.node1[k] - 1)];
    P.fcoord.push_back(c1[0]);
    P.fcoord.push_back(c1[1]);
    if (P.two) {
      const double *c2 = &g.coord[2 * size_t(P.node2[k] - 1)];
      if (std::fabs(c1[0] - c2[0]) > kTinyXabs || std::fabs(c1[1] - c2[1]) > kTinyXabs)
        throw BuildError("bc_dynflt_init: coordinates on boundaries do not match properly");
    }
  }
  P.coefA2V = coefA2V(P);
  P.coefA2D = coefA2D(P);
  P.invM1.assign(size_t(nf) * nd, 0.0);
  P.invM2.assign(size_t(nf) * nd, 0.0);
  P.Z.assign(size_t(nf) * nd, 0.0);
  for (int d = 0; d < nd; ++d)
    for (int k = 0; k < nf; ++k) {
      const size_t o = size_t(k) + size_t(nf) * d;
      P.invM1[o] = 1.0 / P.mass[size_t(P.node1[k] - 1) + size_t(g.npoin) * d];
      if (P.two) {
        P.invM2[o] = 1.0 / P.mass[size_t(P.node2[k] - 1) + size_t(g.npoin) * d];
        P.Z[o] = 1.0 / (P.coefA2V * P.B[k] * (P.invM1[o] + P.invM2[o]));
      } else {
        P.Z[o] = 0.5 / (P.coefA2V * P.B[k] * P.invM1[o]);
      }
    }
  for (int q = 0; q < SEM2D_FP_NPARAM; ++q) {
    P.prm[q].resize(nf);
    for (int k = 0; k < nf; ++k) P.prm[q][k] = dk.flt_array[q] ? dk.flt_array[q][k] : dk.flt_value[q];
  }
  P.T0.assign(2 * size_t(nf), 0.0);
  P.coh.resize(nf);
  for (int k = 0; k < nf; ++k) {
    const double nx = P.n1[k], nz = P.n1[k + nf];
    const double Sxx = P.prm[SEM2D_FP_SXX][k], Sxy = P.prm[SEM2D_FP_SXY][k];
    const double Sxz = P.prm[SEM2D_FP_SXZ][k], Syz = P.prm[SEM2D_FP_SYZ][k];
    const double Szz = P.prm[SEM2D_FP_SZZ][k];
    const double Tx = Sxx * nx + Sxz * nz, Ty = Sxy * nx + Syz * nz, Tz = Sxz * nx + Szz * nz;
    P.T0[k] = nd == 1 ? P.prm[SEM2D_FP_TT][k] + Ty : P.prm[SEM2D_FP_TT][k] + Tx * nz - Tz * nx;
    P.T0[k + nf] = P.prm[SEM2D_FP_TN][k] + Tx * nx + Tz * nz;
    P.coh[k] = P.prm[SEM2D_FP_COHESION][k];
    if (P.coh[k] < 0.0) throw BuildError("bc_dynflt_init: cohesion must be positive");
  }
  P.oix1 = std::max(dk.flt_oxi[0], 1);
  P.oixn = (dk.flt_oxi[1] > 0 && dk.flt_oxi[1] < nf) ? dk.flt_oxi[1] : nf;
  P.oixd = dk.flt_oxi[2] > 0 ? dk.flt_oxi[2] : 1;
  P.oitd = int(std::max(1L, nint_ref(dk.flt_otd / P.dt)));
  P.oit = int(nint_ref(dk.flt_ot1 / P.dt));
  P.fnsamp = (P.nt - P.oit) / P.oitd + 1;
}

// SE_find_nearest_node (spec_grid.f90:410-435): last node at the minimum
int nearest_node(const sem2d_grid &g, const double *xz) {
  double d2min = 1.7976931348623157e308;
  int ig = 0;
  for (int p = 0; p < g.npoin; ++p) {
    const double dx = xz[0] - g.coord[2 * size_t(p)], dz = xz[1] - g.coord[2 * size_t(p) + 1];
    const double d2 = dx * dx + dz * dz;
    if (d2 <= d2min) {
      d2min = d2;
      ig = p + 1;
    }
  }
  return ig;
}

// SE_find_point / FE_find_point (spec_grid.f90:471-497, fem_grid.f90:451-501):
// Newton iteration for (xi,eta) in the first element holding the nearest node
void find_point(const sem2d_grid &g, const double *xz, int &e_out, double &xi, double &eta,
                double *newc) {
  const int ig = nearest_node(g, xz), N = g.ngll;
  for (int e = 0; e < g.nelem; ++e)
    for (int j = 0; j < N; ++j)
      for (int i = 0; i < N; ++i) {
        if (g.ibool[i + N * (j + size_t(N) * e)] != ig) continue;
        double c[18];
        g.control(e, c);
        const int ng = g.ngnod;
        const double x1 = c[0] - c[4], x2 = c[1] - c[5], y1 = c[2] - c[6], y2 = c[3] - c[7];
        const double area = 0.5 * std::fabs(x1 * y2 - x2 * y1);
        const double tolf = kTinyXabs * std::sqrt(area / kPi), tolx = kTinyXabs;
        double X[2] = {g.gll.x[i], g.gll.x[j]};
        int it;
        for (it = 1; it <= 100; ++it) {
          double sh[9], J[4];
          shape(ng, X[0], X[1], sh);
          const double f0 = interp(c, ng, 0, sh) - xz[0], f1 = interp(c, ng, 1, sh) - xz[1];
          jacobian(ng, c, X[0], X[1], J);
          if (std::fabs(f0) + std::fabs(f1) <= tolf) break;
          const double det = J[0] * J[3] - J[2] * J[1];
          const double i00 = J[3] / det, i10 = -J[1] / det, i01 = -J[2] / det, i11 = J[0] / det;
          const double p0 = -f0, p1 = -f1;
          const double q0 = i00 * p0 + i01 * p1, q1 = i10 * p0 + i11 * p1;
          X[0] = X[0] + q0;
          X[1] = X[1] + q1;
          if (std::fabs(q0) + std::fabs(q1) <= tolx) break;
        }
        if (it >= 100) throw BuildError("FE_find_point: did not converge");
        e_out = e + 1;
        xi = X[0];
        eta = X[1];
        double sh[9];
        shape(ng, xi, eta, sh);
        newc[0] = interp(c, ng, 0, sh);
        newc[1] = interp(c, ng, 1, sh);
        return;
      }
  throw BuildError("SE_find_point: point not found");
}

void rec_init(sem2d_problem &P, const sem2d_deck &dk) {
  const sem2d_grid &g = *P.g;
  const int nx = dk.rec_number;
  if (nx <= 0) return;
  std::vector<double> rc(2 * size_t(nx));
  if (dk.rec_coord) {
    std::copy(dk.rec_coord, dk.rec_coord + 2 * nx, rc.begin());
  } else if (nx > 1) {
    for (int i = 0; i < nx; ++i)
      for (int a = 0; a < 2; ++a)
        rc[2 * i + a] = dk.rec_first[a] + (double(i) / double(nx - 1)) * (dk.rec_last[a] - dk.rec_first[a]);
  } else {
    rc[0] = dk.rec_first[0];
    rc[1] = dk.rec_first[1];
  }
  P.rec_isamp = dk.rec_isamp > 0 ? dk.rec_isamp : 1;
  P.rec_field = dk.rec_field ? dk.rec_field : 'V';
  if (P.rec_field != 'D' && P.rec_field != 'V' && P.rec_field != 'A')
    throw BuildError("REC_read: parameter field has wrong value [D,V,A]");
  const int n2 = g.ngll * g.ngll;
  if (dk.rec_atnode) {
    for (int k = 0; k < nx; ++k) {
      const int ip = nearest_node(g, &rc[2 * k]);
      // receivers.f90:255 only de-duplicates from the third kept receiver on
      if (P.rec_node.size() > 1 && std::find(P.rec_node.begin(), P.rec_node.end(), ip) != P.rec_node.end())
        continue;
      P.rec_node.push_back(ip);
    }
    P.nrec = int(P.rec_node.size());
    for (int ip : P.rec_node) {
      P.rec_coord.push_back(g.coord[2 * size_t(ip - 1)]);
      P.rec_coord.push_back(g.coord[2 * size_t(ip - 1) + 1]);
    }
  } else {
    P.nrec = nx;
    for (int k = 0; k < nx; ++k) {
      int e;
      double xi, eta, nc[2];
      find_point(g, &rc[2 * k], e, xi, eta, nc);
      P.rec_elem.push_back(e);
      for (int j = 0; j < g.ngll; ++j) {
        const double fj = lagrange(j, eta, g.gll);
        for (int i = 0; i < g.ngll; ++i) P.rec_interp.push_back(lagrange(i, xi, g.gll) * fj);
      }
      P.rec_coord.push_back(nc[0]);
      P.rec_coord.push_back(nc[1]);
    }
    (void)n2;
  }
  P.rec_nsamp = P.nt / P.rec_isamp + 1;
}

// WAVE_read + WAVE_init (src_wave.f90:78-180) for the first wave source,
// the one every absorbing side with let_wave takes (bc_abso.f90:245-256).
// The reference point: the domain corner the wave enters first (maximum x
// for angle >= 0, minimum z for |angle| < 90), moved to its nearest node;
// the material values are those of the first element point at that node.
// WAVE_init computes that corner but then searches from wave%coord, which
// it never assigns, and leaves wave%coord unset for the phase
// (src_wave.f90:133-157, 183-187); the corner is the reading its comments
// and the input documentation give, and the C-ABI takes the point
// explicitly (wave_ref) for a caller who wants another.
void wave_init(sem2d_problem &P, const sem2d_deck &dk, const sem2d_stf &stf) {
  const sem2d_grid &g = *P.g;
  double angle = dk.wave_angle + 180.0;
  angle = angle - std::floor(angle / 360.0) * 360.0 - 180.0;  // modulo(angle+180,360)-180
  if (dk.wave_phase != SEM2D_WAVE_P && dk.wave_phase != SEM2D_WAVE_S)
    throw BuildError("WAVE_read: phase must be S or P");
  double xmin = g.coord[0], xmax = g.coord[0], zmin = g.coord[1], zmax = g.coord[1];
  for (int p = 0; p < g.npoin; ++p) {
    xmin = std::min(xmin, g.coord[2 * size_t(p)]);
    xmax = std::max(xmax, g.coord[2 * size_t(p)]);
    zmin = std::min(zmin, g.coord[2 * size_t(p) + 1]);
    zmax = std::max(zmax, g.coord[2 * size_t(p) + 1]);
  }
  const double corner[2] = {angle >= 0.0 ? xmax : xmin, std::fabs(angle) < 90.0 ? zmin : zmax};
  const int ig = nearest_node(g, corner);
  const int N = g.ngll;
  size_t at = 0;
  bool found = false;
  for (int e = 0; e < g.nelem && !found; ++e)  // SE_node_belongs_to_1, spec_grid.f90:441-456
    for (int j = 0; j < N && !found; ++j)
      for (int i = 0; i < N && !found; ++i)
        if (g.ibool[i + N * (j + size_t(N) * e)] == ig) {
          at = i + N * (j + size_t(N) * e);
          found = true;
        }
  const sem2d_material *m = find_mat(dk, g.tag[at / (size_t(N) * N)]);
  if (m && m->aniso) throw BuildError("MAT_getProp: the incident wave needs mu and lambda of an isotropic material");
  P.wave_phase = dk.wave_phase;
  P.wave_angle = angle;
  P.wave_ref[0] = g.coord[2 * size_t(ig - 1)];
  P.wave_ref[1] = g.coord[2 * size_t(ig - 1) + 1];
  const double rho = P.rho[at], cp = P.cp[at], cs = P.cs[at];
  P.wave_cp = cp;
  P.wave_cs = cs;
  P.wave_mu = rho * cs * cs;                      // mat_elastic.f90:214-215
  P.wave_lambda = rho * (cp * cp - 2.0 * cs * cs);
  P.wave_tdelay = dk.src_tdelay ? dk.src_tdelay[0] : 0.0;
  P.wave_stf = stf;
}

void src_init(sem2d_problem &P, const sem2d_deck &dk) {
  const int ns = dk.nsrc;
  if (ns <= 0) return;
  // the time function all sources share (SO_read, src_gen.f90:150-158)
  sem2d_stf in = dk.stf;
  if (in.kind == SEM2D_STF_NONE) {
    in.kind = SEM2D_STF_RICKER;
    in.f0 = dk.ricker_f0;
    in.onset = dk.ricker_onset;
    in.ampli = dk.ricker_ampli;
  }
  const sem2d_stf stf = read_stf(P, in);
  if (dk.src_mech == 4) {
    wave_init(P, dk, stf);
    return;
  }
  if (stf.kind != SEM2D_STF_RICKER) {
    P.has_src_stf = true;
    P.src_stf = stf;
  }
  const double ang = dk.force_angle * kPi / 180.0;
  auto push = [&](int node, double dx, double dz, double rel, double td) {
    P.src_node.push_back(node);
    P.src_dir.push_back(dx);
    P.src_dir.push_back(dz);
    P.src_f0.push_back(stf.f0);
    P.src_t0.push_back(stf.onset);
    P.src_amp.push_back(stf.ampli);
    P.src_rel.push_back(rel);
    P.src_tdelay.push_back(td);
  };
  if (dk.src_mech == 0) {
    for (int k = 0; k < ns; ++k)
      push(nearest_node(*P.g, dk.src_coord + 2 * k), -std::sin(ang), std::cos(ang),
           dk.src_ampli ? dk.src_ampli[k] : 1.0, dk.src_tdelay ? dk.src_tdelay[k] : 0.0);
    return;
  }
  // SRC_MOMENT_read (src_moment.f90:27-110): the tensor M(2,ndof)
  const int nd = P.ndof;
  double M[2][2] = {{0, 0}, {0, 0}};
  if (dk.src_mech == 1) {
    if (nd != 2) throw BuildError("SRC_MOMENT_read: explosion only allowed in PSV (ndof=2)");
    M[0][0] = 1.0;
    M[1][1] = 1.0;
  } else if (dk.src_mech == 2) {
    const double dip = dk.src_dip * kPi / 180.0, n0 = std::sin(dip), n1 = std::cos(dip);
    if (nd == 2) {
      const double r0 = -std::cos(dip), r1 = std::sin(dip);
      M[0][0] = 2.0 * r0 * n0;
      M[0][1] = r0 * n1 + r1 * n0;
      M[1][0] = M[0][1];
      M[1][1] = 2.0 * r1 * n1;
    } else {
      M[0][0] = n0;
      M[1][0] = n1;
    }
  } else if (dk.src_mech == 3) {
    if (nd == 2) {
      M[0][0] = dk.src_M[0];
      M[0][1] = dk.src_M[1];
      M[1][0] = dk.src_M[2];
      M[1][1] = dk.src_M[3];
    } else {
      M[0][0] = dk.src_M[0];
      M[1][0] = dk.src_M[1];
    }
  } else {
    throw BuildError("unknown source mechanism");
  }
  // SRC_MOMENT_init / SRC_MOMENT_add (src_moment.f90:118-175): in every
  // element holding the source node (i, j), the row of nodes (:, j) gets
  // G(c,1) h'_l(xi_i) and the column (i, :) G(c,2) h'_l(eta_j), with
  // G = M jac_inv^T (SH: G = jac_inv M(:,1)); here the coefficients are
  // summed per node into point forces of the same time function
  const sem2d_grid &g = *P.g;
  const int N = g.ngll;
  for (int k = 0; k < ns; ++k) {
    const int node = nearest_node(g, dk.src_coord + 2 * k);
    const double rel = dk.src_ampli ? dk.src_ampli[k] : 1.0, td = dk.src_tdelay ? dk.src_tdelay[k] : 0.0;
    std::vector<int> nodes;
    std::vector<double> F;  // 2 per node
    auto add = [&](int n, double fx, double fz) {
      for (size_t q = 0; q < nodes.size(); ++q)
        if (nodes[q] == n) {
          F[2 * q] += fx;
          F[2 * q + 1] += fz;
          return;
        }
      nodes.push_back(n);
      F.push_back(fx);
      F.push_back(fz);
    };
    for (int e = 0; e < g.nelem; ++e)
      for (int j = 0; j < N; ++j)
        for (int i = 0; i < N; ++i) {
          if (g.ibool[i + N * (j + size_t(N) * e)] != node) continue;
          double c8[18], J[4];
          g.control(e, c8);
          jacobian(g.ngnod, c8, g.gll.x[i], g.gll.x[j], J);
          const double det = J[0] * J[3] - J[2] * J[1];
          const double inv[2][2] = {{J[3] / det, -J[2] / det}, {-J[1] / det, J[0] / det}};  // d(xi,eta)/d(x,z)
          double G[2][2];
          if (nd == 2) {
            for (int a = 0; a < 2; ++a)
              for (int b = 0; b < 2; ++b) G[a][b] = M[a][0] * inv[b][0] + M[a][1] * inv[b][1];
          } else {
            G[0][0] = inv[0][0] * M[0][0] + inv[0][1] * M[1][0];
            G[0][1] = inv[1][0] * M[0][0] + inv[1][1] * M[1][0];
            G[1][0] = G[1][1] = 0.0;
          }
          for (int l = 0; l < N; ++l) {
            const double hx = g.gll.H[l + N * i], he = g.gll.H[l + N * j];
            add(g.ibool[l + N * (j + size_t(N) * e)], G[0][0] * hx, G[1][0] * hx);
            add(g.ibool[i + N * (l + size_t(N) * e)], G[0][1] * he, G[1][1] * he);
          }
        }
    for (size_t q = 0; q < nodes.size(); ++q) {
      if (nd == 2)
        push(nodes[q], F[2 * q], F[2 * q + 1], rel, td);
      else  // SH: the force is the amplitude itself
        push(nodes[q], 1.0, 0.0, rel * F[2 * q], td);
    }
  }
}

int fail(const std::exception &e) {
  g_err = e.what();
  return SEM2D_E_ARG;
}

}  // namespace

// ----------------------------------------------------------------------
extern "C" {

int sem2d_grid_build(const sem2d_deck *deck, sem2d_grid **out) {
  if (!deck || !out) return g_err = "null argument", SEM2D_E_ARG;
  try {
    auto g = std::make_unique<sem2d_grid>();
    build_grid(*g, *deck);
    *out = g.release();
    return SEM2D_OK;
  } catch (const std::bad_alloc &) {
    g_err = "out of host memory";
    return SEM2D_E_NOMEM;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

int sem2d_grid_sizes(const sem2d_grid *g, int *nelem, int *npoin, int *ngll) {
  if (!g) return SEM2D_E_ARG;
  if (nelem) *nelem = g->nelem;
  if (npoin) *npoin = g->npoin;
  if (ngll) *ngll = g->ngll;
  return SEM2D_OK;
}

int sem2d_grid_ibool(const sem2d_grid *g, int *ibool) {
  if (!g || !ibool) return SEM2D_E_ARG;
  std::copy(g->ibool.begin(), g->ibool.end(), ibool);
  return SEM2D_OK;
}

int sem2d_grid_coord(const sem2d_grid *g, double *coord) {
  if (!g || !coord) return SEM2D_E_ARG;
  std::copy(g->coord.begin(), g->coord.end(), coord);
  return SEM2D_OK;
}

int sem2d_grid_tags(const sem2d_grid *g, int *tag) {
  if (!g || !tag) return SEM2D_E_ARG;
  std::copy(g->tag.begin(), g->tag.end(), tag);
  return SEM2D_OK;
}

int sem2d_grid_boundary(const sem2d_grid *g, int tag, int *npoin, int *nodes) {
  if (!g || !npoin) return SEM2D_E_ARG;
  const sem2d_grid::Boundary *b = g->find(tag);
  *npoin = b ? int(b->node.size()) : 0;
  if (b && nodes) std::copy(b->node.begin(), b->node.end(), nodes);
  return SEM2D_OK;
}

int sem2d_grid_gll(const sem2d_grid *g, double *x, double *w, double *H) {
  if (!g) return SEM2D_E_ARG;
  if (x) std::copy(g->gll.x.begin(), g->gll.x.end(), x);
  if (w) std::copy(g->gll.w.begin(), g->gll.w.end(), w);
  if (H) std::copy(g->gll.H.begin(), g->gll.H.end(), H);
  return SEM2D_OK;
}

void sem2d_grid_destroy(sem2d_grid *g) { delete g; }

int sem2d_problem_build(const sem2d_grid *g, const sem2d_deck *deck, sem2d_problem **out) {
  if (!g || !deck || !out) return g_err = "null argument", SEM2D_E_ARG;
  try {
    auto P = std::make_unique<sem2d_problem>();
    P->g = g;
    P->deck = *deck;
    P->ndof = g->ndof;
    if (deck->ndof != g->ndof || deck->ngll != g->ngll) throw BuildError("deck does not match the grid");
    build_materials(*P, *deck);
    build_time(*P, *deck);
    if (P->has_kv) {
      const size_t n2 = size_t(g->ngll) * g->ngll;
      for (int e = 0; e < g->nelem; ++e) {
        const sem2d_material *m = find_mat(*deck, g->tag[e]);
        if (m->kv && m->kv_etaxdt)
          for (size_t q = 0; q < n2; ++q) P->kveta[q + n2 * e] = P->dt * P->kveta[q + n2 * e];
      }
    }
    build_mass(*P);
    if (!g->flat) build_general_geometry(*P);
    // periodic sides first (bc_gen.f90:221-228)
    for (int b = 0; b < deck->nbcs; ++b)
      if (deck->bcs[b].kind == SEM2D_BC_PERIOD) {
        if (!P->per_master.empty()) throw BuildError("more than one pair of periodic sides");
        perio_init(*P, deck->bcs[b].tag);
      }
    bool fault_seen = false;
    for (int b = 0; b < deck->nbcs; ++b) {
      const sem2d_bc &bc = deck->bcs[b];
      if (bc.kind == SEM2D_BC_ABSORB) {
        abso_init(*P, bc.tag[0], bc.stacey, !bc.no_wave, deck->nsrc > 0 && deck->src_mech == 4);
      } else if (bc.kind == SEM2D_BC_DYNFLT) {
        dynflt_init(*P, *deck, bc.tag);
        fault_seen = true;
      } else if (bc.kind == SEM2D_BC_DIRNEU) {
        dirneu_init(*P, bc, fault_seen ? 1 : 0);
      } else if (bc.kind == SEM2D_BC_PERIOD) {
        continue;
      } else {
        throw BuildError("unsupported boundary condition kind");
      }
    }
    rec_init(*P, *deck);
    src_init(*P, *deck);
    for (double &m : P->mass) m = 1.0 / m;  // init.f90:112-116
    const int nd = P->ndof;
    const size_t na = P->abs_node.size();
    P->abs_C.resize(na * nd);
    for (int d = 0; d < nd && na; ++d)
      for (size_t k = 0; k < na; ++k) P->abs_C[k + na * d] = P->abs_Cd[d][k];
    P->abs_n = P->abs_n0;
    P->abs_n.insert(P->abs_n.end(), P->abs_n1.begin(), P->abs_n1.end());  // n(nabs, 2)
    P->st_K0.insert(P->st_K0.end(), P->st_K1.begin(), P->st_K1.end());  // K(nstacey, 2)
    *out = P.release();
    return SEM2D_OK;
  } catch (const std::bad_alloc &) {
    g_err = "out of host memory";
    return SEM2D_E_NOMEM;
  } catch (const std::exception &e) {
    return fail(e);
  }
}

#define VPTR(v) ((v).empty() ? nullptr : (v).data())

int sem2d_problem_get_desc(const sem2d_problem *P, sem2d_problem_desc *d) {
  if (!P || !d) return SEM2D_E_ARG;
  const sem2d_grid &g = *P->g;
  std::memset(d, 0, sizeof(*d));
  d->ngll = g.ngll;
  d->ndof = P->ndof;
  d->nelem = g.nelem;
  d->npoin = g.npoin;
  d->ibool = g.ibool.data();
  d->coord = g.coord.data();
  d->hprime = g.gll.H.data();
  d->wgll = g.gll.w.data();
  d->Kx = P->Kx.data();
  d->Kz = P->Kz.data();
  d->la = P->la.data();
  d->mu = P->mu.data();
  d->mux = P->mux.data();
  d->kv_eta = P->has_kv ? P->kveta.data() : nullptr;
  d->kd2_form = P->deck.kd2_form >= 0 ? P->deck.kd2_form : (g.ngll == 5);
  d->rmass = P->mass.data();
  d->nabs = int(P->abs_node.size());
  d->abs_node = VPTR(P->abs_node);
  d->abs_C = VPTR(P->abs_C);
  d->nstacey = int(P->st_node.size());
  d->stacey_node = VPTR(P->st_node);
  d->stacey_k = VPTR(P->st_k);
  d->stacey_edge = VPTR(P->st_edge);
  d->stacey_K = VPTR(P->st_K0);
  d->ndir = int(P->dir_node.size());
  d->dir_node = VPTR(P->dir_node);
  d->dir_comp = VPTR(P->dir_comp);
  d->dir_after_fault = VPTR(P->dir_after);
  d->nperio = int(P->per_master.size());
  d->perio_master = VPTR(P->per_master);
  d->perio_slave = VPTR(P->per_slave);
  d->time_scheme = P->time_kind;
  d->dt = P->dt;
  d->beta = P->beta;
  d->gamma = P->gamma;
  d->alpha = P->alpha;
  d->nt = P->nt;
  d->nsrc = int(P->src_node.size());
  d->src_node = VPTR(P->src_node);
  d->src_dir = VPTR(P->src_dir);
  d->src_f0 = VPTR(P->src_f0);
  d->src_t0 = VPTR(P->src_t0);
  d->src_ampli = VPTR(P->src_amp);
  d->src_relamp = VPTR(P->src_rel);
  d->src_tdelay = VPTR(P->src_tdelay);
  d->nrec = P->nrec;
  d->rec_field = P->rec_field;
  d->rec_isamp = P->rec_isamp;
  d->rec_nsamp = P->rec_nsamp;
  d->rec_node = VPTR(P->rec_node);
  d->rec_elem = VPTR(P->rec_elem);
  d->rec_interp = VPTR(P->rec_interp);
  d->nflt = P->nflt;
  if (P->nflt) {
    const sem2d_deck &dk = P->deck;
    d->flt_node1 = P->node1.data();
    d->flt_node2 = P->two ? P->node2.data() : nullptr;
    d->flt_n1 = P->n1.data();
    d->flt_B = P->B.data();
    d->flt_invM1 = P->invM1.data();
    d->flt_invM2 = P->two ? P->invM2.data() : nullptr;
    d->flt_Z = P->Z.data();
    d->flt_T0 = P->T0.data();
    d->flt_cohesion = P->coh.data();
    d->flt_coefA2V = P->coefA2V;
    d->flt_coefA2D = P->coefA2D;
    d->flt_opening = dk.flt_opening;
    d->flt_friction = dk.flt_friction;
    d->swf_kind = dk.swf_kind;
    d->swf_healing = dk.swf_healing;
    d->swf_dc = P->prm[SEM2D_FP_SWF_DC].data();
    d->swf_mus = P->prm[SEM2D_FP_SWF_MUS].data();
    d->swf_mud = P->prm[SEM2D_FP_SWF_MUD].data();
    d->swf_p = P->prm[SEM2D_FP_SWF_P].data();
    d->swf_alpha = P->prm[SEM2D_FP_SWF_ALPHA].data();
    d->rsf_kind = dk.rsf_kind;
    d->rsf_dc = P->prm[SEM2D_FP_RSF_DC].data();
    d->rsf_mus = P->prm[SEM2D_FP_RSF_MUS].data();
    d->rsf_a = P->prm[SEM2D_FP_RSF_A].data();
    d->rsf_b = P->prm[SEM2D_FP_RSF_B].data();
    d->rsf_vstar = P->prm[SEM2D_FP_RSF_VSTAR].data();
    d->rsf_vc = P->prm[SEM2D_FP_RSF_VC].data();
    d->rsf_theta = P->prm[SEM2D_FP_RSF_THETA].data();
    d->flt_V0 = P->prm[SEM2D_FP_V0].data();
    d->normal_kind = dk.normal_kind;
    d->normal_T = dk.normal_T;
    d->normal_L = dk.normal_L;
    d->normal_V = dk.normal_V;
    d->flt_oit = P->oit;
    d->flt_oitd = P->oitd;
    d->flt_oix1 = P->oix1;
    d->flt_oixn = P->oixn;
    d->flt_oixd = P->oixd;
    d->flt_nsamp = P->fnsamp;
  }
  d->precision = P->deck.precision;
  d->width = P->deck.width;
  d->rho = P->rho.data();
  if (P->nflt) {
    const sem2d_deck &dk = P->deck;
    d->twf_kind = dk.flt_friction == SEM2D_FRICTION_TWF && dk.twf_kind == 0 ? 1 : dk.twf_kind;
    d->twf_mus = dk.twf_mus;
    d->twf_mud = dk.twf_mud;
    d->twf_mu0 = dk.twf_mu0;
    d->twf_X = dk.twf_X;
    d->twf_Z = dk.twf_Z;
    d->twf_V = dk.twf_V;
    d->twf_L = dk.twf_L;
    d->twf_T = dk.twf_T;
    d->twf_Dc = dk.twf_Dc;
    d->flt_potency = dk.flt_potency;
  }
  d->src_stf = P->has_src_stf ? &P->src_stf : nullptr;
  d->wave_phase = P->wave_phase;
  if (P->wave_phase) {
    d->wave_angle = P->wave_angle;
    d->wave_ref[0] = P->wave_ref[0];
    d->wave_ref[1] = P->wave_ref[1];
    d->wave_cp = P->wave_cp;
    d->wave_cs = P->wave_cs;
    d->wave_mu = P->wave_mu;
    d->wave_lambda = P->wave_lambda;
    d->wave_tdelay = P->wave_tdelay;
    d->wave_stf = &P->wave_stf;
  }
  d->abs_B = VPTR(P->abs_B);
  d->abs_n = VPTR(P->abs_n);
  d->abs_wave = P->wave_phase ? VPTR(P->abs_wave) : nullptr;
  d->nneu = int(P->neu_node.size());
  d->neu_node = VPTR(P->neu_node);
  d->neu_comp = VPTR(P->neu_comp);
  d->neu_B = VPTR(P->neu_B);
  d->neu_stf = VPTR(P->neu_stf);
  d->nneu_stf = int(P->neu_stfs.size());
  d->neu_stfs = VPTR(P->neu_stfs);
  d->xjaci = VPTR(P->xjaci);
  d->dvol = VPTR(P->dvol);
  return SEM2D_OK;
}

int sem2d_problem_time(const sem2d_problem *P, double *dt, int *nt, double *courant) {
  if (!P) return SEM2D_E_ARG;
  if (dt) *dt = P->dt;
  if (nt) *nt = P->nt;
  if (courant) *courant = P->courant;
  return SEM2D_OK;
}

int sem2d_problem_rec_coord(const sem2d_problem *P, double *coord) {
  if (!P) return SEM2D_E_ARG;
  if (coord) std::copy(P->rec_coord.begin(), P->rec_coord.end(), coord);
  return P->nrec;
}

int sem2d_problem_fault_coord(const sem2d_problem *P, double *coord) {
  if (!P) return SEM2D_E_ARG;
  if (coord) std::copy(P->fcoord.begin(), P->fcoord.end(), coord);
  return P->nflt;
}

void sem2d_problem_destroy(sem2d_problem *P) { delete P; }

const char *sem2d_host_last_error(void) { return g_err.c_str(); }

int sem2d_abi_struct_sizes(int *desc_size, int *deck_size) {
  if (desc_size) *desc_size = int(sizeof(sem2d_problem_desc));
  if (deck_size) *deck_size = int(sizeof(sem2d_deck));
  return SEM2D_OK;
}

}  // extern "C"

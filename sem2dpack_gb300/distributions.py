"""Spatial distributions of the reference's input (&DIST_* blocks), evaluated
on the host at the points where the reference evaluates them: the fault
nodes for fault parameters (BC_DYNFLT_init, bc_dynflt.f90:302,373-416) and
the element GLL points for material properties (MAT_setProp).

  PWCONR    piecewise constant on rings around ref (distribution_pwconr.f90)
  GAUSSIAN  offset + ampli exp(-(((x-x0)/lx)^2 + ((z-z0)/lz)^2)^order)
            (distribution_gaussian.f90)
  ORDER0    piecewise constant on a rectangular x-z zoning
            (distribution_order0.f90:55-109)
  LINEAR    linear interpolation along x (dim=1) or z (dim=2) of a table,
            with end segments extended, optionally averaged over a window
            of width `length` (distribution_linear.f90:60-188)
  GRADIENT  valref + grad (yref - y) in a frame rotated by `angle`, yref
            interpolated from a reference line (distribution_gradient.f90)
  SPLINE    cubic spline with zero end slopes through a table sorted by x,
            along x (dim=1) or z (dim=2) (distribution_spline.f90:34-109,
            spline and splint utils.f90:652-734); a point outside the table
            is refused (the reference reads outside its arrays there)

HETE1 is refused.  Tables given by `file=` are read relative to
the folder of the Par.inp.
"""
import os

import numpy as np

__all__ = ["Dist", "KINDS"]

KINDS = ("PWCONR", "GAUSSIAN", "ORDER0", "LINEAR", "GRADIENT", "SPLINE")


def _spline_d2(x, y):
    """spline (utils.f90:652-691) with yp1 = ypn = 0: the second
    derivatives, in the reference's order of operations."""
    n = len(x)
    y2, u = [0.0] * n, [0.0] * n
    y2[0] = -0.5
    u[0] = (3.0 / (x[1] - x[0])) * ((y[1] - y[0]) / (x[1] - x[0]) - 0.0)
    for i in range(1, n - 1):
        sig = (x[i] - x[i - 1]) / (x[i + 1] - x[i - 1])
        p = sig * y2[i - 1] + 2.0
        y2[i] = (sig - 1.0) / p
        u[i] = (6.0 * ((y[i + 1] - y[i]) / (x[i + 1] - x[i]) - (y[i] - y[i - 1]) / (x[i] - x[i - 1]))
                / (x[i + 1] - x[i - 1]) - sig * u[i - 1]) / p
    qn, un = 0.5, (3.0 / (x[n - 1] - x[n - 2])) * (0.0 - (y[n - 1] - y[n - 2]) / (x[n - 1] - x[n - 2]))
    y2[n - 1] = (un - qn * u[n - 2]) / (qn * y2[n - 2] + 1.0)
    for k in range(n - 2, -1, -1):
        y2[k] = y2[k] * y2[k + 1] + u[k]
    return y2


def _splint(xa, ya, y2, x):
    """splint (utils.f90:697-734) at each x: the bracket [klo, klo+1] with
    xa[klo] < x <= xa[klo+1] (hunt's bisection, utils.f90:596-646)."""
    out = []
    n = len(xa)
    for v in x:
        lo, hi = 0, n - 1
        while hi - lo > 1:
            m = (lo + hi) // 2
            if v > xa[m]:
                lo = m
            else:
                hi = m
        h = xa[hi] - xa[lo]
        a, b = (xa[hi] - v) / h, (v - xa[lo]) / h
        out.append(a * ya[lo] + b * ya[hi] + ((a ** 3 - a) * y2[lo] + (b ** 3 - b) * y2[hi]) * (h * h) / 6.0)
    return np.array(out)


def _interpol(xi, yi, xo):
    """interpol (distribution_linear.f90:118-139): the segment of the table
    that brackets each point (hunt, utils.f90:596-646), the first or last
    segment outside the table."""
    xi, yi, xo = np.asarray(xi, float), np.asarray(yi, float), np.asarray(xo, float)
    n = len(xi)
    ipos = np.clip(np.searchsorted(xi, xo, side="right"), 1, n - 1) - 1
    eta = (xo - xi[ipos]) / (xi[ipos + 1] - xi[ipos])
    return yi[ipos] + eta * (yi[ipos + 1] - yi[ipos])


def _smooth_interpol(xi, yi, xo, length):
    """smooth_interpol (distribution_linear.f90:145-188): the trapezoid
    average of the interpolant over [x - length/2, x + length/2]."""
    xi, yi = np.asarray(xi, float), np.asarray(yi, float)
    n = len(xi)
    out = np.empty(len(xo))
    for q, x in enumerate(np.asarray(xo, float)):
        x0, xn = x - length / 2.0, x + length / 2.0
        i0 = int(np.clip(np.searchsorted(xi, x0, side="right"), 1, n - 1))
        iN = int(np.clip(np.searchsorted(xi, xn, side="right"), 1, n - 1))
        sx = np.concatenate([[x0], xi[i0:iN], [xn]])
        sy = np.concatenate([[_interpol(xi, yi, [x0])[0]], yi[i0:iN], [_interpol(xi, yi, [xn])[0]]])
        out[q] = 0.5 * np.sum((sy[:-1] + sy[1:]) * (sx[1:] - sx[:-1])) / length
    return out


def _zone(c, n, bounds):
    """zone (distribution_order0.f90:93-109), 0-based."""
    if n == 1:
        return np.zeros(len(c), dtype=int)
    return np.minimum(np.searchsorted(np.asarray(bounds, float), c, side="right"), n - 1)


def _table(path):
    a = np.loadtxt(path, ndmin=2)
    return a[:, 0], a[:, 1]


class Dist:
    """One &DIST_<kind> block with the data that follows it."""

    def __init__(self, kind, items, data, base=None):
        self.kind = kind.upper()
        if self.kind not in KINDS:
            raise ValueError("&DIST_%s is not supported by the front end" % self.kind)
        self.items, self.data = dict(items), [float(v) for v in data if not isinstance(v, str)]
        self.base = base or "."
        it, d = self.items, self.data
        if self.kind == "PWCONR":
            num = int(it["num"])
            if num < 2:
                raise ValueError("DIST_PWCONR needs num >= 2")
            if len(d) < 2 * num - 1:
                raise ValueError("DIST_PWCONR: %d radii and %d values expected" % (num - 1, num))
            ref = it.get("ref", [0.0, 0.0])
            self.ref = (float(ref[0]), float(ref[1]))
            self.rad, self.val = np.array(d[:num - 1]), np.array(d[num - 1:2 * num - 1])
        elif self.kind == "GAUSSIAN":
            c = it.get("centered_at", [0.0, 0.0])
            ln = it.get("length", [1.0, 1.0])
            self.x0, self.z0 = float(c[0]), float(c[1])
            self.lx, self.lz = float(ln[0]), float(ln[1])
            self.offset, self.ampli = float(it.get("offset", 0.0)), float(it.get("ampli", 1.0))
            self.order = int(it.get("order", 1))
        elif self.kind == "ORDER0":
            xn, zn = int(it["xn"]), int(it["zn"])
            nb = (xn - 1) + (zn - 1)
            if len(d) < nb + xn * zn:
                raise ValueError("DIST_ORDER0: %d bounds and %d values expected" % (nb, xn * zn))
            self.xn, self.zn = xn, zn
            self.xb, self.zb = d[:xn - 1], d[xn - 1:nb]
            self.val = np.array(d[nb:nb + xn * zn]).reshape(zn, xn)  # row i: zone i in z
        elif self.kind == "LINEAR":
            self.length = float(it.get("length", 0.0))
            self.dim = int(it.get("dim", 1))
            if self.dim not in (1, 2):
                raise ValueError("DIST_LINEAR: dim must be 1 or 2")
            f = str(it.get("file", "")).strip()
            if f:
                self.x, self.y = _table(os.path.join(self.base, f))
            else:
                n = int(it.get("n", 0))
                if len(d) < 2 * n:
                    raise ValueError("DIST_LINEAR: %d (x, value) pairs expected" % n)
                self.x, self.y = np.array(d[0:2 * n:2]), np.array(d[1:2 * n:2])
        elif self.kind == "SPLINE":
            self.dim = int(it.get("dim", 1))
            if self.dim not in (1, 2):
                raise ValueError("read_spline_dist: dim must be 1 or 2")
            xs, ys = _table(os.path.join(self.base, str(it["file"]).strip()))
            order = np.argsort(xs, kind="stable")  # dsort (utils.f90)
            self.x, self.y = [float(v) for v in xs[order]], [float(v) for v in ys[order]]
            self.y2 = _spline_d2(self.x, self.y)
        else:  # GRADIENT
            self.grad = abs(float(it["grad"]))
            self.angle = float(it.get("angle", 0.0)) * 3.141592653589793 / 180.0
            self.valref = float(it["valref"])
            xr, yr = _table(os.path.join(self.base, str(it["file"]).strip()))
            ca, sa = np.cos(self.angle), np.sin(self.angle)
            x, y = ca * xr + sa * yr, -sa * xr + ca * yr
            order = np.argsort(x, kind="stable")
            self.x, self.y = x[order], y[order]

    def __call__(self, x, z):
        """Values at the points (x, z)."""
        x, z = np.asarray(x, float), np.asarray(z, float)
        if self.kind == "PWCONR":
            rad = np.sqrt((x - self.ref[0]) ** 2 + (z - self.ref[1]) ** 2)
            zone = np.full(len(rad), len(self.rad), dtype=int)
            for i in range(len(self.rad) - 1, -1, -1):
                zone[rad <= self.rad[i]] = i
            return self.val[zone]
        if self.kind == "GAUSSIAN":
            r = ((x - self.x0) / self.lx) ** 2 + ((z - self.z0) / self.lz) ** 2
            return self.offset + self.ampli * np.exp(-r ** self.order)
        if self.kind == "ORDER0":
            return self.val[_zone(z, self.zn, self.zb), _zone(x, self.xn, self.xb)]
        if self.kind == "LINEAR":
            c = x if self.dim == 1 else z
            if self.length > 0:
                return _smooth_interpol(self.x, self.y, c, self.length)
            return _interpol(self.x, self.y, c)
        if self.kind == "SPLINE":
            c = np.atleast_1d(x if self.dim == 1 else z)
            if c.min() < self.x[0] or c.max() > self.x[-1]:
                raise ValueError("DIST_SPLINE: a point lies outside the table")
            return _splint(self.x, self.y, self.y2, c)
        ca, sa = np.cos(self.angle), np.sin(self.angle)
        xr, yr = ca * x + sa * z, -sa * x + ca * z
        if xr.min() < self.x[0] or xr.max() > self.x[-1]:
            raise ValueError("DIST_GRADIENT: reference line is too short for this angle")
        return self.valref + self.grad * (_interpol(self.x, self.y, xr) - yr)

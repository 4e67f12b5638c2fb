"""FP64 autograd-through-time reference of the leapfrog step -- ORACLE,
test infrastructure only (tests import it; the product never does).

A differentiable restatement, in PyTorch FP64, of the explicit time step of
SEM2DPACK on a structured Cartesian mesh (uniform rectangular elements, no
fault), with the elastic moduli, the mass and the absorbing dashpots all
built from per-node density and wave speeds, so that autograd gives the
gradient of a seismogram misfit with respect to (rho, vp, vs) at every GLL
node.  It follows the same routines as the C oracle:

  moduli        MAT_ELAST_init (mat_elastic.f90:189-321): mu = rho vs^2,
                lambda = rho (vp^2 - 2 vs^2)
  element force ELAST_KD1/KD2 (mat_elastic.f90:464-775) with the
                a-coefficients of MAT_ELAST_init_a (mat_elastic.f90:290-360)
  mass          MAT_MASS_init (mat_mass.f90:29-61), inverted after the
                absorbing fold (init.f90:112-116, bc_abso.f90:243)
  dashpots      BC_ABSO_init / BC_ABSO_apply for flat sides
                (bc_abso.f90:195-207, 286-319)
  sources       SO_add with a Ricker force (src_gen.f90:290-317)
  time step     solve_leapfrog (solver.f90:140-161)
  receivers     REC_store at nodes (receivers.f90:309-344)

Fields live on the lattice as tensors (ndof, LZ, LX); element views are
taken with unfold and assembled with fold (overlapping windows sum).
"""
import numpy as np
import torch
import torch.nn.functional as F

from oracle.pyoracle import gll


class Lattice:
    """Geometry of an nx x nz mesh of hx x hz elements with NGLL = n."""

    def __init__(self, nx, nz, hx, hz, n=5, ndof=2, kd2=None):
        self.nx, self.nz, self.hx, self.hz, self.n, self.ndof = nx, nz, hx, hz, n, ndof
        self.LX, self.LZ = nx * (n - 1) + 1, nz * (n - 1) + 1
        x, w, H = gll(n)
        self.xg = torch.tensor(x, dtype=torch.float64)
        self.wg = torch.tensor(w, dtype=torch.float64)
        # H[i, j] = h'_i(x_j)
        self.H = torch.tensor(np.asarray(H).reshape(n, n, order="F"), dtype=torch.float64)
        self.kd2 = (n == 5) if kd2 is None else bool(kd2)
        self.xix, self.etaz = 2.0 / hx, 2.0 / hz
        self.det = (hx / 2.0) * (hz / 2.0)
        # W[j, i] = det * (w_i * w_j)   (SE_VolumeWeights, spec_grid.f90:590-602)
        self.W = self.det * (self.wg[None, :] * self.wg[:, None])

    # element views [c, ez, ex, j, i] of a lattice field [c, J, I]
    def elems(self, u):
        n = self.n
        return u.unfold(1, n, n - 1).unfold(2, n, n - 1)

    # sum element arrays [c, ez, ex, j, i] into the lattice [c, J, I]
    def assemble(self, fe):
        n, nc = self.n, fe.shape[0]
        cols = fe.permute(0, 3, 4, 1, 2).reshape(1, nc * n * n, self.nz * self.nx)
        out = F.fold(cols, output_size=(self.LZ, self.LX), kernel_size=(n, n), stride=(n - 1, n - 1))
        return out.reshape(nc, self.LZ, self.LX)

    def moduli(self, rho, vp, vs):
        mu = rho * vs * vs
        lam = rho * (vp * vp - 2.0 * vs * vs)
        return lam, mu

    def element_force(self, d, lam, mu):
        """f = -K d on the lattice for node moduli lam, mu (LZ x LX)."""
        H, Ht = self.H, self.H.t()
        L = self.elems(lam[None])[0]
        M = self.elems(mu[None])[0]
        W, xix, etaz = self.W, self.xix, self.etaz
        if self.ndof == 1:
            U = self.elems(d)[0]
            dxi, deta = U @ H, Ht @ U
            t1 = -(W * ((M * xix) * xix)) * dxi
            t2 = -(W * ((M * etaz) * etaz)) * deta
            fe = t1 @ Ht + H @ t2
            return self.assemble(fe[None])
        Ue = self.elems(d)
        Ux, Uz = Ue[0], Ue[1]
        gxx, gxz = Ux @ H, Uz @ H          # d/dxi
        gex, gez = Ht @ Ux, Ht @ Uz        # d/deta
        K = L + 2.0 * M
        a1 = -(W * ((K * xix) * xix))
        a2 = -(W * ((L * xix) * etaz))
        a3 = -(W * ((K * etaz) * etaz))
        a4 = -(W * ((M * etaz) * etaz))
        a5 = -(W * ((M * xix) * etaz))
        a6 = -(W * ((M * xix) * xix))
        rowx = a4 * (gex + gxz) if self.kd2 else a4 * gex + a5 * gxz
        fx = (a1 * gxx + a2 * gez) @ Ht + H @ rowx
        fz = (a5 * gex + a6 * gxz) @ Ht + H @ (a2 * gxx + a3 * gez)
        return self.assemble(torch.stack([fx, fz]))

    def mass(self, rho):
        Re = self.elems(rho[None])[0]
        return self.assemble((Re * self.W)[None])[0]

    def dashpots(self, rho, vp, vs, sides):
        """Absorbing coefficients C[c, J, I] summed over the given sides
        (1 bottom, 2 right, 3 top, 4 left: the tags of the Cartesian mesher)."""
        n, LX, LZ = self.n, self.LX, self.LZ
        C = torch.zeros(self.ndof, LZ, LX, dtype=torch.float64)
        wx = self.wg * (self.hx / 2.0)  # w_k |J1D| along a horizontal edge
        wz = self.wg * (self.hz / 2.0)
        for side in sides:
            if side in (1, 3):
                J = 0 if side == 1 else LZ - 1
                r, p, s = rho[J], vp[J], vs[J]
                parts = []
                for c in range(self.ndof):
                    cel = s if (self.ndof == 1 or c == 0) else p  # normal z: cp on dof z
                    v = torch.zeros(LX, dtype=torch.float64)
                    for ex in range(self.nx):
                        i0 = ex * (n - 1)
                        v = v + F.pad(r[i0:i0 + n] * cel[i0:i0 + n] * wx, (i0, LX - i0 - n))
                    parts.append(v)
                C = C + torch.stack([F.pad(v[None], (0, 0, J, LZ - 1 - J)) for v in parts])
            else:
                I = 0 if side == 4 else LX - 1
                r, p, s = rho[:, I], vp[:, I], vs[:, I]
                parts = []
                for c in range(self.ndof):
                    cel = s if (self.ndof == 1 or c == 1) else p  # normal x: cp on dof x
                    v = torch.zeros(LZ, dtype=torch.float64)
                    for ez in range(self.nz):
                        j0 = ez * (n - 1)
                        v = v + F.pad(r[j0:j0 + n] * cel[j0:j0 + n] * wz, (j0, LZ - j0 - n))
                    parts.append(v)
                C = C + torch.stack([F.pad(v[:, None], (I, LX - 1 - I)) for v in parts])
        return C


def ricker_table(nt, dt, f0, t0, ampli, tdelay=0.0):
    """Ricker amplitude at t = it*dt, it = 0..nt (stf_ricker.f90:89-103)."""
    t = np.arange(nt + 1) * dt - tdelay
    arg = (np.pi * f0 * (t - t0)) ** 2
    return -(ampli * (1.0 - 2.0 * arg)) * np.exp(-arg)


def forward(lat, rho, vp, vs, dt, nt, sides, sources, receivers, field="V", isamp=1,
            checkpoint_every=0):
    """Seismograms sis[sample, receiver, dof] of a leapfrog run.

    sources: list of (I, J, dir(ndof), amplitude table[nt+1]);
    receivers: list of (I, J) lattice nodes.
    """
    lam, mu = lat.moduli(rho, vp, vs)
    C = lat.dashpots(rho, vp, vs, sides)
    M = lat.mass(rho)[None].expand(lat.ndof, -1, -1) + (0.5 * dt) * C
    rmass = 1.0 / M
    nd = lat.ndof
    d = torch.zeros(nd, lat.LZ, lat.LX, dtype=torch.float64)
    v = torch.zeros_like(d)
    ri = torch.tensor([r[0] for r in receivers])
    rj = torch.tensor([r[1] for r in receivers])
    src = torch.zeros(nt + 1, nd, lat.LZ, lat.LX, dtype=torch.float64)
    for (I, J, dirv, amp) in sources:
        for c in range(nd):
            src[:, c, J, I] += torch.tensor(np.asarray(amp) * dirv[c], dtype=torch.float64)
    out = [torch.zeros(len(receivers), nd, dtype=torch.float64)]

    def step(d, v, it):
        d = d + dt * v
        f = lat.element_force(d, lam, mu) + src[it] - C * v
        a = rmass * f
        v = v + dt * a
        return d, v

    def seg(d, v, it0, it1):
        recs = []
        for it in range(it0, it1):
            d, v = step(d, v, it)
            if it % isamp == 0:
                fld = v if field == "V" else d
                recs.append(fld[:, rj, ri].t())
        return d, v, recs

    it = 1
    k = checkpoint_every if checkpoint_every > 0 else nt
    while it <= nt:
        it1 = min(nt + 1, it + k)
        if checkpoint_every > 0:
            res = torch.utils.checkpoint.checkpoint(
                lambda dd, vv, a=it, b=it1: (lambda o: (o[0], o[1], *o[2]))(seg(dd, vv, a, b)),
                d, v, use_reentrant=False)
            d, v, recs = res[0], res[1], list(res[2:])
        else:
            d, v, recs = seg(d, v, it, it1)
        out += recs
        it = it1
    return torch.stack(out)

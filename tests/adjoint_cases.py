"""Small gradient-workflow problems shared by the adjoint tests: P-SV or SH
boxes of uniform square elements, free top and absorbing other sides, one
Ricker force, receivers at the surface, and smooth node models."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

from sem2dpack_gb300 import PRECISION_FP64, workloads  # noqa: E402
from sem2dpack_gb300.deck import Material, ParDeck, Receivers, Sources, Time  # noqa: E402
from sem2dpack_gb300.gradient import NodeModel  # noqa: E402

SIDES = [1, 2, 4]  # absorbing: bottom, right, left (top free)


def box(nx=10, nz=10, h=100.0, ndof=2, nsteps=200, precision=PRECISION_FP64):
    Lx, Lz = nx * h, nz * h
    deck = ParDeck(
        ngll=5, ndof=ndof, fmax=10.0, xlim=(0.0, Lx), zlim=(0.0, Lz), nelem=(nx, nz),
        materials=[Material(tag=1, rho=2700.0, cp=6000.0, cs=3464.0)], absorbing=list(SIDES),
        # a fixed dt: a Courant-derived dt would move with the model
        time=Time(kind="leapfrog", dt=1.2e-3 * h / 100.0, nsteps=nsteps),
        sources=Sources(coords=[(0.45 * Lx, 0.55 * Lz)], f0=8.0, onset=0.15, ampli=1.0e10, angle=20.0),
        receivers=Receivers(number=6, first=(0.1 * Lx, Lz), last=(0.9 * Lx, Lz), field="V"),
        precision=precision,
    )
    return NodeModel(deck)


def smooth_model(model, amp=0.05, seed=0):
    """Background 2700 / 6000 / 3464 with smooth seeded perturbations."""
    rng = np.random.default_rng(seed)
    X, Z = np.meshgrid(np.linspace(0, 1, model.LX), np.linspace(0, 1, model.LZ))
    out = []
    for base in (2700.0, 6000.0, 3464.0):
        a, b, c, d = rng.uniform(1.0, 3.0, 4)
        out.append(base * (1.0 + amp * np.sin(a * np.pi * X + c) * np.cos(b * np.pi * Z + d)))
    return out


def smooth_direction(model, seed):
    rng = np.random.default_rng(1000 + seed)
    X, Z = np.meshgrid(np.linspace(0, 1, model.LX), np.linspace(0, 1, model.LZ))
    out = []
    for base in (2700.0, 6000.0, 3464.0):
        a, b, c, d = rng.uniform(0.5, 2.5, 4)
        out.append(base * 0.01 * np.sin(a * np.pi * X + c) * np.cos(b * np.pi * Z + d))
    return out


def torch_setup(model, rho, vp, vs):
    """Inputs of oracle.torch_ref.forward for the node model."""
    from oracle import torch_ref as tr
    P = workloads.build(model.deck_for(rho, vp, vs))
    d = P.desc()
    dk = model.deck
    lat = tr.Lattice(dk.nelem[0], dk.nelem[1], (dk.xlim[1] - dk.xlim[0]) / dk.nelem[0],
                     (dk.zlim[1] - dk.zlim[0]) / dk.nelem[1], n=dk.ngll, ndof=dk.ndof)
    srcs = []
    for k in range(d.nsrc):
        g = d.src_node[k] - 1
        amp = tr.ricker_table(d.nt, d.dt, d.src_f0[k], d.src_t0[k], d.src_ampli[k])
        dirv = (d.src_dir[2 * k], d.src_dir[2 * k + 1]) if dk.ndof == 2 else (1.0,)
        srcs.append((int(model.I[g]), int(model.J[g]), dirv, amp))
    recs = [(int(model.I[d.rec_node[r] - 1]), int(model.J[d.rec_node[r] - 1])) for r in range(d.nrec)]
    return lat, dict(dt=d.dt, nt=d.nt, sides=list(SIDES), sources=srcs, receivers=recs,
                     field=d.rec_field.decode(), isamp=d.rec_isamp), P


def torch_misfit_grad(model, rho, vp, vs, obs):
    """J and the autograd gradient of the FP64 reference (lattice arrays)."""
    import torch
    from oracle import torch_ref as tr
    lat, kw, _ = torch_setup(model, rho, vp, vs)
    T = lambda a: torch.tensor(a, dtype=torch.float64, requires_grad=True)
    r, p, s = T(rho), T(vp), T(vs)
    sis = tr.forward(lat, r, p, s, kw["dt"], kw["nt"], kw["sides"], kw["sources"], kw["receivers"],
                     field=kw["field"], isamp=kw["isamp"], checkpoint_every=50)
    res = sis - torch.tensor(obs, dtype=torch.float64)
    J = 0.5 * torch.sum(res * res)
    J.backward()
    g = lambda t: t.grad.numpy() if t.grad is not None else np.zeros(tuple(t.shape))
    return float(J.detach()), sis.detach().numpy(), g(r), g(p), g(s)


def oracle_misfit(model, rho, vp, vs, obs):
    """J = 1/2 sum (sis - obs)^2 with the C oracle (FP64)."""
    from oracle import pyoracle as po
    P = workloads.build(model.deck_for(rho, vp, vs))
    d = P.desc()
    o = po.OracleSim(d, owner=P)
    o.run(d.nt)
    r = o.seismograms() - obs
    return 0.5 * float(np.sum(r * r)), o.seismograms()

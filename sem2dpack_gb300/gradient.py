"""Seismogram misfit gradients with respect to density and wave speeds.

The model is given per GLL node of the structured lattice of a Cartesian
deck, as arrays (LZ, LX): node (I, J) is column I (x increasing) and row J
(z increasing).  ``NodeModel`` maps those arrays to the per-element-point
``hetero`` inputs of the deck (the reference's DIST_HETE1-style material
given at every GLL point) and maps per-global-node results back to the
lattice.  ``forward_and_gradient`` runs the forward solve with checkpoints
and the adjoint (sem2d_gpu_checkpoint_every + sem2d_gpu_adjoint);
``SeismogramFunction`` exposes the same pair as a torch.autograd.Function
whose backward is the hand-written adjoint.
"""
import ctypes as C
import dataclasses

import numpy as np

from . import abi
from ._lib import lib
from .api import Grid, Problem, Sem2dError, Solver


class NodeModel:
    """Lattice <-> reference numbering for a Cartesian deck without a fault."""

    def __init__(self, deck):
        if deck.fault is not None:
            raise ValueError("the gradient workflow has no fault")
        self.deck = deck
        self.grid = Grid(deck)
        coord = self.grid.coord()
        ux = np.unique(np.round(coord[0], 6))
        uz = np.unique(np.round(coord[1], 6))
        self.LX, self.LZ = len(ux), len(uz)
        self.I = np.searchsorted(ux, np.round(coord[0], 6))
        self.J = np.searchsorted(uz, np.round(coord[1], 6))
        self.ib = self.grid.ibool() - 1  # (ngll, ngll, nelem) global nodes

    def deck_for(self, rho, vp, vs):
        """The deck with the node model as per-element-point material."""
        take = lambda a: np.asarray(a, dtype=np.float64)[self.J[self.ib], self.I[self.ib]]
        mats = [dataclasses.replace(m, hetero=True) for m in self.deck.materials]
        return dataclasses.replace(self.deck, materials=mats,
                                   hetero={"rho": take(rho), "cp": take(vp), "cs": take(vs)})

    def to_lattice(self, values):
        """Per-global-node values -> (LZ, LX) array."""
        out = np.zeros((self.LZ, self.LX))
        out[self.J, self.I] = values
        return out


def forward_and_gradient(model, rho, vp, vs, obs=None, resid_fn=None, checkpoint_every=32,
                         precision=None):
    """Seismograms of the node model and the gradient of the misfit.

    The misfit is J = 1/2 sum (sis - obs)^2 over every sample, receiver and
    component (obs = 0 when not given), unless ``resid_fn(sis)`` returns
    (J, dJ/dsis).  Returns (J, sis, grad_rho, grad_vp, grad_vs), gradients as
    (LZ, LX) arrays.
    """
    deck = model.deck_for(rho, vp, vs)
    P = Problem(deck, model.grid)
    d = P.desc()
    if precision is not None:
        d.precision = precision
    d.adjoint = 1
    sim = Solver(d, owner=P)
    sim._check(lib().sem2d_gpu_checkpoint_every(sim.h, int(checkpoint_every)))
    sim.step(d.nt)
    sis = sim.seismograms()
    if resid_fn is None:
        r = sis - (0.0 if obs is None else obs)
        J, resid = 0.5 * float(np.sum(r * r)), r
    else:
        J, resid = resid_fn(sis)
    resid = np.asfortranarray(resid, dtype=np.float64)
    g = [np.zeros(d.npoin) for _ in range(3)]
    pp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    sim._check(lib().sem2d_gpu_adjoint(sim.h, pp(resid), pp(g[0]), pp(g[1]), pp(g[2])))
    sim.close()
    return (J, sis) + tuple(model.to_lattice(x) for x in g)


try:
    import torch

    class SeismogramFunction(torch.autograd.Function):
        """sis = F(rho, vp, vs) on the GPU; backward = the discrete adjoint.

        Inputs are (LZ, LX) FP64 tensors on any device; the output is the
        (rec_nsamp, nrec, ndof) seismogram tensor (FP64, CPU).  The forward
        keeps its GPU handle (with the checkpoints) in the autograd graph
        until the backward, which releases it: each forward supports one
        backward, and a forward without backward holds the handle until the
        graph is freed.
        """

        @staticmethod
        def forward(ctx, rho, vp, vs, model, checkpoint_every=32, precision=None):
            deck = model.deck_for(rho.detach().cpu().numpy(), vp.detach().cpu().numpy(),
                                  vs.detach().cpu().numpy())
            P = Problem(deck, model.grid)
            d = P.desc()
            if precision is not None:
                d.precision = precision
            d.adjoint = 1
            sim = Solver(d, owner=P)
            sim._check(lib().sem2d_gpu_checkpoint_every(sim.h, int(checkpoint_every)))
            sim.step(d.nt)
            sis = sim.seismograms()
            ctx.sim, ctx.model, ctx.problem = sim, model, P
            ctx.npoin = d.npoin
            ctx.device = rho.device
            return torch.from_numpy(sis.copy())

        @staticmethod
        def backward(ctx, grad_sis):
            # the adjoint consumes the handle's checkpoints: one backward per
            # forward (retain_graph does not make a second one possible)
            if ctx.sim is None:
                raise RuntimeError("SeismogramFunction supports one backward per forward: its GPU state "
                                   "was released by the first")
            resid = np.asfortranarray(grad_sis.detach().cpu().numpy(), dtype=np.float64)
            g = [np.zeros(ctx.npoin) for _ in range(3)]
            pp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
            sim = ctx.sim
            try:
                sim._check(lib().sem2d_gpu_adjoint(sim.h, pp(resid), pp(g[0]), pp(g[1]), pp(g[2])))
            finally:
                sim.close()
                ctx.sim = None
            out = [torch.from_numpy(ctx.model.to_lattice(x)).to(ctx.device) for x in g]
            return out[0], out[1], out[2], None, None, None

except ImportError:  # torch is optional for the C-ABI users
    SeismogramFunction = None

__all__ = ["NodeModel", "forward_and_gradient", "SeismogramFunction", "Sem2dError", "abi"]

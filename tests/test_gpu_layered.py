"""Grids that are not flat on the GPU: the general element coefficients
(nelast 10 in P-SV, 3 in SH; mat_elastic.f90:290-360, 499-516, 620-636)
in the strip kernel, the lattice recovered from the connectivity, against
the FP64 oracle (FP64 <= 1e-10, mixed <= 1e-4 relative L2): a layered mesh
of Q9 elements under a curved surface, SH and P-SV, Newmark, and a layered
mesh split by a slip-weakening fault."""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Problem, Solver
from sem2dpack_gb300.deck import Fault
from test_layered import layered_box

pytestmark = pytest.mark.gpu

TOL = {PRECISION_FP64: 1e-10, PRECISION_MIXED: 1e-4}
BOTH = pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def run_both(dk, precision, nsteps):
    P = Problem(dk)
    d = P.desc()
    d.precision = precision
    nsteps = min(nsteps, d.nt)
    g = Solver(d, owner=P)
    g.step(nsteps)
    o = po.OracleSim(d, owner=P)
    o.run(nsteps)
    return d, g, o


@BOTH
@pytest.mark.parametrize("ndof,scheme", [(2, "leapfrog"), (1, "leapfrog"), (2, "newmark")])
def test_curved_layers(ndof, scheme, precision):
    dk = layered_box(ndof, curved=True)
    dk.time.kind = scheme
    d, g, o = run_both(dk, precision, 250)
    assert d.xjaci
    so = o.seismograms()
    assert np.abs(so).max() > 0
    assert rel_l2(g.seismograms(), so) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision] and rel_l2(vg, vo) <= TOL[precision]


@BOTH
def test_layered_fault(precision):
    dk = layered_box(2, curved=False, ezflt=5)
    dk.fault = Fault(tags=(5, 6), friction="SWF", values={"Tn": -100e6, "Tt": 55e6, "swf_mus": 0.6,
                                                         "swf_mud": 0.5, "swf_dc": 0.4})
    dk.sources = None
    # a patch above the static strength nucleates the rupture
    x = np.linspace(0.0, 2000.0, (dk.ngll - 1) * 16 + 1)
    dk.fault.values["Tt"] = np.where(np.abs(x - 1000.0) < 200.0, 62e6, 55e6)
    d, g, o = run_both(dk, precision, 200)
    fg, fo = g.fault_series(), o.fault_series()
    for rec in (0, 1):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= TOL[precision], rec
    assert np.abs(fo[:, 1, :]).max() > 0  # the fault slips

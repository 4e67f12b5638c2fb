"""Periodic left/right sides (&BC_DEF kind='PERIOD', bc_periodic.f90) on the
GPU against the FP64 oracle: FP64 <= 1e-10, mixed <= 1e-4 relative L2.
The step kernel leaves the raw forces of the columns I = 0 and LX-1 and a
second pass sums each pair, adds the boundary terms and updates both
copies (on fault rows through the fault node update)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Problem, Solver, workloads
from sem2dpack_gb300.parinp import deck_from_parinp

from test_boundaries import periodic_box

pytestmark = pytest.mark.gpu

TOL = {PRECISION_FP64: 1e-10, PRECISION_MIXED: 1e-4}


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def run_both(deck_or_pair, nsteps, precision):
    P = workloads.build(deck_or_pair)
    d = P.desc()
    d.precision = precision
    g = Solver(d, owner=P)
    g.step(nsteps)
    o = po.OracleSim(d, owner=P)
    o.run(nsteps)
    return P, d, g, o


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("scheme", ["leapfrog", "newmark"])
def test_box(precision, scheme):
    dk = periodic_box()
    dk.time.kind = scheme
    dk.receivers.first, dk.receivers.last = (-1.5e3, -600.0), (0.9e3, -600.0)  # both periodic columns
    P, d, g, o = run_both(dk, 200, precision)
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision] and rel_l2(vg, vo) <= TOL[precision]
    m = np.ctypeslib.as_array(d.perio_master, shape=(d.nperio,)) - 1
    s = np.ctypeslib.as_array(d.perio_slave, shape=(d.nperio,)) - 1
    assert np.array_equal(dg[m], dg[s]) and np.array_equal(vg[m], vg[s])  # the copies stay one node
    assert np.abs(dg[m]).max() > 0


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_testflt1d_deck(golden, precision):
    """EXAMPLES/TestFlt1D as written: periodic sides crossed by a split
    slip-weakening fault, HHT-alpha, 40 receivers; and the 1-D steady slip
    rate 2.2 on the GPU.  The whole 568-step run of steady sliding is
    compared, so the mixed path's bound is 3e-4 here."""
    P = Problem(deck_from_parinp(str(golden["parinp_TestFlt1D"])))
    d = P.desc()
    d.precision = precision
    g = Solver(d, owner=P)
    g.run()
    o = po.OracleSim(d, owner=P)
    o.run(d.nt)
    fg, fo = g.fault_series(), o.fault_series()
    tol = TOL[precision] if precision == PRECISION_FP64 else 3e-4
    for rec in (0, 1, 2, 4):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= tol, rec
    assert rel_l2(g.seismograms(), o.seismograms()) <= tol
    t = np.arange(fg.shape[2]) * d.flt_oitd * d.dt
    assert abs(fg[0, 1, t >= 2.5].mean() / 2.2 - 1) < 5e-3


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_split_fault_across_periodic_sides(precision):
    """SH rupture on a split fault whose ends are a periodic pair."""
    deck, grid = workloads.sh_rupture(scale=0.1, nsteps=300)
    deck.absorbing = [1, 3]
    deck.periodic = (2, 4)
    P, d, g, o = run_both((deck, grid), 300, precision)
    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 0, -1].max() > 0.1
    for rec in (0, 1, 2, 4):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= TOL[precision], rec
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_bimaterial_fault_deck(golden, precision):
    """EXAMPLES/Bimaterial_fault as written (NGLL 3, two Kelvin-Voigt
    layers along a fault between two materials, Prakash-Clifton normal
    stress, periodic sides crossed by the fault), 200 steps."""
    dk = deck_from_parinp(str(golden["parinp_Bimaterial_fault"]))
    assert dk.ngll == 3 and dk.periodic == (2, 4) and dk.fault.normal_kind == 2
    P, d, g, o = run_both(dk, 200, precision)
    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 1, :].max() > 1.0  # sliding at m/s
    for rec in (0, 1, 2, 3, 4):
        assert rel_l2(fg[:, rec, :201], fo[:, rec, :201]) <= TOL[precision], rec


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("sides", ["bottom_top", "bottom_top_stacey", "left_right_stacey"])
def test_box_other_sides(sides, precision):
    """Bottom/top periodic sides (the rows J = 0 and LZ-1 finished by the
    periodic pass, as EXAMPLES/TestAbso/Par.inp has them) and Stacey sides
    that cross periodic sides (the Stacey forces of a side's two ends, a
    periodic pair, summed and shared: bc_abso.f90:329-332)."""
    dk = periodic_box(stacey="stacey" in sides)
    if sides.startswith("bottom_top"):
        dk.absorbing, dk.periodic = [2, 4], (1, 3)
        dk.stacey = [2, 4] if "stacey" in sides else []
        dk.receivers.first, dk.receivers.last = (-1.2e3, -1.0e3), (0.6e3, -1.0e3)  # on the bottom row
    else:
        dk.stacey = [1, 3]
        dk.receivers.first, dk.receivers.last = (-1.5e3, -600.0), (0.9e3, -600.0)
    P, d, g, o = run_both(dk, 200, precision)
    assert d.nstacey == (0 if sides == "bottom_top" else d.nstacey) and (d.nstacey > 0) == ("stacey" in sides)
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision] and rel_l2(vg, vo) <= TOL[precision]
    m = np.ctypeslib.as_array(d.perio_master, shape=(d.nperio,)) - 1
    s = np.ctypeslib.as_array(d.perio_slave, shape=(d.nperio,)) - 1
    assert np.array_equal(dg[m], dg[s]) and np.array_equal(vg[m], vg[s])
    assert np.abs(dg[m]).max() > 0

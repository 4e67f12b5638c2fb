"""Stacey P3 absorbing boundaries (BC_ABSO_init/BC_ABSO_apply,
bc_abso.f90:174-218,321-334) on the GPU.

Parity: the GPU step against the FP64 oracle, FP64 <= 1e-10 and mixed
<= 1e-4 relative L2, on small P-SV boxes (with and without a fault
reaching the Stacey sides).

Pin: the reference's own absorbing-boundary test (EXAMPLES/TestAbso:
Par.inp.template, run_test_PSV, test_abso_PSV.m) runs the same Ricker
force in a box whose bottom boundary is on the receiver line and in a
deeper box, and measures the misfit of the direct P and S waves against
incidence angle.  The misfit curves it saved for Stacey (stacey_PSV.mat)
and Clayton-Engquist (paraxial_PSV.mat) boundaries are golden fixtures;
this test recomputes them from GPU runs of the two boxes.
"""
import numpy as np
import pytest
from conftest import watch_launches

import decks
from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Problem, Solver, workloads
from sem2dpack_gb300.deck import Time

pytestmark = pytest.mark.gpu

TOL = {PRECISION_FP64: 1e-10, PRECISION_MIXED: 1e-4}


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def small_box(stacey=True):
    """A 2.4 x 1.5 km corner of the TestAbso box at NGLL=5, the source near
    the bottom-left corner so that P and S waves reach two Stacey sides."""
    dk = decks.test_abso(-1.0e3, 12, stacey)
    dk.ngll, dk.fmax, dk.nelem = 5, 20.0, (24, 15)
    dk.xlim, dk.zlim = (-1.5e3, 0.9e3), (-1.0e3, 0.5e3)
    dk.time = Time(kind="leapfrog", nsteps=400, courant=0.5)
    dk.sources.coords = [(-1100.0, -700.0)]
    dk.sources.f0, dk.sources.onset = 10.0, 0.1
    dk.receivers.first, dk.receivers.last = (-1500.0, -1000.0), (900.0, -1000.0)
    dk.receivers.number = 25
    return dk


def run_both(deck_or_pair, nsteps, precision):
    P = workloads.build(deck_or_pair)
    d = P.desc()
    d.precision = precision
    g = Solver(d, owner=P)
    g.step(nsteps)
    o = po.OracleSim(d, owner=P)
    o.run(nsteps)
    return P, g, o


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("field", ["V", "D"])
def test_small_box_against_oracle(precision, field):
    dk = small_box()
    dk.receivers.field = field
    P, g, o = run_both(dk, 400, precision)
    assert P.desc().nstacey == (2 * 24 + 2 * 15) * 5
    s_g, s_o = g.seismograms(), o.seismograms()
    assert np.abs(s_o).max() > 0
    assert rel_l2(s_g, s_o) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision]
    assert rel_l2(vg, vo) <= TOL[precision]
    assert g.launches == 2 * 400 + watch_launches(400)  # Stacey forces, then the step


def test_stacey_changes_the_answer():
    _, g1, _ = run_both(small_box(True), 400, PRECISION_FP64)
    _, g0, _ = run_both(small_box(False), 400, PRECISION_FP64)
    assert rel_l2(g1.seismograms(), g0.seismograms()) > 1e-3


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_fault_reaching_stacey_sides(precision):
    """P-SV rate-and-state fault whose end nodes lie on the left and right
    Stacey sides: the boundary force enters the fault's trial traction."""
    deck, grid = workloads.psv_rsf(scale=0.05, nsteps=300, rsf_kind=2)
    deck.stacey = list(deck.absorbing)
    P, g, o = run_both((deck, grid), 300, precision)
    assert P.desc().nstacey > 0
    fg, fo = g.fault_series(), o.fault_series()
    if precision == PRECISION_FP64:  # the rate-and-state solve: 1e-9, as for the fault without Stacey sides
        for rec in (0, 1, 2, 3, 4):
            assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= 1e-9, rec
        assert rel_l2(g.seismograms(), o.seismograms()) <= 1e-9
    else:
        for rec in (0, 1):
            assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= 1e-4, rec


def abso_misfit(s1, s2, dt, xsta, t0=0.05, delta=1.0e3, vp=5000.0, vs=2887.0):
    """The misfits of test_abso_PSV.m:95-136.  s1 (shallow box) and s2 (deep
    box) are velocity seismograms (nsamp + 1, nsta, 2) with row 0 at time 0;
    the script integrates them by a cumulative sum (:14-15) and compares
    windows of 2 x 1.5 t0 around the direct P and S arrivals."""
    u1 = np.cumsum(s1[1:], axis=0)
    u2 = np.cumsum(s2[1:], axis=0)
    nsamp, nsta = u1.shape[0], u1.shape[1]
    theta = np.degrees(np.arctan(xsta / delta))
    tw = 1.5 * t0

    def err(i, tp):
        w1, w2 = int(np.floor((tp - tw) / dt)), int(np.ceil((tp + tw) / dt))
        a, b = u1[w1 - 1:w2, i], u2[w1 - 1:w2, i]
        return np.sqrt(((b - a) ** 2).sum() / (b ** 2).sum())

    tp = t0 + np.sqrt(delta ** 2 + xsta ** 2) / vp
    errp = np.zeros(nsta)
    for i in range(nsta):
        if np.ceil((tp[i] + tw) / dt) > nsamp:
            break
        errp[i] = err(i, tp[i])
    ts = t0 + np.sqrt(delta ** 2 + xsta ** 2) / vs
    tp2 = np.floor((t0 + np.sqrt((5 * delta) ** 2 + xsta ** 2) / vp - tw) / dt)
    nsta_s = int(np.count_nonzero(np.ceil((ts + tw) / dt) <= tp2))
    errs = np.array([err(i, ts[i]) for i in range(nsta_s)])
    return theta, errp, errs


# the reference's seismograms were FP32 files: its misfits carry ~1e-5 of
# rounding against these FP64 runs
MISFIT_ATOL = 1e-4


@pytest.mark.parametrize("kind", ["stacey", "paraxial"])
def test_testabso_misfit_curves(kind, golden):
    runs = []
    for zb, nz in ((-1.0e3, 60), (-3.0e3, 100)):
        P = Problem(decks.test_abso(zb, nz, kind == "stacey"))
        d = P.desc()
        d.precision = PRECISION_FP64
        g = Solver(d, owner=P)
        g.run()
        runs.append((g.seismograms(), P.rec_coord()[0], d.dt * d.rec_isamp))
    (s1, xsta, dt), (s2, _, _) = runs
    theta, errp, errs = abso_misfit(s1, s2, dt, xsta)
    np.testing.assert_allclose(theta, golden["abso_%s_theta" % kind], atol=1e-6)
    assert len(errs) == len(golden["abso_%s_errs" % kind])
    gp, gs = golden["abso_%s_errp" % kind], golden["abso_%s_errs" % kind]
    assert np.abs(errp - gp).max() <= MISFIT_ATOL, np.abs(errp - gp).max()
    assert np.abs(errs - gs).max() <= MISFIT_ATOL, np.abs(errs - gs).max()


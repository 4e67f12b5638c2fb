"""Explicit HHT-alpha (solve_HHT_alpha, solver.f90:89-131) on the GPU
against the FP64 oracle: forces, Kelvin-Voigt and dashpot terms at
d_alpha, v_alpha; sources at t + (alpha-1) dt; the Newmark corrector with
the beta and gamma the scheme derives from alpha and rho (time.f90:222-240).
FP64 <= 1e-10, mixed <= 1e-4 relative L2.
"""
import numpy as np
import pytest
from conftest import watch_launches

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Solver, workloads
from sem2dpack_gb300.deck import Time

from test_gpu_newmark import box

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
    return P, g, o


def hht_box(field, alpha=0.5, rho=0.5, atnode=True):
    dk = box(0.0, field, atnode)
    dk.time = Time(kind="hht-alpha", nsteps=200, courant=0.3, alpha=alpha, rho=rho)
    return dk


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("field", ["D", "V", "A"])
def test_box(precision, field):
    P, g, o = run_both(hht_box(field), 200, precision)
    d = P.desc()
    assert d.alpha == 0.5 and d.gamma == 1.0 and abs(d.beta - (0.5 - 0.25 * -0.5 / (0.5 * 1.5 ** 3))) < 1e-15
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    dg, vg, ag = g.fields(accel=True)
    do, vo, ao = o.fields()
    for x, y in ((dg, do), (vg, vo), (ag, ao)):
        assert rel_l2(x, y) <= TOL[precision]


def test_interpolated_displacement():
    P, g, o = run_both(hht_box("D", atnode=False), 200, PRECISION_FP64)
    assert rel_l2(g.seismograms(), o.seismograms()) <= 1e-10
    assert g.launches == 2 * 200 + watch_launches(200)


def test_alpha_one_is_newmark():
    """alpha = 1 sets rho aside: gamma = 1/2, beta = 0, the explicit Newmark
    scheme (time.f90:230-236), bit for bit on the GPU."""
    _, g1, _ = run_both(hht_box("V", alpha=1.0), 200, PRECISION_FP64)
    dk = box(0.0, "V")
    dk.time.nsteps = 200
    _, g0, _ = run_both(dk, 200, PRECISION_FP64)
    assert np.array_equal(g1.seismograms(), g0.seismograms())


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_kelvin_voigt(precision):
    dk = workloads.plain_psv(scale=0.2, nsteps=200)
    dk.materials[0].kv_eta = 0.2
    dk.time = Time(kind="hht-alpha", nsteps=200, courant=0.4, alpha=0.6, rho=0.8)
    P, g, o = run_both(dk, 200, precision)
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_fault(precision):
    """SH slip-weakening rupture under HHT-alpha; receivers on the fault line."""
    deck, grid = workloads.sh_rupture(scale=0.1, nsteps=400)
    deck.time = Time(kind="hht-alpha", nsteps=400, courant=0.5, alpha=0.7, rho=0.7)
    deck.fault.potency = True
    zf = 0.5 * deck.zlim[1]
    deck.receivers.first, deck.receivers.last = (deck.receivers.first[0], zf), (deck.receivers.last[0], zf)
    P, g, o = run_both((deck, grid), 400, precision)
    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 0, -1].max() > 0.1
    for rec in (0, 1, 2, 4):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= TOL[precision], rec
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    assert rel_l2(g.fault_potency(), o.fault_potency()) <= TOL[precision]


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_stacey(precision):
    """Stacey P3 sides under HHT-alpha take d_alpha (displ_alpha,
    bc_gen.f90:295)."""
    dk = hht_box("V")
    dk.stacey = list(dk.absorbing)
    P, g, o = run_both(dk, 200, precision)
    assert P.desc().nstacey > 0
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision]

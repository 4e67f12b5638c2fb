"""Newmark predictor-corrector with beta != 0 on the GPU against the FP64
oracle (solve_Newmark, solver.f90:42-84): the predictor
d + dt v + (1/2 - beta) dt^2 a, the corrector d += beta dt^2 a.

The step buffers hold the predictor; the corrected displacement reaches the
receivers, the fault (slip uses CoefA2D = beta dt^2, bc_dynflt.f90:333-335,
and the slip-weakening state takes |D| on that branch, bc_dynflt.f90:645),
the potency, get_fields and the strain output.

Tolerances as in the other parity tests: FP64 <= 1e-10, mixed <= 1e-4
relative L2.
"""
import numpy as np
import pytest
from conftest import watch_launches

import decks
from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Solver, workloads

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


def box(beta, field, atnode=True):
    dk = decks.inabox()
    dk.time.total_time = 0.0
    dk.time.nsteps = 200
    dk.time.beta = beta
    dk.receivers = workloads.plain_psv(scale=0.4).receivers
    dk.receivers.first, dk.receivers.last = (-800.0, -700.0), (800.0, 600.0)
    dk.receivers.field = field
    dk.receivers.atnode = atnode
    return dk


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("field", ["D", "V", "A"])
def test_box_receivers_and_fields(precision, field):
    P, g, o = run_both(box(0.25, field), 200, precision)
    s_g, s_o = g.seismograms(), o.seismograms()
    assert np.abs(s_o).max() > 0
    assert rel_l2(s_g, s_o) <= TOL[precision]
    dg, vg, ag = g.fields(accel=True)
    do, vo, ao = o.fields()
    assert rel_l2(dg, do) <= TOL[precision]
    assert rel_l2(vg, vo) <= TOL[precision]
    assert rel_l2(ag, ao) <= TOL[precision]
    assert g.launches == 200 + watch_launches(200)  # node receivers inside the step kernel


def test_corrector_changes_the_answer():
    """beta = 0.25 and beta = 0 differ well above the tolerance, so the
    parity above is a test of the corrector."""
    _, g0, _ = run_both(box(0.0, "D"), 200, PRECISION_FP64)
    _, g1, _ = run_both(box(0.25, "D"), 200, PRECISION_FP64)
    assert rel_l2(g1.seismograms(), g0.seismograms()) > 1e-6


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_interpolated_displacement(precision):
    """Interpolated displacement with the corrector needs the new
    accelerations of nodes owned by several CTAs: the separate sampling
    kernel records it after the step."""
    P, g, o = run_both(box(0.25, "D", atnode=False), 200, precision)
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    assert g.launches == 2 * 200 + watch_launches(200)


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_strain_stress(precision):
    P, g, o = run_both(box(0.25, "V"), 150, precision)
    eg, sg = g.strain_stress()
    eo, so = o.strain_stress()
    assert rel_l2(eg, eo) <= TOL[precision]
    assert rel_l2(sg, so) <= TOL[precision]


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("field", ["D", "V"])
def test_fault_rupture(precision, field):
    """SH slip-weakening rupture with beta = 0.25: CoefA2D != 0 selects the
    theta = |D| state update; receivers on the fault line are sampled after
    the fault update, by the separate sampling kernel."""
    deck, grid = workloads.sh_rupture(scale=0.1, nsteps=400)
    deck.time.kind = "newmark"
    deck.time.beta, deck.time.gamma = 0.25, 0.5
    deck.fault.potency = True
    deck.receivers.field = field
    zf = 0.5 * deck.zlim[1]  # receivers on the fault line
    deck.receivers.first, deck.receivers.last = (deck.receivers.first[0], zf), (deck.receivers.last[0], zf)
    P, g, o = run_both((deck, grid), 400, precision)
    assert np.all(P.rec_coord()[1] == zf)
    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 0, -1].max() > 0.1  # the rupture slipped
    for rec, name in ((0, "slip"), (1, "slip rate"), (2, "shear"), (4, "friction")):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= TOL[precision], name
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    pg, po_ = g.fault_potency(), o.fault_potency()
    assert rel_l2(pg, po_) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision]

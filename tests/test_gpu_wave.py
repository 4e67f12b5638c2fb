"""Incident plane waves (src_wave.f90, BC_ABSO_apply bc_abso.f90:279-306),
source time functions other than Ricker (stf_*.f90) and time-dependent
Neumann tractions (bc_DIRNEU_apply bc_dirneu.f90:148-169) on the GPU
against the FP64 oracle: FP64 <= 1e-10, mixed <= 1e-4 relative L2 of the
seismograms and the velocity field; and the GPU's plane wave against its
analytic form in the periodic box of test_oracle_wave."""
import numpy as np
import pytest

import decks
from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Problem, Solver
from sem2dpack_gb300.deck import Stf
from test_oracle_wave import analytic_case, compare

pytestmark = pytest.mark.gpu

TOL = {PRECISION_FP64: 1e-10, PRECISION_MIXED: 1e-4}
BOTH = pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def run_both(dk, precision, nsteps=None):
    """GPU and oracle runs of nsteps (default: half the run, while the
    incident wave is still in the box: after it has left, the fields are
    residues at the FP32 rounding level of the pulse)."""
    P = Problem(dk)
    d = P.desc()
    d.precision = precision
    n = nsteps or d.nt // 2
    g = Solver(d, owner=P)
    g.step(n)
    o = po.OracleSim(d, owner=P)
    o.run(n)
    return d, g, o


def check(g, o, precision):
    so = o.seismograms()
    assert np.abs(so).max() > 0
    assert rel_l2(g.seismograms(), so) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(vg, vo) <= TOL[precision]
    assert rel_l2(dg, do) <= TOL[precision]


@BOTH
@pytest.mark.parametrize("ndof,phase,angle", [(1, "S", 0.0), (1, "S", 30.0), (2, "P", 0.0), (2, "S", -45.0),
                                              (2, "P", 150.0), (2, "S", 60.0)])
def test_incident_wave(ndof, phase, angle, precision):
    d, g, o = run_both(decks.wave_box(ndof, phase, angle, tdelay=0.02), precision)
    check(g, o, precision)


@BOTH
def test_incident_wave_periodic_and_let_wave(precision):
    """Periodic left/right sides (their own pass adds the wave to the summed
    node pairs) and a top side with let_wave=F."""
    d, g, o = run_both(decks.wave_box(2, "S", 20.0, periodic=True, no_wave=[3]), precision)
    check(g, o, precision)


@BOTH
def test_incident_wave_other_time_functions(precision):
    t = np.linspace(0.0, 0.4, 17)
    for stf in (Stf("GAUSSIAN", f0=8.0, onset=0.15, ampli=1.0),
                Stf("TAB", tab=(t, np.exp(-((t - 0.15) / 0.04) ** 2)))):
        d, g, o = run_both(decks.wave_box(2, "P", 10.0, stf=stf), precision)
        check(g, o, precision)


@pytest.mark.parametrize("ndof,phase", [(1, "S"), (2, "P"), (2, "S")])
def test_gpu_wave_is_the_analytic_plane_wave(ndof, phase):
    dk = analytic_case(ndof, phase)
    P = Problem(dk)
    d = P.desc()
    for precision in (PRECISION_FP64, PRECISION_MIXED):
        d.precision = precision
        g = Solver(d, owner=P)
        g.step(d.nt)
        assert compare(dk, g.seismograms(), d.dt, d.rec_isamp) <= 5e-3
        g.close()


# the receivers are 700 and 1200 m from the source: the P wave of the pulse
# centred at 0.15 s passes them by 0.55 s (1100 steps of 0.5 ms); before it
# arrives they record only the tail of the discrete operator, a residue that
# is no test of the precision
STF_STEPS = 1100


def stf_deck(kind, ngll):
    dk = decks.lambs_problem()
    dk.nelem, dk.fmax, dk.ngll = (20, 10), 8.0 if ngll == 9 else 4.0, ngll
    t = np.linspace(0.0, 0.5, 11)
    dk.sources.stf = Stf(kind, f0=10.1, onset=0.15, ampli=1.3, par1=0.7,
                         tab=(t, np.sin(20 * t)) if kind == "TAB" else None)
    return dk


@BOTH
@pytest.mark.parametrize("kind", ["GAUSSIAN", "BRUNE", "HARMONIC", "USER", "TAB"])
def test_point_source_time_functions(kind, precision):
    """NGLL 5: the one-element-per-thread kernel, which keeps the elastic
    force as its state in mixed precision when a time function has a net
    impulse (a static displacement that FP32 would not resolve against the
    dynamic one)."""
    d, g, o = run_both(stf_deck(kind, 5), precision, nsteps=STF_STEPS)
    check(g, o, precision)


@BOTH
@pytest.mark.parametrize("kind", ["GAUSSIAN", "TAB"])
def test_point_source_time_functions_strip(kind, precision):
    """NGLL 9: the strip kernel, which keeps the force state too under
    leapfrog."""
    d, g, o = run_both(stf_deck(kind, 9), precision, nsteps=STF_STEPS)
    check(g, o, precision)


@BOTH
@pytest.mark.parametrize("ndof", [1, 2])
def test_neumann_tractions(ndof, precision):
    dk = decks.traction_box(ndof, hstf=Stf("GAUSSIAN", f0=8.0, onset=0.1, ampli=1e6),
                            vstf=Stf("RICKER", f0=10.0, onset=0.12, ampli=2e6) if ndof == 2 else None)
    d, g, o = run_both(dk, precision)
    assert d.nneu > 0
    check(g, o, precision)


def test_boundary_forces_refused_where_unsupported():
    """Batches and the adjoint refuse problems with boundary time functions."""
    from sem2dpack_gb300 import Sem2dError
    from sem2dpack_gb300.api import BatchSolver
    dk = decks.wave_box(2, "P", 0.0)
    P = Problem(dk)
    d = P.desc()
    d.precision = PRECISION_MIXED
    with pytest.raises(Sem2dError):
        BatchSolver([d], owners=[P])

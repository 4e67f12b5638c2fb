"""GPU against the FP64 oracle for the 2.5D crustal-plane term
(mat_elastic.f90:363-383, 447-459) and time-weakening friction
(bc_dynflt_twf.f90:117-184), alone and superimposed on slip weakening or
rate and state.  Tolerances as in test_gpu_parity.py: FP64 <= 1e-10
(rate and state <= 1e-9), mixed <= 1e-4 relative L2."""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Solver, workloads
from sem2dpack_gb300.deck import TimeWeakening

pytestmark = pytest.mark.gpu

TOL = {PRECISION_FP64: 1e-10, PRECISION_MIXED: 1e-4}


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def run_both(pair, nsteps, precision):
    P = workloads.build(pair)
    d = P.desc()
    d.precision = precision
    g = Solver(d, owner=P)
    g.step(nsteps)
    o = po.OracleSim(d, owner=P)
    o.run(nsteps)
    return g, o


def twf_pair(kind, friction, nsteps=300):
    deck, grid = workloads.sh_rupture(scale=0.1, nsteps=nsteps, out_every=5)
    n1, _ = grid.fault_nodes()
    xz = grid.coord()[:, n1 - 1]
    x0 = float(xz[0, xz.shape[1] // 2])
    deck.fault.friction = friction
    deck.fault.twf = TimeWeakening(kind=kind, mus=0.68, mud=0.52, mu0=0.6, X=x0,
                                   Z=float(xz[1, 0]), V=1500.0, L=250.0, T=0.5, Dc=0.4)
    return deck, grid


@pytest.mark.parametrize("kind", [1, 2, 3])
def test_time_weakening_alone(kind):
    g, o = run_both(twf_pair(kind, "TWF"), 300, PRECISION_FP64)
    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 0, -1].max() > 0.0  # the imposed front slipped the fault
    for rec in (0, 1, 2, 5):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= 1e-10, rec
    # friction: huge(1d0) ahead of the front, the law's value behind it
    big_g, big_o = fg[:, 4, :] > 1e300, fo[:, 4, :] > 1e300
    assert np.array_equal(big_g, big_o) and big_o.any() and (~big_o).any()
    assert rel_l2(fg[:, 4, :][~big_o], fo[:, 4, :][~big_o]) <= 1e-10
    assert rel_l2(g.seismograms(), o.seismograms()) <= 1e-10


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_time_weakening_on_slip_weakening(precision):
    deck, grid = twf_pair(1, "SWF")
    deck.fault.twf.mu0 = 0.55  # below the stress ratio: the front nucleates slip
    deck.fault.twf.V = 2000.0
    g, o = run_both((deck, grid), 300, precision)
    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 0, -1].max() > 1e-3
    for rec in (0, 1, 2, 4):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= TOL[precision], rec


def test_time_weakening_on_rate_and_state():
    deck, grid = workloads.psv_rsf(scale=0.05, nsteps=300, rsf_kind=2)
    n1, _ = grid.fault_nodes()
    xz = grid.coord()[:, n1 - 1]
    deck.fault.twf = TimeWeakening(kind=1, mus=0.6, mud=0.3, mu0=0.55,
                                   X=float(xz[0, xz.shape[1] // 3]), Z=float(xz[1, 0]),
                                   V=2000.0, L=200.0, T=0.2)
    g, o = run_both((deck, grid), 300, PRECISION_FP64)
    fg, fo = g.fault_series(), o.fault_series()
    for rec in (0, 1, 2, 3, 4):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= 1e-9, rec


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_25d_psv(precision):
    deck = workloads.plain_psv(scale=0.2, nsteps=300)
    deck.width = 2.0e3
    g, o = run_both(deck, 300, precision)
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision]


def test_25d_sh_rupture():
    deck, grid = workloads.sh_rupture(scale=0.1, nsteps=300)
    deck.width = 4.0e3
    g, o = run_both((deck, grid), 300, PRECISION_FP64)
    fg, fo = g.fault_series(), o.fault_series()
    for rec in (0, 1, 2):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= 1e-10, rec
    assert rel_l2(g.seismograms(), o.seismograms()) <= 1e-10


def test_25d_rejects_anisotropic():
    import decks
    deck = decks.anisotropic()
    deck.width = 1.0
    P = workloads.build(deck)
    with pytest.raises(RuntimeError, match="isotropic"):
        Solver(P.desc(), owner=P)

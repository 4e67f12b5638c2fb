"""Oracle checks of the 2.5D term and time-weakening friction that need no GPU.

* twf_mu kind 1 (bc_dynflt_twf.f90:136-167): at time 0 the friction at the
  hypocentre equals Mu0 (the time shift is chosen for that), MuD well inside
  the front and the large value beyond it; kind 2 likewise gives Mu0 at the
  hypocentre.
* MAT_ELAST_add_25D_f (mat_elastic.f90:447-459) vanishes as W grows: W = 1e30
  reproduces the 2D run.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, workloads
from sem2dpack_gb300.deck import TimeWeakening


def twf_sim(kind, **kw):
    deck, grid = workloads.sh_rupture(scale=0.05, nsteps=20, out_every=5)
    n1, _ = grid.fault_nodes()
    xz = grid.coord()[:, n1 - 1]
    k0 = xz.shape[1] // 2
    deck.fault.friction = "TWF"
    prm = dict(kind=kind, mus=0.68, mud=0.52, mu0=0.6, X=float(xz[0, k0]), Z=float(xz[1, 0]),
               V=1500.0, L=250.0, T=0.5)
    prm.update(kw)
    deck.fault.twf = TimeWeakening(**prm)
    P = workloads.build((deck, grid))
    d = P.desc()
    d.precision = PRECISION_FP64
    return po.OracleSim(d, owner=P), xz, k0, prm


@pytest.mark.parametrize("kind", [1, 2])
def test_twf_hypocentre_starts_at_mu0(kind):
    sim, xz, k0, prm = twf_sim(kind)
    MU = sim.fault_state()[3]
    assert MU[k0] == pytest.approx(prm["mu0"], rel=1e-12)
    far = np.abs(xz[0] - prm["X"]) > 2000.0
    assert np.all(MU[far] > 1e300)  # beyond the front: stuck


def test_twf_kind1_front_moves_at_V():
    sim, xz, k0, prm = twf_sim(1, mu0=0.68)  # front starts at the hypocentre
    dt = sim.desc.dt
    sim.run(20)
    MU = sim.fault_state()[3]
    r = np.abs(xz[0] - prm["X"]) - prm["V"] * 20 * dt
    mid = (r > -prm["L"]) & (r <= prm["L"])
    expect = prm["mus"] + (prm["mus"] - prm["mud"]) / prm["L"] * r[mid]
    np.testing.assert_allclose(MU[mid], expect, rtol=1e-12)
    assert np.all(MU[r < -prm["L"]] == prm["mud"])


def test_25d_vanishes_for_large_width():
    deck = workloads.plain_psv(scale=0.05, nsteps=60)
    P0 = workloads.build(deck)
    deck.width = 1e30
    P1 = workloads.build(deck)
    out = []
    for P in (P0, P1):
        d = P.desc()
        o = po.OracleSim(d, owner=P)
        o.run(60)
        out.append(o.seismograms())
    assert np.abs(out[0]).max() > 0
    np.testing.assert_allclose(out[1], out[0], rtol=0, atol=1e-14 * np.abs(out[0]).max())


def test_25d_finite_width_changes_the_response():
    deck = workloads.plain_psv(scale=0.05, nsteps=60)
    P0 = workloads.build(deck)
    deck.width = 500.0
    P1 = workloads.build(deck)
    s = []
    for P in (P0, P1):
        o = po.OracleSim(P.desc(), owner=P)
        o.run(60)
        s.append(o.seismograms())
    assert np.linalg.norm(s[1] - s[0]) > 1e-6 * np.linalg.norm(s[0])

"""The oracle against the reference's own data (EXAMPLES/ of SEM2DPACK).

These pin the CPU restatement before it is trusted as the checker:
  * GLL points and weights for n=5 in closed form;
  * InaBox check-mode log: element and node counts, dt and nt;
  * Lamb's problem: the reference's recorded misfits to the analytic
    solution (LambsProblem/test.out:12) are reproduced;
  * TestSH: the reference's pass criterion (TestSH/analyze_test.m:14-15);
  * Anisotropic: the reference's own seismograms p1..p4.tab.
"""
import numpy as np
import pytest

import decks
from oracle import pyoracle as po


def test_gll_closed_form():
    x, w, H = po.gll(5)
    r = np.sqrt(3.0 / 7.0)
    np.testing.assert_allclose(x, [-1, -r, 0, r, 1], rtol=0, atol=1e-15)
    np.testing.assert_allclose(w, [1 / 10, 49 / 90, 32 / 45, 49 / 90, 1 / 10], rtol=1e-14)
    assert x[2] == 0.0
    # derivative matrix: rows of H^T differentiate polynomials of degree <= 4 exactly
    for k in range(5):
        np.testing.assert_allclose(H.T @ x ** k, k * x ** max(k - 1, 0) if k else 0 * x, atol=1e-12)


def test_inabox_known_answers(golden):
    s = po.OracleSetup(decks.inabox())
    dt, nt, courant = s.time()
    assert s.nelem == int(golden["inabox_nelem"])
    assert s.npoin == int(golden["inabox_npoin"])
    assert nt == int(golden["inabox_nt"])
    assert abs(dt - float(golden["inabox_dt"])) <= 0.5e-9  # log prints 681.605E-06
    assert abs(courant - 0.3) < 1e-12


def test_ibool_hand_3x2():
    """ibool of a 3 x 2 Q4 mesh, NGLL=2, numbered by hand from the rules of
    SE_init_numbering (spec_grid.f90:198-314) after RCM renumbering."""
    from sem2dpack_gb300.deck import Material, ParDeck, Time
    dk = ParDeck(ngll=2, ndof=1, fmax=1e-3, xlim=(0, 3), zlim=(0, 2), nelem=(3, 2),
                 materials=[Material(tag=1, rho=1, cp=2, cs=1)], time=Time(dt=0.01, nsteps=1))
    s = po.OracleSetup(dk, grid_only=True)
    ib = s.ibool()
    # every element owns exactly its four corners; 12 nodes in total
    assert s.npoin == 12
    coord = s.coord()
    kn = s.knods()
    for e in range(6):
        corners = coord[:, ib[:, :, e].ravel(order="F") - 1]
        xs, zs = sorted(set(corners[0])), sorted(set(corners[1]))
        assert len(xs) == 2 and len(zs) == 2 and xs[1] - xs[0] == 1 and zs[1] - zs[0] == 1
    # element 1 (first in RCM order) gets nodes 1..4 in vertex order 1,2,3,4
    assert list(ib[:, :, 0].ravel(order="F")) == [1, 2, 4, 3]
    # RCM starts from a corner element of the 3 x 2 box (pseudo-peripheral root)
    first = kn[:, 0]
    assert set(first) <= set(range(1, 13))


@pytest.mark.slow
def test_lamb_recorded_misfit(golden):
    s, sim = po.run_deck(decks.lambs_problem())
    sis = sim.seismograms()
    uxa = np.vstack([np.zeros((1, 2)), golden["lamb_ux"].reshape(3000, 2, order="F")])
    uza = np.vstack([np.zeros((1, 2)), golden["lamb_uz"].reshape(3000, 2, order="F")])
    A = np.hstack([uxa, uza])
    U = np.hstack([sis[:, :, 0], sis[:, :, 1]])
    err = np.abs(U - A).max(0) / np.abs(A).max(0)
    assert err.max() < 0.005                       # analyze_test.m:22
    # the reference's recorded misfits (5 significant digits, FP32 output)
    np.testing.assert_allclose(err, golden["lamb_recorded_misfit"], rtol=2e-4)


@pytest.mark.slow
def test_sh_point_force(golden):
    s, sim = po.run_deck(decks.test_sh())
    u = sim.seismograms()[:, 4, 0]
    uref = golden["sh_uref"]
    assert u.shape == uref.shape
    err = np.abs(u - uref).max() / np.abs(uref).max()
    assert err < 0.02                              # analyze_test.m:15


@pytest.mark.slow
def test_anisotropic_reference_output(golden):
    """p{1..4}.tab hold t, ux, uz of the reference at stations 4, 18, 23, 46
    (Anisotropic/write_seis.m); row k is sample k (t = k dt).  1000 of the
    2001 steps are run to keep the suite short."""
    nsteps = 1000
    s, sim = po.run_deck(decks.anisotropic(), nsteps=nsteps)
    sis = sim.seismograms()
    for k, st in enumerate(golden["aniso_stations"]):
        p = golden["aniso_p%d" % (k + 1)][: nsteps]
        for c in (0, 1):
            ref = p[:, 1 + c]
            got = sis[1:nsteps + 1, st - 1, c]
            scale = np.abs(golden["aniso_p%d" % (k + 1)][:, 1 + c]).max()
            assert np.abs(got - ref).max() / scale < 2e-6

"""Stacey P3 and zero-Dirichlet (&BC_DIRNEU) boundary tables of the host
builder, and the oracle's use of them, on the CPU.

Stacey (BC_ABSO_init, bc_abso.f90:174-218): on the Cartesian mesher's flat
rectangular elements |dx/dloc_t| dloc_t/dx_t = 1, so
K(k,c,e) = w_k rho cs (2 cs - cp), negated for the tangential component;
each term lists its element edge's nodes in SE_inquire's traversal order
(spec_grid.f90:876-881).
"""
import numpy as np
import pytest

import decks
from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, Problem
from sem2dpack_gb300.deck import Time
from sem2dpack_gb300.parinp import deck_from_parinp


def arr(d, name, n):
    return np.ctypeslib.as_array(getattr(d, name), shape=(n,)).copy()


def small_box(stacey=True):
    dk = decks.test_abso(-1.0e3, 12, stacey)
    dk.ngll, dk.fmax, dk.nelem = 5, 20.0, (24, 15)
    dk.xlim, dk.zlim = (-1.5e3, 0.9e3), (-1.0e3, 0.5e3)
    dk.time = Time(kind="leapfrog", nsteps=200, courant=0.5)
    dk.sources.coords = [(-1100.0, -700.0)]
    dk.sources.f0, dk.sources.onset = 10.0, 0.1
    dk.receivers.first, dk.receivers.last = (-1500.0, -1000.0), (900.0, -1000.0)
    dk.receivers.number = 25
    return dk


def test_stacey_table():
    P = Problem(small_box())
    d = P.desc()
    N, nt = d.ngll, d.nstacey
    assert nt == (2 * 24 + 2 * 15) * N
    K = arr(d, "stacey_K", 2 * nt).reshape(2, nt)
    node = arr(d, "stacey_node", nt)
    k = arr(d, "stacey_k", nt)
    edge = arr(d, "stacey_edge", N * nt).reshape(nt, N)
    _, w, _ = P.grid.gll()
    rho, cp, cs = 2500.0, 5000.0, 2887.0
    kmag = w[k] * rho * cs * (2 * cs - cp)
    xz = P.grid.coord()
    x, z = xz[0, node - 1], xz[1, node - 1]
    horiz = np.isclose(z, -1.0e3) | np.isclose(z, 0.5e3)
    # corner nodes belong to both sides: the side is the one the edge runs along
    ex, ez = xz[0, edge - 1], xz[1, edge - 1]
    along_x = np.ptp(ez, axis=1) < 1e-9
    assert np.all(along_x[horiz & ~(np.isclose(x, -1.5e3) | np.isclose(x, 0.9e3))])
    np.testing.assert_allclose(np.abs(K[0]), kmag, rtol=1e-13)
    np.testing.assert_allclose(K[0][along_x], -kmag[along_x], rtol=1e-13)
    np.testing.assert_allclose(K[1][along_x], kmag[along_x], rtol=1e-13)
    np.testing.assert_allclose(K[0][~along_x], kmag[~along_x], rtol=1e-13)
    np.testing.assert_allclose(K[1][~along_x], -kmag[~along_x], rtol=1e-13)
    # the term's node is edge point k of its edge
    assert np.array_equal(edge[np.arange(nt), k], node)
    # counter-clockwise traversal: the bottom side runs in +x, the top in -x
    bottom = along_x & np.isclose(ez[:, 0], -1.0e3)
    top = along_x & np.isclose(ez[:, 0], 0.5e3)
    assert np.all(np.diff(ex[bottom], axis=1) > 0) and np.all(np.diff(ex[top], axis=1) < 0)


def test_stacey_needs_psv_and_is_absorbing():
    dk = small_box()
    dk.ndof = 1
    P = Problem(dk)
    assert P.desc().nstacey == 0  # bc_abso.f90:176: P-SV only
    dk = small_box(False)
    dk.stacey = [2]
    dk.absorbing = [1, 3, 4]
    with pytest.raises(ValueError):
        Problem(dk)


def test_oracle_stacey_changes_the_answer():
    out = []
    for st in (True, False):
        P = Problem(small_box(st))
        d = P.desc()
        d.precision = PRECISION_FP64
        o = po.OracleSim(d, owner=P)
        o.run(200)
        out.append(o.seismograms())
    assert np.abs(out[0]).max() > 0
    assert np.linalg.norm(out[0] - out[1]) > 1e-3 * np.linalg.norm(out[1])


def dirneu_box(h="N", v="D", tag=4):
    dk = small_box(False)
    dk.absorbing = [t for t in dk.absorbing if t != tag]
    dk.dirneu = [(tag, h, v, True)]
    return dk


def test_dirneu_table_and_oracle_zero():
    P = Problem(dirneu_box())
    d = P.desc()
    assert d.ndir == 15 * 4 + 1  # the left side's nodes, vertical component
    node = arr(d, "dir_node", d.ndir)
    assert np.all(arr(d, "dir_comp", d.ndir) == 1)
    assert np.all(arr(d, "dir_after_fault", d.ndir) == 0)
    xz = P.grid.coord()
    assert np.allclose(xz[0, node - 1], -1.5e3)
    d.precision = PRECISION_FP64
    o = po.OracleSim(d, owner=P)
    o.run(200)
    D, V, A = o.fields()
    assert np.abs(D[:, 1]).max() > 0
    assert np.all(D[node - 1, 1] == 0) and np.all(V[node - 1, 1] == 0)
    assert np.abs(D[node - 1, 0]).max() > 0  # 'N' on the horizontal component


def test_dirneu_order_against_the_fault():
    text = """
&GENERAL ngll=5, fmax=10d0, ndof=2 /
&MESH_DEF method='CARTESIAN' /
&MESH_CART xlim=0d0,4d3, zlim=0d0,2d3, nelem=40,20 /
&MATERIAL tag=1, kind='ELAST' /
&MAT_ELASTIC rho=2670d0, cp=6000d0, cs=3464d0 /
&BC_DEF tag=4, kind='DIRNEU' /
&BC_DIRNEU h='N', v='D' /
&BC_DEF tag = 1, kind = 'DYNFLT' /
&BC_DYNFLT friction='SWF', Tn=-120d6, Tt=70d6 /
&BC_DYNFLT_SWF Dc=0.4d0, MuS=0.677d0, MuD=0.525d0 /
&BC_DEF tag=2, kind='ABSORB' /
&BC_DEF tag=3, kind='ABSORB' /
&BC_DEF tag=4, kind='DIRNEU' /
&BC_DIRNEU h='D' /
&TIME TotalTime=0.1d0, courant=0.5d0, kind='newmark' /
"""
    dk = deck_from_parinp(text)
    assert dk.fault.tags == (1, 0)  # one tag: a one-sided fault (bc_gen.f90:126-133)
    assert dk.dirneu == [(4, "N", "D", True), (4, "D", "N", False)]
    P = Problem(dk)
    d = P.desc()  # points into P's arrays
    n = d.ndir
    comp, after = arr(d, "dir_comp", n), arr(d, "dir_after_fault", n)
    assert set(zip(comp.tolist(), after.tolist())) == {(1, 0), (0, 1)}
    with pytest.raises(ValueError):
        deck_from_parinp(text.replace("&BC_DIRNEU h='D' /", "&BC_DIRNEU h='D', hsrc='RICKER' /"))


def periodic_box(stacey=False):
    """The corner box with its left and right sides periodic (tags 2 and 4),
    absorbing at the bottom and top."""
    dk = small_box(stacey)
    dk.absorbing = [1, 3]
    dk.stacey = [t for t in dk.stacey if t in (1, 3)]
    dk.periodic = (2, 4)
    return dk


def test_periodic_pairs_and_mass():
    Pp, P0 = Problem(periodic_box()), Problem(small_box(False))
    d, d0 = Pp.desc(), P0.desc()
    n = d.nperio
    assert n == 15 * 4 + 1
    m, s = arr(d, "perio_master", n), arr(d, "perio_slave", n)
    xz = Pp.grid.coord()
    assert np.allclose(xz[0, m - 1], 0.9e3) and np.allclose(xz[0, s - 1], -1.5e3)
    assert np.allclose(xz[1, m - 1], xz[1, s - 1])
    # BC_PERIO_init: the masses are summed and shared (bc_periodic.f90:77-88);
    # absorbing dashpots are absent on the periodic sides
    rm, rm0 = arr(d, "rmass", 2 * d.npoin), arr(d0, "rmass", 2 * d.npoin)
    np.testing.assert_array_equal(rm[m - 1], rm[s - 1])
    # away from the four sides nothing changes
    z = xz[1]
    inner = (np.abs(xz[0] + 1.5e3) > 1) & (np.abs(xz[0] - 0.9e3) > 1) & (np.abs(z + 1e3) > 1) & (np.abs(z - 0.5e3) > 1)
    np.testing.assert_array_equal(rm[:d.npoin][inner], rm0[:d.npoin][inner])
    # Stacey sides that cross the periodic ones keep their terms at both ends
    Ps = Problem(periodic_box(stacey=True))
    assert Ps.desc().nstacey == Problem(small_box(True)).desc().nstacey - 2 * 15 * 5


def test_oracle_periodic_copies_stay_equal():
    P = Problem(periodic_box())
    d = P.desc()
    d.precision = PRECISION_FP64
    o = po.OracleSim(d, owner=P)
    o.run(200)
    D, V, A = o.fields()
    m, s = arr(d, "perio_master", d.nperio) - 1, arr(d, "perio_slave", d.nperio) - 1
    assert np.abs(D[m]).max() > 0
    np.testing.assert_array_equal(D[m], D[s])
    np.testing.assert_array_equal(V[m], V[s])


def test_testflt1d_steady_slip_rate(golden):
    """EXAMPLES/TestFlt1D (periodic sides, split fault, slip weakening,
    HHT-alpha): after the slip passes Dc the 1-D fault slides at the
    steady rate 2 (Tt - MuD |Tn|) / (rho cs) = 2.2 under the stress
    MuD |Tn| (the check named for this example); from t = 2.5 s on the
    oracle's rate averages it to 0.5 % and rings within 3 % of it."""
    dk = deck_from_parinp(str(golden["parinp_TestFlt1D"]))
    assert dk.periodic == (2, 4) and dk.time.kind == "hht-alpha"
    P = Problem(dk)
    d = P.desc()
    d.precision = PRECISION_FP64
    o = po.OracleSim(d, owner=P)
    o.run(d.nt)
    f = o.fault_series()
    t = np.arange(f.shape[2]) * d.flt_oitd * d.dt
    late = t >= 2.5
    assert abs(f[0, 1, late].mean() / 2.2 - 1) < 5e-3
    np.testing.assert_allclose(f[0, 1, late], 2.2, rtol=0.03)
    np.testing.assert_allclose(f[0, 2, late], -1.1, rtol=1e-9)


def test_oracle_hht_alpha_one_is_newmark():
    """HHT-alpha with alpha = 1 is the explicit Newmark scheme (beta = 0,
    gamma = 1/2; time.f90:230-236): the oracle's two paths agree bit for
    bit, and alpha = 0.5 differs."""
    from sem2dpack_gb300.deck import Time
    out = []
    for kind, alpha in (("newmark", 1.0), ("hht-alpha", 1.0), ("hht-alpha", 0.5)):
        dk = small_box(False)
        dk.time = Time(kind=kind, nsteps=150, courant=0.3, alpha=alpha, rho=0.5)
        P = Problem(dk)
        d = P.desc()
        d.precision = PRECISION_FP64
        o = po.OracleSim(d, owner=P)
        o.run(150)
        out.append(o.seismograms())
    assert np.array_equal(out[0], out[1])
    assert np.linalg.norm(out[2] - out[0]) > 1e-6 * np.linalg.norm(out[0])


@pytest.mark.parametrize("mech", ["EXPLOSION", "DOUBLE_COUPLE", "MOMENT"])
def test_moment_source_point_forces(mech):
    """Moment sources (SRC_MOMENT_init/add, src_moment.f90:118-175) become
    point forces on the rows and columns through the source node of every
    element holding it: they sum to zero and their first moment is
    (elements holding the node) x M, since sum_l x_l h'_l = dx/dxi."""
    dk = small_box(False)
    dk.sources.mechanism = mech
    dk.sources.dip = 60.0
    dk.sources.M = (1.0, 0.3, 0.3, -0.5)
    dk.sources.coords = [(-1100.0, -700.0)]  # a node shared by four elements
    P = Problem(dk)
    d = P.desc()
    n = d.nsrc
    node = arr(d, "src_node", n) - 1
    F = arr(d, "src_dir", 2 * n).reshape(n, 2)
    xz = P.grid.coord()
    np.testing.assert_allclose(F.sum(axis=0), 0.0, atol=1e-15)
    first = np.array([[np.sum(F[:, c] * xz[dd, node]) for dd in range(2)] for c in range(2)])
    if mech == "EXPLOSION":
        M = np.eye(2)
    elif mech == "DOUBLE_COUPLE":
        dip = np.radians(60.0)
        nv, r = np.array([np.sin(dip), np.cos(dip)]), np.array([-np.cos(dip), np.sin(dip)])
        M = np.outer(r, nv) + np.outer(nv, r)
    else:
        M = np.array([[1.0, 0.3], [0.3, -0.5]])
    np.testing.assert_allclose(first, 4 * M, rtol=1e-12, atol=1e-12)
    d.precision = PRECISION_FP64
    o = po.OracleSim(d, owner=P)
    o.run(100)
    assert np.isfinite(o.seismograms()).all() and np.abs(o.seismograms()).max() > 0


def test_moment_source_parinp():
    text = """
&GENERAL ngll=5, fmax=10d0, ndof=2 /
&MESH_DEF method='CARTESIAN' /
&MESH_CART xlim=0d0,4d3, zlim=0d0,2d3, nelem=40,20 /
&MATERIAL tag=1, kind='ELAST' /
&MAT_ELASTIC rho=2670d0, cp=6000d0, cs=3464d0 /
&TIME TotalTime=0.2d0, courant=0.5d0 /
&SRC_DEF stf='RICKER', mechanism='MOMENT', coord=2d3,1d3 /
&STF_RICKER f0=10d0, onset=0.1d0, ampli=1d0 /
&SRC_MOMENT Mxx=1d0, Mxz=0d0, Mzx=0d0, Mzz=-1d0 /
"""
    d = deck_from_parinp(text)
    assert d.sources.mechanism == "MOMENT" and d.sources.M == (1.0, 0.0, 0.0, -1.0)
    P = Problem(d)
    # the element corner at the source: a 9-node line across two elements in
    # x and one in z, sharing the node
    assert P.desc().nsrc == 9 + 9 - 1

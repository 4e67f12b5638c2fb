"""Product host builder (C++) against the oracle's restated init_main.

Integer data (ibool, boundary tables, node pairs) must be bit-exact; the
floating-point arrays of the descriptor are compared bit-exactly too, since
both follow the reference's operation order in FP64 without contraction.
"""
import numpy as np
import pytest

import decks
from oracle import pyoracle as po
from sem2dpack_gb300 import Grid, Problem, abi, workloads
from sem2dpack_gb300.deck import Stf

INT_FIELDS = ["ibool", "abs_node", "src_node", "rec_node", "rec_elem", "flt_node1", "flt_node2"]


def _arr(d, name, n):
    p = getattr(d, name)
    if not p:
        return None
    return np.ctypeslib.as_array(p, shape=(n,)).copy()


def _sizes(d):
    n2, ne, npn, nd = d.ngll * d.ngll, d.nelem, d.npoin, d.ndof
    return {"ibool": n2 * ne, "coord": 2 * npn, "hprime": n2, "wgll": d.ngll, "Kx": n2 * ne,
            "Kz": n2 * ne, "la": n2 * ne, "mu": n2 * ne, "mux": n2 * ne, "rmass": npn * nd,
            "abs_node": d.nabs, "abs_C": d.nabs * nd, "src_node": d.nsrc, "src_dir": 2 * d.nsrc,
            "src_f0": d.nsrc, "src_t0": d.nsrc, "src_ampli": d.nsrc, "src_relamp": d.nsrc,
            "rec_node": d.nrec, "rec_elem": d.nrec, "rec_interp": n2 * d.nrec,
            "flt_node1": d.nflt, "flt_node2": d.nflt, "flt_n1": 2 * d.nflt, "flt_B": d.nflt,
            "flt_invM1": d.nflt * nd, "flt_invM2": d.nflt * nd, "flt_Z": d.nflt * nd,
            "flt_T0": 2 * d.nflt, "flt_cohesion": d.nflt, "swf_dc": d.nflt, "swf_mus": d.nflt,
            "swf_mud": d.nflt, "rsf_a": d.nflt, "rsf_b": d.nflt, "rsf_theta": d.nflt,
            "flt_V0": d.nflt}


def _stf_fields(p):
    if not p:
        return None
    s = p.contents
    out = [s.kind, s.ntab, s.f0, s.onset, s.ampli, s.par1, s.par2]
    if s.ntab:
        out += list(np.ctypeslib.as_array(s.tab_t, shape=(s.ntab,)))
        out += list(np.ctypeslib.as_array(s.tab_v, shape=(s.ntab,)))
    return out


def assert_same_desc(a, b):
    for attr in ("ngll", "ndof", "nelem", "npoin", "nabs", "nt", "nsrc", "nrec", "rec_nsamp",
                 "rec_isamp", "nflt", "flt_nsamp", "flt_oit", "flt_oitd", "flt_oix1", "flt_oixn",
                 "kd2_form", "time_scheme", "wave_phase", "nneu", "nneu_stf"):
        assert getattr(a, attr) == getattr(b, attr), attr
    assert a.dt == b.dt and a.flt_coefA2V == b.flt_coefA2V
    for attr in ("wave_angle", "wave_cp", "wave_cs", "wave_mu", "wave_lambda", "wave_tdelay"):
        assert getattr(a, attr) == getattr(b, attr), attr
    assert list(a.wave_ref) == list(b.wave_ref)
    assert _stf_fields(a.src_stf) == _stf_fields(b.src_stf)
    assert _stf_fields(a.wave_stf) == _stf_fields(b.wave_stf)
    for k in range(a.nneu_stf):
        sa, sb = abi.P_Stf(a.neu_stfs[k]), abi.P_Stf(b.neu_stfs[k])
        assert _stf_fields(sa) == _stf_fields(sb), k
    sizes = _sizes(a)
    sizes.update({"abs_B": a.nabs, "abs_n": 2 * a.nabs, "abs_wave": a.nabs, "neu_node": a.nneu,
                  "neu_comp": a.nneu, "neu_B": a.nneu, "neu_stf": a.nneu,
                  "xjaci": 4 * a.ngll * a.ngll * a.nelem, "dvol": a.ngll * a.ngll * a.nelem})
    for name, n in sizes.items():
        x, y = _arr(a, name, n), _arr(b, name, n)
        assert (x is None) == (y is None), name
        if x is not None:
            assert np.array_equal(x, y), name


@pytest.mark.parametrize("name", ["lambs_problem", "test_sh", "inabox", "anisotropic"])
def test_grid_bit_exact(name):
    dk = getattr(decks, name)()
    g, o = Grid(dk), po.OracleSetup(dk, grid_only=True)
    assert (g.nelem, g.npoin) == (o.nelem, o.npoin)
    assert np.array_equal(g.ibool(), o.ibool())
    assert np.array_equal(g.coord(), o.coord())
    assert np.array_equal(g.tags(), o.tags())
    for t in (1, 2, 3, 4):
        assert np.array_equal(g.boundary(t), o.boundary(t))


@pytest.mark.parametrize("name", ["lambs_problem", "test_sh", "inabox"])
def test_problem_bit_exact(name):
    dk = getattr(decks, name)()
    P, O = Problem(dk), po.OracleSetup(dk)
    assert_same_desc(P.desc(), O.desc())


def test_fault_problem_bit_exact():
    dk, g = workloads.sh_rupture(scale=0.1, nsteps=200)
    P = Problem(dk, g)
    O = po.OracleSetup(dk)
    assert_same_desc(P.desc(), O.desc())
    # split rows: every fault node pair is distinct and sorted along x
    d = P.desc()
    n1 = _arr(d, "flt_node1", d.nflt)
    n2 = _arr(d, "flt_node2", d.nflt)
    assert np.all(n1 != n2)
    x = g.coord()[0, n1 - 1]
    assert np.all(np.diff(x) > 0)


def test_fault_before_absorbing_order():
    """&BC_DEF order decides whether the fault snapshots the mass before or
    after the absorbing fold (bc_gen.f90:229-246)."""
    dk, g = workloads.sh_rupture(scale=0.1, nsteps=50)
    Pa = Problem(dk, g)
    a = Pa.desc()
    dk.fault_first = True
    Pb = Problem(dk, g)
    b = Pb.desc()
    inv_a, inv_b = _arr(a, "flt_invM1", a.nflt), _arr(b, "flt_invM1", b.nflt)
    # the end nodes lie on the absorbing sides: only they differ
    diff = np.nonzero(inv_a != inv_b)[0]
    assert set(diff.tolist()) == {0, a.nflt - 1}
    O = po.OracleSetup(dk)
    assert_same_desc(b, O.desc())


@pytest.mark.parametrize("atnode", [True, False])
def test_receivers(atnode):
    dk = workloads.plain_psv(scale=0.1, nsteps=10, nrec=5)
    dk.receivers.atnode = atnode
    P, O = Problem(dk), po.OracleSetup(dk)
    assert_same_desc(P.desc(), O.desc())
    np.testing.assert_array_equal(P.rec_coord(), O.rec_coord())


def test_reference_warnings_abort():
    """Warnings abort by default in the reference (stdio.f90:13,218-227)."""
    from sem2dpack_gb300 import Sem2dError
    dk = workloads.plain_psv(scale=0.1, nsteps=10)
    dk.fmax = 1000.0  # resolution warning (init.f90:271-281)
    with pytest.raises(Sem2dError):
        Problem(dk)
    dk = workloads.plain_psv(scale=0.1, nsteps=10)
    dk.sources.onset = 0.05  # onset < 1/f0 (stf_ricker.f90:63-68)
    with pytest.raises(Sem2dError):
        Problem(dk)


def test_hht_alpha_problem_bit_exact():
    """&TIME kind='HHT-alpha' + &TIME_HHTA (time.f90:222-240): gamma = 3/2 -
    alpha, beta from alpha and rho, the absorbing fold with alpha gamma dt
    (TIME_getCoefA2Vrhs, time.f90:467-486), on a fault deck."""
    from sem2dpack_gb300.deck import Time
    dk, g = workloads.sh_rupture(scale=0.1, nsteps=200)
    dk.time = Time(kind="hht-alpha", nsteps=200, courant=0.5, alpha=0.7, rho=0.7)
    P = Problem(dk, g)
    O = po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    assert (a.alpha, a.beta, a.gamma) == (b.alpha, b.beta, b.gamma)
    assert a.alpha == 0.7 and abs(a.gamma - 0.8) < 1e-15
    r = 0.7
    assert abs(a.beta - (1 - 0.7 - r * r * (r - 1) / (0.3 * (1 + r) ** 3))) < 1e-15
    assert a.flt_coefA2D == a.beta * a.dt ** 2
    dk.time.alpha = 1.5
    with pytest.raises(Exception):
        Problem(dk, g)


def test_stacey_problem_bit_exact():
    """The Stacey P3 terms (BC_ABSO_init, bc_abso.f90:174-218): the product
    builder and the oracle's restated setup agree bit for bit."""
    dk = decks.test_abso(-1.0e3, 12, True)
    dk.ngll, dk.fmax, dk.nelem = 5, 20.0, (24, 15)
    dk.xlim, dk.zlim = (-1.5e3, 0.9e3), (-1.0e3, 0.5e3)
    dk.sources.coords = [(-1100.0, -700.0)]
    dk.sources.f0, dk.sources.onset = 10.0, 0.1
    dk.receivers.first, dk.receivers.last = (-1500.0, -1000.0), (900.0, -1000.0)
    dk.receivers.number = 25
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    n = a.nstacey
    assert n == b.nstacey == (2 * 24 + 2 * 15) * 5
    for name, m in (("stacey_node", n), ("stacey_k", n), ("stacey_edge", 5 * n), ("stacey_K", 2 * n)):
        assert np.array_equal(_arr(a, name, m), _arr(b, name, m)), name


@pytest.mark.parametrize("case", ["periodic", "periodic_fault", "dirneu", "periodic_bt_stacey", "periodic_lr_stacey"])
def test_periodic_and_dirichlet_bit_exact(case):
    """BC_PERIO_init (summed mass, boundary weights and dashpots at the ends
    of crossing sides) and BC_DIRNEU_init: the product builder and the
    oracle's restated setup agree bit for bit."""
    if case == "periodic_fault":
        dk, _ = workloads.sh_rupture(scale=0.1, nsteps=50)
        dk.absorbing = [1, 3]
        dk.periodic = (2, 4)
    else:
        dk = decks.inabox()
        dk.time.total_time, dk.time.nsteps = 0.0, 50
        if case == "periodic":
            dk.absorbing = [1, 3]
            dk.periodic = (2, 4)
        elif case == "periodic_bt_stacey":  # as EXAMPLES/TestAbso/Par.inp
            dk.absorbing, dk.stacey = [2, 4], [2, 4]
            dk.periodic = (1, 3)
        elif case == "periodic_lr_stacey":
            dk.absorbing, dk.stacey = [1, 3], [1, 3]
            dk.periodic = (2, 4)
        else:
            dk.absorbing = [1, 2, 3]
            dk.dirneu = [(4, "N", "D", True)]
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    assert (a.nperio, a.ndir) == (b.nperio, b.ndir)
    for name, m in (("perio_master", a.nperio), ("perio_slave", a.nperio), ("dir_node", a.ndir),
                    ("dir_comp", a.ndir), ("dir_after_fault", a.ndir)):
        if m:
            assert np.array_equal(_arr(a, name, m), _arr(b, name, m)), name
    assert (a.nperio > 0) == (case != "dirneu") and (a.ndir > 0) == (case == "dirneu")
    if "stacey" in case:
        assert a.nstacey == b.nstacey > 0
        for name, m in (("stacey_node", a.nstacey), ("stacey_k", a.nstacey), ("stacey_K", 2 * a.nstacey)):
            assert np.array_equal(_arr(a, name, m), _arr(b, name, m)), name


@pytest.mark.parametrize("mech,ndof", [("EXPLOSION", 2), ("DOUBLE_COUPLE", 2), ("MOMENT", 2), ("MOMENT", 1),
                                       ("DOUBLE_COUPLE", 1)])
def test_moment_sources_bit_exact(mech, ndof):
    """Moment sources as point forces (src_moment.f90:27-175): builder and
    the oracle's restated setup agree bit for bit."""
    dk = decks.inabox()
    dk.ndof = ndof
    dk.time.total_time, dk.time.nsteps = 0.0, 50
    dk.sources.mechanism, dk.sources.dip, dk.sources.M = mech, 35.0, (1.0, 0.2, 0.3, -0.6)
    dk.sources.coords = [(0.0, 0.0), (125.0, -310.0)]
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert a.nsrc == b.nsrc > 2
    assert_same_desc(a, b)


@pytest.mark.parametrize("ndof,phase,angle", [(1, "S", 0.0), (1, "P", 30.0), (2, "P", 0.0), (2, "S", -45.0),
                                              (2, "P", 150.0), (2, "S", 200.0)])
def test_wave_problem_bit_exact(ndof, phase, angle):
    """Incident plane wave (src_wave.f90): boundary weights, normals, the
    entries it enters and its reference point and material, product
    builder against the oracle's restatement."""
    dk = decks.wave_box(ndof, phase, angle, tdelay=0.01)
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    assert a.nsrc == 0 and a.wave_phase == (abi.WAVE_P if phase == "P" else abi.WAVE_S)
    assert -180.0 <= a.wave_angle <= 180.0 and a.wave_tdelay == 0.01
    # the reference point: the corner the wave reaches first
    ang = (angle + 180.0) % 360.0 - 180.0
    assert list(a.wave_ref) == [2000.0 if ang >= 0 else 0.0, 0.0 if abs(ang) < 90 else 1000.0]
    assert a.wave_mu == 2500.0 * 2887.0 ** 2
    n = a.nabs
    wave = np.ctypeslib.as_array(a.abs_wave, shape=(n,))
    assert wave.all()
    B = np.ctypeslib.as_array(a.abs_B, shape=(n,))
    nrm = np.ctypeslib.as_array(a.abs_n, shape=(2 * n,)).reshape(2, n)
    assert np.allclose(np.hypot(nrm[0], nrm[1]), 1.0)
    # the weights of a side add up to its length
    assert np.isclose(B.sum(), 2 * 2000.0 + 2 * 1000.0)


def test_wave_let_wave_false_and_periodic():
    dk = decks.wave_box(2, "P", 0.0, periodic=True, no_wave=[3])
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    n = a.nabs
    wave = np.ctypeslib.as_array(a.abs_wave, shape=(n,))
    xz = P.grid.coord()
    node = np.ctypeslib.as_array(a.abs_node, shape=(n,)) - 1
    assert wave[xz[1, node] < 1.0].all() and not wave[xz[1, node] > 999.0].any()


@pytest.mark.parametrize("kind", ["GAUSSIAN", "BRUNE", "HARMONIC", "USER", "TAB"])
def test_source_time_functions_bit_exact(kind):
    dk = decks.lambs_problem()
    dk.nelem, dk.fmax = (20, 10), 8.0
    t = np.linspace(0.0, 0.5, 11)
    dk.sources.stf = Stf(kind, f0=10.1, onset=0.15, ampli=1.3, par1=0.7, par2=0.2,
                         tab=(t, np.sin(20 * t)) if kind == "TAB" else None)
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    s = a.src_stf.contents
    assert s.kind == abi.STF_KINDS[kind]
    # the REAL namelist variables of the reference hold FP32 values
    if kind in ("GAUSSIAN", "HARMONIC"):
        assert s.f0 == float(np.float32(10.1))
    if kind == "BRUNE":
        assert s.f0 == 10.1


def test_traction_problem_bit_exact():
    dk = decks.traction_box(2, hstf=Stf("GAUSSIAN", f0=8.0, onset=0.1, ampli=1e6),
                            vstf=Stf("RICKER", f0=10.0, onset=0.12, ampli=2e6))
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    assert a.nneu_stf == 2 and a.nneu == 2 * (20 * 4 + 1)
    comp = np.ctypeslib.as_array(a.neu_comp, shape=(a.nneu,))
    B = np.ctypeslib.as_array(a.neu_B, shape=(a.nneu,))
    assert np.isclose(B[comp == 0].sum(), 2000.0) and np.isclose(B[comp == 1].sum(), 2000.0)
    # a Dirichlet component drops its time function (bc_dirneu.f90:70-101)
    dk = decks.traction_box(2, hstf=Stf("GAUSSIAN", f0=8.0, onset=0.1, ampli=1e6),
                            vstf=Stf("RICKER", f0=10.0, onset=0.12, ampli=2e6), v="D")
    P, O = Problem(dk), po.OracleSetup(dk)
    a, b = P.desc(), O.desc()
    assert_same_desc(a, b)
    assert a.nneu_stf == 1 and a.ndir == 20 * 4 + 1

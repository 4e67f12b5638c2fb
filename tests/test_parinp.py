"""Par.inp front end (sem2dpack_gb300.parinp) and the reference-format
output writers (sem2dpack_gb300.outputs), on the CPU.

The reference's own example decks (text fixtures from
tests/golden/make_golden.py) parse to the decks tests/decks.py restates by
hand; the writers' files read back bit-for-bit in the layout the
reference's readers expect (direct-access FP32 traces, Fortran sequential
records with 4-byte markers)."""
import os

import numpy as np
import pytest

import decks
from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, Problem, workloads
from sem2dpack_gb300 import outputs
from sem2dpack_gb300.parinp import deck_from_parinp, read_namelists

EXAMPLES = {"LambsProblem": decks.lambs_problem, "TestSH": decks.test_sh,
            "Anisotropic": decks.anisotropic, "InaBox": decks.inabox}


def same_deck(a, b):
    for f in ("ngll", "ndof", "fmax", "xlim", "zlim", "nelem", "absorbing", "domains", "materials",
              "ezflt", "width"):
        assert getattr(a, f) == getattr(b, f), f
    assert vars(a.time) == vars(b.time)
    for f in ("sources", "receivers"):
        x, y = getattr(a, f), getattr(b, f)
        assert (x is None) == (y is None), f
        if x is not None:
            assert vars(x) == vars(y), f


@pytest.mark.parametrize("name", list(EXAMPLES))
def test_example_decks_parse_to_the_restated_decks(name, golden):
    d = deck_from_parinp(str(golden["parinp_" + name]))
    same_deck(d, EXAMPLES[name]())
    assert all(s.startswith(("SNAP", "SRC_")) for s in d.skipped)


def test_example_deck_builds_the_same_problem(golden):
    pa, pb = Problem(deck_from_parinp(str(golden["parinp_TestSH"]))), Problem(decks.test_sh())
    a, b = pa.desc(), pb.desc()  # the descriptors point into the problems' arrays
    assert (a.nelem, a.npoin, a.nt, a.dt) == (b.nelem, b.npoin, b.nt, b.dt)
    n = a.npoin
    assert np.array_equal(np.ctypeslib.as_array(a.rmass, shape=(n,)), np.ctypeslib.as_array(b.rmass, shape=(n,)))


def test_namelist_reader():
    text = """
    # comment &NOT_A_BLOCK x=1 /
    &ONE a=1.5d3, b = -2.d-1 , s='x/y' , t=T, f=.false., v=1,2,3, r=3*0.5 / trailing, k='ignored' /
    &TWO name = "q" ! comment
         n=4 /
    """
    b = read_namelists(text)
    assert [n for n, _ in b] == ["ONE", "TWO"]
    one = b[0][1]
    assert one == {"a": 1500.0, "b": -0.2, "s": "x/y", "t": True, "f": False, "v": [1, 2, 3],
                   "r": [0.5, 0.5, 0.5]}
    assert b[1][1] == {"name": "q", "n": 4}


@pytest.mark.parametrize("bad", [
    "&MESH_DEF method='MESH2D' /",
    "&BC_DEF tags=1,3, kind='KINFLT' /",
    "&TIME kind='hhta' /",
    "&SRC_DEF stf='BUTTERWORTH', coord=0,0, mechanism='FORCE' /",
    "&SRC_DEF stf='RICKER', coord=0,0, mechanism='WAVE' / &STF_RICKER f0=1, onset=2 /",
    "&MATERIAL tag=1, kind='PLAST' /",
    "&BC_DEF tags=5,6, kind='DYNFLT' / &BC_DYNFLT TtH='PWCONR' /",
    "&BC_DEF tags=5,6, kind='DYNFLT' / &BC_DYNFLT_SWF MuSH='LINEAR' /",
])
def test_off_path_blocks_are_refused(bad):
    with pytest.raises(ValueError):
        deck_from_parinp(bad)


FAULT_PARINP = """
&GENERAL ngll=5, fmax=10d0, ndof=1 /
&MESH_DEF method='CARTESIAN' /
&MESH_CART xlim=0d0,4d3, zlim=0d0,2d3, nelem=40,20, ezflt=-1 /
&MATERIAL tag=1, kind='ELAST' /
&MAT_ELASTIC rho=2670d0, cp=6000d0, cs=3464d0 /
&BC_DEF tags=5,6, kind='DYNFLT' /
&BC_DYNFLT friction='SWF', Tn=-120d6, Tt=70d6, otd=0.01d0 /
&BC_DYNFLT_SWF Dc=0.4d0, MuS=0.677d0, MuD=0.525d0 /
&BC_DEF tag=1, kind='ABSORB' /
&BC_DEF tag=3, kind='ABSORB' /
&TIME TotalTime=0.2d0, courant=0.5d0 /
&REC_LINE number=5, first=500d0,1500d0, last=3500d0,1500d0 /
"""


def test_fault_deck():
    d = deck_from_parinp(FAULT_PARINP)
    assert d.fault is not None and d.fault.friction == "SWF" and d.fault_first
    assert d.fault.values == {"Tn": -120e6, "Tt": 70e6, "swf_dc": 0.4, "swf_mus": 0.677, "swf_mud": 0.525}
    assert d.fault.otd == 0.01 and d.absorbing == [1, 3] and d.ezflt == -1
    P = Problem(d)
    desc = P.desc()
    assert desc.nflt == 4 * 40 + 1 and desc.flt_node2


def test_seismogram_files_round_trip(tmp_path):
    P = Problem(workloads.plain_psv(scale=0.05, nsteps=40))
    d = P.desc()
    d.precision = PRECISION_FP64
    o = po.OracleSim(d, owner=P)
    o.run(40)
    sis = o.seismograms()
    coords = P.rec_coord()
    outputs.write_seismograms(str(tmp_path), sis, d.rec_isamp * d.dt, coords)
    assert os.path.getsize(tmp_path / "Ux_sem2d.dat") == 4 * sis.shape[0] * sis.shape[1]
    back, tsamp, xz = outputs.read_seismograms(str(tmp_path), 2)
    assert np.array_equal(back, sis.astype(np.float32))
    assert tsamp == pytest.approx(d.rec_isamp * d.dt, rel=1e-6)
    np.testing.assert_allclose(xz, coords, rtol=1e-15)
    # record k holds receiver k's samples (the reference's direct access)
    raw = np.fromfile(tmp_path / "Uz_sem2d.dat", dtype="<f4").reshape(sis.shape[1], sis.shape[0])
    assert np.array_equal(raw[3], sis[:, 3, 1].astype(np.float32))


def test_fault_files_round_trip(tmp_path):
    P = Problem(deck_from_parinp(FAULT_PARINP))
    d = P.desc()
    o = po.OracleSim(d, owner=P)
    o.run(60)
    series = o.fault_series()
    xz = P.fault_coord()
    onx = series.shape[0]
    cxz = xz[:, (d.flt_oix1 - 1):(d.flt_oixn):d.flt_oixd] if xz.shape[1] != onx else xz
    outputs.write_fault(str(tmp_path), 5, series, d.flt_oitd * d.dt, cxz)
    back, odt, bxz = outputs.read_fault(str(tmp_path), 5)
    assert np.array_equal(back, series.astype(np.float32))
    assert odt == pytest.approx(d.flt_oitd * d.dt, rel=1e-12)
    assert (tmp_path / "Flt05_sem2d.csh").exists()
    pot = o.fault_potency()
    outputs.write_potency(str(tmp_path), 5, pot, 1)
    lines = open(tmp_path / "Flt05_potency_sem2d.tab").read().splitlines()
    assert len(lines) == d.nt + 1 and len(lines[0]) == 4 * 24
    v = [float(x.replace("D", "E")) for x in lines[40].split()]
    np.testing.assert_allclose(v, [pot[40, 0, 0], pot[40, 0, 1], pot[40, 1, 0], pot[40, 1, 1]], rtol=1e-15)


def test_grid_files_round_trip(tmp_path):
    P = Problem(deck_from_parinp(FAULT_PARINP))
    g = P.grid
    outputs.write_grid(str(tmp_path), g)
    sizes, ib, xz = outputs.read_grid(str(tmp_path))
    # 40 x 20 elements, the fault splits the corner rows: 41 x 22 geometric nodes
    assert sizes == {"NELEM": 800, "NPGEO": 41 * 22, "NGNOD": 4, "NPOIN": g.npoin, "NGLL": 5}
    assert np.array_equal(ib, g.ibool()) and ib.min() == 1 and ib.max() == g.npoin
    assert np.array_equal(xz, g.coord().astype(np.float32))
    # record e of ibool_sem2d.dat is element e's NGLL x NGLL table, i fastest
    raw = np.fromfile(tmp_path / "ibool_sem2d.dat", dtype="<i4")
    assert os.path.getsize(tmp_path / "ibool_sem2d.dat") == 4 * 25 * 800
    assert np.array_equal(raw[25 * 7:25 * 8], g.ibool()[:, :, 7].ravel(order="F"))


def test_tpv3_inplane_deck_with_distributions(golden):
    """EXAMPLES/TestFlt2D_SCEC_TPV3_inplane/Par.inp: TtH and MuSH as
    &DIST_PWCONR rings, the Kelvin-Voigt eta as a &DIST_GAUSSIAN band along
    the fault, a one-sided fault on the bottom side and v = 'D' on the left."""
    d = deck_from_parinp(str(golden["parinp_TestFlt2D_SCEC_TPV3_inplane"]))
    assert (d.ngll, d.ndof, d.nelem) == (6, 2, (70, 40))
    assert d.fault.tags == (1, 0) and d.dirneu == [(4, "N", "D", False)] and d.absorbing == [2, 3]
    assert d.time.kind == "newmark" and d.receivers.atnode is False and d.fault.oxi == (1, 65, 4)
    from sem2dpack_gb300.api import Grid
    g = Grid(d)
    n1, _ = g.fault_nodes()
    x = g.coord()[0, n1 - 1]
    np.testing.assert_array_equal(d.fault.values["Tt"], np.where(x <= 1.5e3, 81.6e6, 70.0e6))
    np.testing.assert_array_equal(d.fault.values["swf_mus"], np.where(x <= 15e3, 0.677, 1e4))
    ib = g.ibool() - 1
    z = g.coord()[1][ib]
    xx = g.coord()[0][ib]
    np.testing.assert_allclose(d.hetero["kveta"], 0.1 * np.exp(-((xx / 1e6) ** 2 + (z / 282.094) ** 2)), rtol=1e-15)
    assert np.all(d.hetero["rho"] == 2670.0) and d.materials[0].hetero
    P = Problem(d)
    desc = P.desc()
    assert desc.nflt == 70 * 5 + 1 and desc.ndir == 40 * 5 + 1


def test_distributions(tmp_path):
    from sem2dpack_gb300.distributions import Dist
    x = np.array([-3.0, -1.0, 0.0, 0.5, 2.0, 5.0])
    z = np.array([0.0, 1.0, -2.0, 0.5, 3.0, -1.0])
    d = Dist("PWCONR", {"num": 3, "ref": [1.0, 0.0]}, [1.0, 3.0, 10.0, 20.0, 30.0])
    r = np.hypot(x - 1.0, z)
    np.testing.assert_array_equal(d(x, z), np.where(r <= 1, 10.0, np.where(r <= 3, 20.0, 30.0)))
    d = Dist("ORDER0", {"xn": 2, "zn": 2}, [0.0, 0.5, 1.0, 2.0, 3.0, 4.0])
    np.testing.assert_array_equal(d(x, z), np.where(z < 0.5, np.where(x < 0, 1.0, 2.0), np.where(x < 0, 3.0, 4.0)))
    d = Dist("LINEAR", {"n": 3, "dim": 2}, [0.0, 1.0, 1.0, 3.0, 2.0, 4.0])
    np.testing.assert_allclose(d(x, z), np.interp(z, [0, 1, 2], [1, 3, 4]) + np.where(z < 0, 2 * z, 0)
                               + np.where(z > 2, (z - 2) * 1.0, 0), rtol=1e-15)
    d = Dist("LINEAR", {"n": 2, "dim": 1, "length": 2.0}, [0.0, 0.0, 1.0, 1.0])
    np.testing.assert_allclose(d(x, z), x, rtol=1e-13)  # the average of a line over a window is its centre value
    d = Dist("GAUSSIAN", {"centered_at": [1.0, -1.0], "length": [2.0, 0.5], "offset": 3.0, "ampli": 2.0,
                          "order": 2}, [])
    np.testing.assert_allclose(d(x, z), 3 + 2 * np.exp(-(((x - 1) / 2) ** 2 + ((z + 1) / 0.5) ** 2) ** 2))
    (tmp_path / "line.tab").write_text("-10 0\n10 0\n")
    d = Dist("GRADIENT", {"file": "line.tab", "grad": -2.0, "valref": 5.0}, [], base=str(tmp_path))
    np.testing.assert_allclose(d(x, z), 5.0 + 2.0 * (0.0 - z))
    with pytest.raises(ValueError):
        Dist("HETE1", {}, [])
    # SPLINE: the clamped cubic spline through the sorted table
    from scipy.interpolate import CubicSpline
    t = np.array([3.0, -2.0, 0.5, 1.0, -1.0, 2.2])
    v = np.sin(t)
    (tmp_path / "sp.tab").write_text("".join("%r %r\n" % (float(a), float(b)) for a, b in zip(t, v)))
    d = Dist("SPLINE", {"file": "sp.tab"}, [], base=str(tmp_path))
    xs = np.linspace(-2.0, 3.0, 57)
    o = np.argsort(t)
    np.testing.assert_allclose(d(xs, 0 * xs), CubicSpline(t[o], v[o], bc_type=((1, 0.0), (1, 0.0)))(xs),
                               rtol=1e-12, atol=1e-14)
    with pytest.raises(ValueError):
        d(np.array([3.5]), np.array([0.0]))


def test_snapshot_files(tmp_path):
    """Snapshot files of D, V, A, strain and stress written from an oracle
    run, read back in the reference's layouts."""
    P = Problem(workloads.plain_psv(scale=0.05, nsteps=40))
    d = P.desc()
    d.precision = PRECISION_FP64
    o = po.OracleSim(d, owner=P)
    o.run(40)

    class Run:  # the getters write_snapshot calls, over the oracle
        desc = d

        def fields(self, accel=False):
            f = o.fields()
            return f if accel else f[:2]

        def strain_stress(self):
            return o.strain_stress()

    outputs.write_snapshot(str(tmp_path), Run(), 3, "DVAES")
    D, V, A = o.fields()
    for c, arr in (("d", D), ("v", V), ("a", A)):
        for k, comp in enumerate("xz"):
            back = np.fromfile(tmp_path / ("%s%s_003_sem2d.dat" % (c, comp)), dtype="<f4")
            assert np.array_equal(back, arr[:, k].astype(np.float32))
    e, s = o.strain_stress()
    N, ne = d.ngll, d.nelem
    for pre, arr in (("e", e), ("s", s)):
        for k, nm in enumerate(("11", "22", "12")):
            raw = np.fromfile(tmp_path / ("%s%s_003_sem2d.dat" % (pre, nm)), dtype="<f4").reshape(ne, N * N)
            assert np.array_equal(raw[5], arr[:, :, k, 5].ravel(order="F").astype(np.float32))
    with pytest.raises(ValueError):
        outputs.write_snapshot(str(tmp_path), Run(), 4, "Vc")  # div/curl need the grid
    with pytest.raises(ValueError):
        outputs.write_snapshot(str(tmp_path), Run(), 4, "Vx")


def test_divcurl_snapshot_of_a_linear_velocity(tmp_path):
    """div and curl of v = (a x + b z, c x + e z) are a + e and b - c at
    every GLL point (MAT_divcurl_PSV, mat_gen.f90:802-825)."""
    P = Problem(workloads.plain_psv(scale=0.05, nsteps=10))
    d = P.desc()
    xz = P.grid.coord()
    a, b, c, e = 1.5e-3, -0.7e-3, 0.4e-3, 2.1e-3
    v = np.stack([a * xz[0] + b * xz[1], c * xz[0] + e * xz[1]], axis=1)

    class Run:
        desc = d

        def fields(self, accel=False):
            return np.zeros_like(v), v

    outputs.write_snapshot(str(tmp_path), Run(), 2, "dc", grid=P.grid)
    div = np.fromfile(tmp_path / "div_002_sem2d.dat", dtype="<f4")
    curl = np.fromfile(tmp_path / "curl_002_sem2d.dat", dtype="<f4")
    assert div.size == curl.size == d.ngll ** 2 * d.nelem
    np.testing.assert_allclose(div, a + e, rtol=1e-5)
    np.testing.assert_allclose(curl, b - c, rtol=1e-5)


def test_sh_snapshot_skips_div_curl(tmp_path):
    """An SH problem has no divergence or curl: asked for them, the writer
    skips them as the reference does (plot_gen.f90:100) and writes the rest."""
    P = Problem(workloads.sh_rupture(scale=0.05, nsteps=10)[0])
    d = P.desc()
    v = np.ones((d.npoin, 1))

    class Run:
        desc = d

        def fields(self, accel=False):
            return np.zeros_like(v), v

    outputs.write_snapshot(str(tmp_path), Run(), 1, "Vdc")
    assert (tmp_path / "vy_001_sem2d.dat").exists()
    assert not (tmp_path / "div_001_sem2d.dat").exists()
    assert not (tmp_path / "curl_001_sem2d.dat").exists()


def test_hht_alpha_time_block():
    d = deck_from_parinp("&TIME TotalTime=1d0, courant=0.3d0, kind='HHT-alpha' / &TIME_HHTA alpha=0.6d0, rho=0.9d0 /")
    assert (d.time.kind, d.time.alpha, d.time.rho) == ("hht-alpha", 0.6, 0.9)


def test_every_example_deck_is_taken_or_refused(golden, tmp_path):
    """Each of the reference's example decks either builds (16, run on the
    GPU by test_gpu_examples.py) or is refused with a ValueError naming the
    block off the GPU path (14)."""
    from conftest import example_deck
    taken = [k for k in golden.files if k.startswith("parinp_")]
    refused = [k for k in golden.files if k.startswith("refused_")]
    assert len(taken) == 16 and len(refused) == 14
    for k in taken:
        P = Problem(example_deck(golden, k[len("parinp_"):], tmp_path))
        assert P.desc().npoin > 0, k
    for k in refused:
        # (two SiteEffects decks name a layer file that the fixtures do not
        # hold; with it their IWAN material is refused)
        with pytest.raises((ValueError, OSError)):
            deck_from_parinp(str(golden[k]))


def test_source_and_receiver_files(tmp_path):
    """&SRC_DEF file (x, z [, delay [, relative amplitude]] per line,
    src_gen.f90:70-79) and &REC_LINE file (x z per line, receivers.f90:
    43-44), read relative to the Par.inp."""
    (tmp_path / "src.tab").write_text("1000 1000 0.0 1.0\n3000 1200 0.05 0.5\n")
    (tmp_path / "rec.tab").write_text("500 1500\n1500 1500\n2500 1500\n")
    text = """
&GENERAL ngll=5, fmax=10d0, ndof=2 /
&MESH_DEF method='CARTESIAN' /
&MESH_CART xlim=0d0,4d3, zlim=0d0,2d3, nelem=40,20 /
&MATERIAL tag=1, kind='ELAST' /
&MAT_ELASTIC rho=2670d0, cp=6000d0, cs=3464d0 /
&TIME TotalTime=0.2d0, courant=0.5d0 /
&SRC_DEF stf='RICKER', mechanism='FORCE', file='src.tab' /
&STF_RICKER f0=10d0, onset=0.1d0, ampli=1d0 /
&SRC_FORCE angle=0d0 /
&REC_LINE file='rec.tab', field='D' /
"""
    (tmp_path / "Par.inp").write_text(text)
    from sem2dpack_gb300.parinp import load_parinp
    d = load_parinp(str(tmp_path / "Par.inp"))
    assert d.sources.coords == [(1000.0, 1000.0), (3000.0, 1200.0)]
    assert d.sources.tdelay == [0.0, 0.05] and d.sources.relamp == [1.0, 0.5]
    assert d.receivers.number == 3 and d.receivers.coords.shape == (3, 2)
    P = Problem(d)
    desc = P.desc()
    assert desc.nsrc == 2 and desc.nrec == 3
    np.testing.assert_allclose(P.rec_coord()[0], [500.0, 1500.0, 2500.0])


def test_tpv3_workload_restates_the_example(golden):
    """workloads.tpv3_inplane(scale=1) builds the same problem as the
    reference's TPV3 in-plane deck parsed from its Par.inp."""
    a = Problem(deck_from_parinp(str(golden["parinp_TestFlt2D_SCEC_TPV3_inplane"])))
    b = workloads.build(workloads.tpv3_inplane(1.0))
    da, db = a.desc(), b.desc()
    assert (da.npoin, da.nt, da.dt, da.nflt, da.nrec, da.ndir) == (db.npoin, db.nt, db.dt, db.nflt, db.nrec, db.ndir)
    for name, n in (("rmass", 2 * da.npoin), ("kv_eta", 36 * da.nelem), ("flt_T0", 2 * da.nflt),
                    ("swf_mus", da.nflt), ("rec_interp", 36 * da.nrec)):
        x = np.ctypeslib.as_array(getattr(da, name), shape=(n,))
        y = np.ctypeslib.as_array(getattr(db, name), shape=(n,))
        assert np.array_equal(x, y), name


WAVE_PARINP = """
&GENERAL ngll=5, fmax=10d0, ndof=2 /
&MESH_DEF method='CARTESIAN' /
&MESH_CART xlim=0d0,2d3, zlim=0d0,1d3, nelem=20,10 /
&MATERIAL tag=1, kind='ELAST' /
&MAT_ELASTIC rho=2500d0, cp=5000d0, cs=2887d0 /
&BC_DEF tag=1, kind='ABSORB' /
&BC_DEF tag=2, kind='ABSORB' /
&BC_ABSORB stacey=F, let_wave=F /
&BC_DEF tag=3, kind='DIRNEU' /
&BC_DIRNEU h='N', v='N', hstf='GAUSSIAN', vstf='RICKER' /
&STF_GAUSSIAN f0=8d0, onset=0.1d0, ampli=1d6 /
&STF_RICKER f0=10d0, onset=0.12d0, ampli=2d6 /
&BC_DEF tag=4, kind='ABSORB' /
&TIME TotalTime=0.3d0, courant=0.5d0 /
&SRC_DEF stf='BRUNE', coord=0d0,0d0, mechanism='WAVE' /
&STF_BRUNE ampli=2d0, fc=3d0 /
&SRC_WAVE angle=30d0, phase='P' /
&REC_LINE number=5, first=200d0,500d0, last=1800d0,500d0 /
"""


def test_wave_traction_and_time_function_blocks():
    """&SRC_DEF mechanism='WAVE' + &SRC_WAVE (src_wave.f90:56-110), a time
    function other than Ricker read from the block after &SRC_DEF, let_wave
    of &BC_ABSORB, and the hstf/vstf blocks that follow &BC_DIRNEU in order
    (bc_dirneu.f90:50-112)."""
    from sem2dpack_gb300 import Problem, abi
    dk = deck_from_parinp(WAVE_PARINP)
    s = dk.sources
    assert s.mechanism == "WAVE" and s.wave_angle == 30.0 and s.wave_phase == "P"
    assert s.stf.kind == "BRUNE" and s.stf.f0 == 3.0 and s.stf.ampli == 2.0
    assert dk.no_wave == [2]
    h, v = dk.dirneu_stf[3]
    assert h.kind == "GAUSSIAN" and h.f0 == 8.0 and v.kind == "RICKER" and v.ampli == 2e6
    P = Problem(dk)
    d = P.desc()
    assert d.wave_phase == abi.WAVE_P and d.nsrc == 0
    assert d.nneu == 2 * 81 and d.nneu_stf == 2
    wave = np.ctypeslib.as_array(d.abs_wave, shape=(d.nabs,))
    assert wave.sum() == d.nabs - 41  # the right side (tag 2) has let_wave=F

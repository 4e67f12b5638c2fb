"""A Par.inp deck through the GPU path and back out in the reference's file
formats: the example Lamb's problem deck (text fixture) and a fault deck."""
import numpy as np
import pytest

from sem2dpack_gb300 import PRECISION_MIXED, Problem, Solver, outputs
from sem2dpack_gb300.parinp import deck_from_parinp
from test_parinp import FAULT_PARINP

pytestmark = pytest.mark.gpu


def test_lamb_parinp_to_seismogram_files(golden, tmp_path):
    P = Problem(deck_from_parinp(str(golden["parinp_LambsProblem"])))
    g = Solver(P)
    g.step(400)
    outputs.write_run(str(tmp_path), g, P)
    sis, tsamp, xz = outputs.read_seismograms(str(tmp_path), 2)
    assert np.array_equal(sis, g.seismograms().astype(np.float32))
    assert np.abs(sis).max() > 0


def test_fault_parinp_to_fault_files(tmp_path):
    dk = deck_from_parinp(FAULT_PARINP, precision=PRECISION_MIXED)
    dk.fault.potency = True
    P = Problem(dk)
    g = Solver(P)
    g.step(P.nt)
    outputs.write_run(str(tmp_path), g, P)
    series, odt, xz = outputs.read_fault(str(tmp_path), 5)
    assert np.array_equal(series, g.fault_series().astype(np.float32))
    lines = open(tmp_path / "Flt05_potency_sem2d.tab").read().splitlines()
    assert len(lines) == P.nt + 1


@pytest.mark.parametrize("precision", [0, 1])
def test_tpv3_inplane_deck_against_oracle(golden, precision):
    """The reference's SCEC TPV3 in-plane deck as written (PWCONR stress and
    friction rings, Gaussian Kelvin-Voigt band, one-sided fault, symmetry
    side, Newmark, interpolated velocity receivers) for 300 steps, GPU
    against the FP64 oracle: FP64 <= 1e-10, mixed <= 1e-4."""
    from oracle import pyoracle as po
    from sem2dpack_gb300 import PRECISION_FP64
    dk = deck_from_parinp(str(golden["parinp_TestFlt2D_SCEC_TPV3_inplane"]))
    P = Problem(dk)
    d = P.desc()
    d.precision = PRECISION_FP64 if precision == 0 else PRECISION_MIXED
    tol = 1e-10 if precision == 0 else 1e-4
    g = Solver(d, owner=P)
    g.step(300)
    o = po.OracleSim(d, owner=P)
    o.run(300)

    def rel(a, b):
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 0, :].max() > 0  # the nucleation patch slipped
    for rec in (0, 1, 2, 4):
        assert rel(fg[:, rec, :], fo[:, rec, :]) <= tol, rec
    assert rel(g.seismograms(), o.seismograms()) <= tol


def test_snapshots_from_the_gpu(tmp_path):
    """write_snapshot over the GPU getters: D, V, A node fields and the
    strain and stress records, against the FP64 oracle (FP32 files)."""
    from oracle import pyoracle as po
    from sem2dpack_gb300 import PRECISION_FP64, workloads
    dk = workloads.plain_psv(scale=0.1, nsteps=100)
    dk.time.kind = "newmark"  # a handle keeps accelerations under Newmark (or for 'A' receivers)
    P = Problem(dk)
    d = P.desc()
    d.precision = PRECISION_FP64
    g = Solver(d, owner=P)
    g.step(100)
    o = po.OracleSim(d, owner=P)
    o.run(100)
    outputs.write_snapshot(str(tmp_path), g, 1, "DVAES")
    D, V, A = o.fields()
    for c, arr in (("d", D), ("v", V), ("a", A)):
        for k, comp in enumerate("xz"):
            back = np.fromfile(tmp_path / ("%s%s_001_sem2d.dat" % (c, comp)), dtype="<f4")
            np.testing.assert_allclose(back, arr[:, k], rtol=1e-6, atol=1e-6 * np.abs(arr).max())
    e, s = o.strain_stress()
    for pre, arr in (("e", e), ("s", s)):
        raw = np.fromfile(tmp_path / ("%s12_001_sem2d.dat" % pre), dtype="<f4").reshape(d.nelem, -1)
        ref = np.transpose(arr[:, :, 2, :], (2, 1, 0)).reshape(d.nelem, -1)
        np.testing.assert_allclose(raw, ref, rtol=1e-6, atol=1e-6 * np.abs(ref).max())


@pytest.mark.parametrize("precision", [0, 1])
def test_ratestate_example_against_reference_traces(golden, precision):
    from sem2dpack_gb300 import PRECISION_FP64
    from test_ratestate_example import check_ratestate
    P = Problem(deck_from_parinp(str(golden["parinp_RateState"])))
    d = P.desc()
    d.precision = PRECISION_FP64 if precision == 0 else PRECISION_MIXED
    g = Solver(d, owner=P)
    g.run()
    check_ratestate(P, g.fault_series(), golden)


@pytest.mark.parametrize("mech", ["EXPLOSION", "DOUBLE_COUPLE", "MOMENT"])
@pytest.mark.parametrize("ndof", [1, 2])
def test_moment_sources_against_oracle(mech, ndof):
    """Explosion, double-couple and moment-tensor sources (point forces on
    the lines through the source node, src_moment.f90:118-175), FP64."""
    from oracle import pyoracle as po
    from sem2dpack_gb300 import PRECISION_FP64, workloads
    if mech == "EXPLOSION" and ndof == 1:
        pytest.skip("explosions are P-SV only (src_moment.f90:56-57)")
    dk = workloads.plain_psv(scale=0.2, nsteps=200)
    dk.ndof = ndof
    dk.sources.mechanism, dk.sources.dip, dk.sources.M = mech, 30.0, (1.0, 0.4, 0.4, -0.7)
    P = Problem(dk)
    d = P.desc()
    d.precision = PRECISION_FP64
    g = Solver(d, owner=P)
    g.step(200)
    o = po.OracleSim(d, owner=P)
    o.run(200)
    s_g, s_o = g.seismograms(), o.seismograms()
    assert np.abs(s_o).max() > 0
    assert np.linalg.norm(s_g - s_o) / np.linalg.norm(s_o) <= 1e-10

"""Parity at the benchmark configurations' full size and length.

The mixed-precision GPU path (FP32 fields, FP64 fault state) against the
FP64 oracle over every time step of:
  * the SH rupture (400 x 200 elements, NGLL=5, 6000 steps, slip weakening);
  * a reduced copy of the P-SV rate-and-state rupture (154 x 77 elements,
    1500 steps, aging law);
the FP64 GPU path against the oracle on the plain P-SV box (100 x 100
elements, 2000 steps), and both forms of the NGLL=5 shear term on elements
that are not square: the reference's optimised kernel uses a4 for both
shear derivatives (ELAST_KD2_PSV, mat_elastic.f90:612-613) where the
general one uses a4 and a5 (ELAST_KD1_PSV, :489-490); the two agree only
on square elements.

Every output of the fault is compared as its own relative L2 error over
all samples and nodes: slip, slip rate, shear and normal traction,
friction coefficient, and the rupture time of every node (the first sample
where the slip rate reaches 1e-3 m/s, POST/python/post-process-fault.py:
55-62).  The errors are printed (pytest -s) for the record.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Material, Solver, abi, workloads
from sem2dpack_gb300.outputs import rupture_time

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

RECORDS = ["slip", "slip rate", "shear traction", "normal traction", "friction"]


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def run_pair(P, precision, nsteps):
    d = P.desc()
    d.precision = precision
    g = Solver(d, owner=P)
    g.step(nsteps)
    d64 = abi.ProblemDesc.from_buffer_copy(d)
    d64.precision = PRECISION_FP64
    o = po.OracleSim(d64, owner=P)
    o.run(nsteps)
    return d, g, o


def fault_errors(d, g, o, rsf=False):
    fg, fo = g.fault_series(), o.fault_series()
    err = {name: rel_l2(fg[:, k, :], fo[:, k, :]) for k, name in enumerate(RECORDS)}
    odt = d.flt_oitd * d.dt
    tg, ig = rupture_time(fg[:, 1, :], odt)
    to, io = rupture_time(fo[:, 1, :], odt)
    err["rupture time"] = rel_l2(tg, to)
    err["ruptured nodes"] = int((io >= 0).sum())
    err["rupture sample shifts"] = int((ig != io).sum())
    return err


def report(name, err):
    print("\n%s: %s" % (name, ", ".join("%s %.3g" % (k, v) if isinstance(v, float) else "%s %d" % (k, v)
                                         for k, v in err.items())))


@pytest.mark.parametrize("kernel", ["march", "strip"])
def test_sh_rupture_full_length_mixed(kernel, monkeypatch):
    """Both step kernels keep the elastic force as their state here (a
    slipped fault leaves a static displacement FP32 cannot resolve)."""
    if kernel == "strip":
        monkeypatch.setenv("SEM2D_MARCH", "0")
    pair = workloads.sh_rupture()
    P = workloads.build(pair)
    d, g, o = run_pair(P, PRECISION_MIXED, 6000)
    err = {"seismograms": rel_l2(g.seismograms(), o.seismograms())}
    err.update(fault_errors(d, g, o))
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    err["final displacement"] = rel_l2(dg, do)
    err["final velocity"] = rel_l2(vg, vo)
    report("SH rupture 400x200, 6000 steps, mixed (%s kernel) vs FP64 oracle" % kernel, err)
    assert err["ruptured nodes"] > 500  # the rupture spreads along the fault
    for k in ["seismograms", "slip", "slip rate", "shear traction", "normal traction", "friction"]:
        assert err[k] <= 1e-4, (k, err[k])
    assert err["rupture time"] <= 1e-4, err["rupture time"]


def test_psv_rsf_reduced_mixed():
    pair = workloads.psv_rsf(scale=0.15, nsteps=1500)
    P = workloads.build(pair)
    d, g, o = run_pair(P, PRECISION_MIXED, 1500)
    err = {"seismograms": rel_l2(g.seismograms(), o.seismograms())}
    err.update(fault_errors(d, g, o, rsf=True))
    report("P-SV rate-and-state 154x77, 1500 steps, mixed vs FP64 oracle", err)
    assert np.abs(o.seismograms()).max() > 0
    for k in ["seismograms", "slip", "slip rate", "shear traction", "friction"]:
        assert err[k] <= 1e-4, (k, err[k])


def test_plain_psv_full_length_fp64():
    P = workloads.build(workloads.plain_psv())
    d, g, o = run_pair(P, PRECISION_FP64, 2000)
    err = {"seismograms": rel_l2(g.seismograms(), o.seismograms())}
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    err["final displacement"] = rel_l2(dg, do)
    err["final velocity"] = rel_l2(vg, vo)
    report("plain P-SV 100x100, 2000 steps, FP64 vs FP64 oracle", err)
    for k, v in err.items():
        assert v <= 1e-10, (k, v)


def rectangular_box(kd2):
    """P-SV box of 40 x 20 elements of 100 m x 200 m (a4 != a5), NGLL=5."""
    dk = workloads.plain_psv(scale=0.4, nsteps=300)
    dk.zlim = (0.0, 4000.0)
    dk.nelem = (40, 20)
    dk.xlim = (0.0, 4000.0)
    dk.materials = [Material(tag=1, rho=2700.0, cp=5000.0, cs=2887.0)]
    dk.time.courant = 0.4
    dk.fmax = 5.0  # resolution check of the reference (init.f90:271-281) on 200 m elements
    dk.kd2_form = kd2
    return dk


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_kd2_shear_form_on_rectangular_elements(precision):
    out = {}
    for kd2 in (1, 0):
        P = workloads.build(rectangular_box(kd2))
        d, g, o = run_pair(P, precision, 300)
        assert d.kd2_form == kd2
        s_g, s_o = g.seismograms(), o.seismograms()
        assert rel_l2(s_g, s_o) <= (1e-10 if precision == PRECISION_FP64 else 1e-4), kd2
        out[kd2] = s_o
    # the flag matters on these elements: the two forms differ well above
    # the tolerance
    assert rel_l2(out[1], out[0]) > 1e-3

"""The one-element-per-thread step kernel (FP32, NGLL=5, isotropic,
leapfrog) against the FP64 oracle, against the strip kernel, and across
chunk heights.

Tolerances (relative L2 over the whole compared array): mixed path against
the oracle <= 1e-4, the two FP32 kernels against each other <= 2e-5 (same
formulas and summation order, FMA contraction may differ); chunk heights of
the march kernel agree bitwise (the per-node summation order does not
depend on the work decomposition).
"""
import numpy as np
import pytest
from conftest import watch_launches

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_MIXED, Solver, workloads

pytestmark = pytest.mark.gpu

MARCH_TX = 31  # element columns of one march unit


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


CASES = {
    # one strip, lanes beyond the last element column idle
    "plain_psv_20": (lambda: workloads.plain_psv(scale=0.2, nsteps=200), 200),
    # two strips, the second ragged
    "plain_psv_45": (lambda: workloads.plain_psv(scale=0.45, nsteps=150), 150),
    # exactly two full strips
    "plain_psv_62": (lambda: workloads.plain_psv(scale=0.62, nsteps=120), 120),
    # SH, split-node fault with slip weakening, material per element
    "sh_rupture": (lambda: workloads.sh_rupture(scale=0.1, nsteps=300), 300),
    # P-SV, rate-and-state fault, material per node (random medium)
    "psv_rsf": (lambda: workloads.psv_rsf(scale=0.05, nsteps=200), 200),
}


def make(case, monkeypatch, env=None):
    for k, v in (env or {}).items():
        monkeypatch.setenv(k, str(v))
    P = workloads.build(case)
    d = P.desc()
    d.precision = PRECISION_MIXED
    g = Solver(d, owner=P)
    for k in (env or {}):
        monkeypatch.delenv(k)
    return P, d, g


def outputs(g, has_fault):
    d, v = g.fields()
    out = {"sis": g.seismograms().copy(), "d": d.copy(), "v": v.copy()}
    if has_fault:
        out["fault"] = g.fault_series().copy()
    return out


@pytest.mark.parametrize("name", list(CASES))
def test_march_against_oracle(name, monkeypatch):
    build, nt = CASES[name]
    P, d, g = make(build(), monkeypatch)
    assert g.tile[0] == MARCH_TX
    g.step(nt)
    o = po.OracleSim(d, owner=P)
    o.run(nt)
    s_o = o.seismograms()
    assert np.abs(s_o).max() > 0
    assert rel_l2(g.seismograms(), s_o) <= 1e-4
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= 1e-4
    assert rel_l2(vg, vo) <= 1e-4
    if d.nflt:
        fg, fo = g.fault_series(), o.fault_series()
        for rec in (0, 1):  # slip, slip rate
            assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= 1e-4, rec


@pytest.mark.parametrize("name", ["plain_psv_45", "sh_rupture", "psv_rsf"])
def test_march_against_strip_kernel(name, monkeypatch):
    """Same formulas in FP32.  With a fault the march kernel carries the
    force state and the strip kernel the displacement state, whose FP32
    displacement next to the slipped fault is the coarser of the two: there
    the two agree to the mixed tolerance (1e-4)."""
    build, nt = CASES[name]
    case = build()
    P, d, g = make(case, monkeypatch)
    _, _, h = make(case, monkeypatch, {"SEM2D_MARCH": 0})
    assert g.tile[0] == MARCH_TX and h.tile[0] != MARCH_TX
    g.step(nt)
    h.step(nt)
    a, b = outputs(g, d.nflt), outputs(h, d.nflt)
    for k in a:
        assert rel_l2(a[k], b[k]) <= (1e-4 if d.nflt else 2e-5), k


@pytest.mark.parametrize("name", ["plain_psv_45", "sh_rupture", "psv_rsf"])
def test_march_chunk_heights_agree(name, monkeypatch):
    build, nt = CASES[name]
    case = build()
    P, d, g = make(case, monkeypatch)
    g.step(nt)
    ref = outputs(g, d.nflt)
    for cz in (1, 2, 3, 7):
        _, _, h = make(case, monkeypatch, {"SEM2D_MARCH_CZ": cz})
        assert h.tile == (MARCH_TX, cz)
        h.step(nt)
        out = outputs(h, d.nflt)
        for k in ref:
            assert np.array_equal(ref[k], out[k]), (cz, k)


@pytest.mark.parametrize("field,atnode", [("D", False), ("A", True), ("V", False), ("D", True)])
def test_march_receivers(field, atnode, monkeypatch):
    dk = workloads.plain_psv(scale=0.45, nsteps=150)
    dk.receivers.atnode = atnode
    dk.receivers.field = field
    P, d, g = make(dk, monkeypatch)
    assert g.tile[0] == MARCH_TX
    g.step(150)
    o = po.OracleSim(d, owner=P)
    o.run(150)
    assert rel_l2(g.seismograms(), o.seismograms()) <= 1e-4
    # interpolated velocity is sampled by the separate kernel after the step
    assert g.launches == 150 * (2 if (field != "D" and not atnode) else 1) + watch_launches(150)


def test_fused_fault_side_equals_separate_kernels(monkeypatch):
    """Slip weakening: the fault-side units and the fault update in one
    launch give the same bits as the two separate launches."""
    build, nt = CASES["sh_rupture"]
    case = build()
    P, d, g = make(case, monkeypatch)
    _, _, h = make(case, monkeypatch, {"SEM2D_FUSED_FAULT": 0})
    lg, lh = g.launches, h.launches
    g.step(nt)
    h.step(nt)
    assert g.launches - lg == 2 * nt + watch_launches(nt) and h.launches - lh == 3 * nt + watch_launches(nt)
    a, b = outputs(g, True), outputs(h, True)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("name", ["sh_rupture", "psv_rsf"])
def test_force_state_is_closer_to_fp64(name, monkeypatch):
    """Problems with a fault carry the elastic force as the state (the
    element pass applies the stiffness to the velocity); in exact arithmetic
    it equals the displacement state, which SEM2D_FORCE_STATE=0 selects.
    In FP32 it is the closer of the two to the FP64 oracle: the displacement
    next to the slipped fault loses the digits of the dynamic stress."""
    build, nt = CASES[name]
    case = build()
    P, d, g = make(case, monkeypatch)
    _, _, h = make(case, monkeypatch, {"SEM2D_FORCE_STATE": 0})
    g.step(nt)
    h.step(nt)
    o = po.OracleSim(d, owner=P)
    o.run(nt)
    s_o, f_o = o.seismograms(), o.fault_series()[:, 1, :]
    e_force = rel_l2(g.seismograms(), s_o) + rel_l2(g.fault_series()[:, 1, :], f_o)
    e_displ = rel_l2(h.seismograms(), s_o) + rel_l2(h.fault_series()[:, 1, :], f_o)
    assert e_force <= 1e-4 and e_displ <= 1e-4
    if name == "sh_rupture":  # slip of a metre within the run
        assert e_force < 0.5 * e_displ, (e_force, e_displ)

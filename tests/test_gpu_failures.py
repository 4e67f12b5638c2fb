"""Failure reporting of the GPU time step, without faulting the GPU.

Each failure is made on the host side of the call and read back as a
status code:
  * the rate-and-state Newton solver capped at one iteration
    (desc.flt_nr_maxit = 1): SEM2D_E_NR, where the reference aborts
    (bc_dynflt_rsf.f90:461-466);
  * the bounded wait of the strip kernel for its shared-memory copies
    given no polls at all (SEM2D_SPIN_LIMIT=0): SEM2D_E_TIMEOUT; every
    CTA still waits (with the normal limit) for the copies it issued, so
    the context stays usable, which the test checks with a normal run;
  * a source amplitude that is NaN: the max|v|, max|d| check every
    info_every steps (main.f90:73-76) reports SEM2D_E_NAN.
The progress values of that check (sem2d_gpu_get_info) are compared with
the fields.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Sem2dError, Solver, abi, workloads
from sem2dpack_gb300._lib import lib

pytestmark = pytest.mark.gpu


def _info(sim):
    st, v, d = C.c_int(), C.c_double(), C.c_double()
    sim._check(lib().sem2d_gpu_get_info(sim.h, C.byref(st), C.byref(v), C.byref(d)))
    return st.value, v.value, d.value


def test_newton_cap_reports_nr():
    P = workloads.build(workloads.psv_rsf(scale=0.05, nsteps=20, rsf_kind=2))
    d = P.desc()
    d.precision = PRECISION_FP64
    d.flt_nr_maxit = 1
    sim = Solver(d, owner=P)
    sim.step(5)
    with pytest.raises(Sem2dError) as e:
        sim.sync()
    assert e.value.code == abi.SEM2D_E_NR
    sim.close()
    # the default cap (200) runs the same steps without error
    d.flt_nr_maxit = 0
    ok = Solver(d, owner=P)
    ok.step(5)
    ok.sync()
    ok.close()


def test_spin_limit_zero_reports_timeout(monkeypatch):
    P = workloads.build(workloads.plain_psv(scale=0.2, nsteps=40))
    d = P.desc()
    d.precision = PRECISION_FP64  # the strip kernel (TMA stages, bounded waits)
    monkeypatch.setenv("SEM2D_SPIN_LIMIT", "0")
    sim = Solver(d, owner=P)
    sim.step(3)
    with pytest.raises(Sem2dError) as e:
        sim.sync()
    assert e.value.code == abi.SEM2D_E_TIMEOUT
    sim.close()
    monkeypatch.delenv("SEM2D_SPIN_LIMIT")
    # the context is still usable: a normal run matches the oracle
    sim = Solver(d, owner=P)
    sim.step(40)
    ref = po.OracleSim(d, owner=P)
    ref.run(40)
    a, b = sim.seismograms(), ref.seismograms()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 1e-10
    sim.close()


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_nan_watchdog(precision):
    P = workloads.build(workloads.plain_psv(scale=0.2, nsteps=40))
    d = P.desc()
    d.precision = precision
    d.info_every = 10
    bad = np.array([np.nan])
    d.src_ampli = bad.ctypes.data_as(abi.P_double)
    sim = Solver(d, owner=P)
    sim.step(25)
    with pytest.raises(Sem2dError) as e:
        sim.sync()
    assert e.value.code == abi.SEM2D_E_NAN
    sim.close()


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
def test_info_values_match_fields(precision):
    P = workloads.build(workloads.plain_psv(scale=0.2, nsteps=60))
    d = P.desc()
    d.precision = precision
    d.info_every = 25
    sim = Solver(d, owner=P)
    sim.step(60)  # checks after steps 25 and 50
    step, vmax, dmax = _info(sim)
    assert step == 50
    sim.reset()
    sim.step(50)
    disp, vel = sim.fields()
    assert vmax == pytest.approx(np.abs(vel).max(), rel=1e-6)
    assert dmax == pytest.approx(np.abs(disp).max(), rel=1e-6)
    assert vmax > 0 and dmax > 0
    sim.close()


def test_watchdog_off_keeps_running():
    P = workloads.build(workloads.plain_psv(scale=0.2, nsteps=30))
    d = P.desc()
    d.precision = PRECISION_MIXED
    d.info_every = -1
    sim = Solver(d, owner=P)
    sim.step(30)
    sim.sync()
    assert _info(sim)[0] == 0
    sim.close()


"""Source time functions (STF_get, stf_gen.f90:99-121).

The library's evaluation (sem2d_stf_eval, the code that fills the point
sources' tables and the boundary forces) and the oracle's restatement are
checked against the closed forms of stf_ricker.f90, stf_gaussian.f90,
stf_brune.f90, stf_harmonic.f90 and stf_user.f90 written here in numpy,
and the tabulated function against scipy's cubic spline with zero end
slopes (the spline STF_TAB_read builds, stf_tabulated.f90:66)."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import abi
from sem2dpack_gb300._lib import lib
from sem2dpack_gb300.deck import Stf

P_d = C.POINTER(C.c_double)


def evaluate(which, stf, t):
    keep = []
    s = stf.to_c(keep)
    t = np.ascontiguousarray(t, dtype=np.float64)
    out = np.zeros_like(t)
    fn = lib().sem2d_stf_eval if which == "lib" else po.lib().oc_stf_eval
    assert fn(C.byref(s), t.size, t.ctypes.data_as(P_d), out.ctypes.data_as(P_d)) == 0
    return out


def closed_form(s, t):
    pi = 3.141592653589793
    if s.kind == "RICKER":
        a = (pi * s.f0 * (t - s.onset)) ** 2
        return -s.ampli * (1 - 2 * a) * np.exp(-a)
    if s.kind == "GAUSSIAN":
        return s.ampli * np.exp(-(pi * s.f0 * (t - s.onset)) ** 2)
    if s.kind == "BRUNE":
        a = 2 * pi * s.f0 * np.maximum(t, 0.0)
        return s.ampli * (1 - (1 + a) * np.exp(-a))
    if s.kind == "HARMONIC":
        return s.ampli * np.sin(2 * pi * t * s.f0)
    if s.kind == "USER":
        a = t - s.onset
        return s.ampli * np.sin(a) + s.par1 * a * a
    raise ValueError(s.kind)


CASES = [Stf("RICKER", f0=3.0, onset=0.5, ampli=2.0), Stf("GAUSSIAN", f0=2.0, onset=0.4, ampli=-1.5),
         Stf("BRUNE", f0=1.5, ampli=3.0), Stf("HARMONIC", f0=2.5, ampli=0.7),
         Stf("USER", onset=0.3, ampli=1.2, par1=0.5, par2=9.0)]


@pytest.mark.parametrize("stf", CASES, ids=[c.kind for c in CASES])
def test_closed_forms(stf):
    t = np.linspace(-0.5, 2.0, 1001)
    ref = closed_form(stf, t)
    scale = np.abs(ref).max()
    for which in ("lib", "oracle"):
        got = evaluate(which, stf, t)
        assert np.abs(got - ref).max() <= 1e-14 * scale * 10, which


def _table():
    rng = np.random.default_rng(20261204)
    t = np.cumsum(rng.uniform(0.05, 0.3, 24))
    v = np.sin(3 * t) + 0.1 * rng.standard_normal(t.size)
    return t, v


def test_tabulated_is_the_clamped_spline():
    from scipy.interpolate import CubicSpline
    t, v = _table()
    stf = Stf("TAB", tab=(t, v))
    x = np.random.default_rng(7).uniform(t[0] - 1, t[-1] + 1, 4000)  # unsorted: the oracle's bracket search moves both ways
    ref = CubicSpline(t, v, bc_type=((1, 0.0), (1, 0.0)))(np.clip(x, t[0], t[-1]))
    for which in ("lib", "oracle"):
        got = evaluate(which, stf, x)
        assert np.abs(got - ref).max() <= 1e-12, which
    # at the rows the function takes the tabulated values exactly
    for which in ("lib", "oracle"):
        assert np.array_equal(evaluate(which, stf, t), v), which


def test_library_and_oracle_agree_on_tables_and_edges():
    t, v = _table()
    stf = Stf("TAB", tab=(t, v))
    x = np.concatenate([t, t[:-1] + 0.5 * np.diff(t), [t[0] - 5, t[-1] + 5, t[0], t[-1]]])
    a, b = evaluate("lib", stf, x), evaluate("oracle", stf, x)
    assert np.abs(a - b).max() <= 1e-15 * np.abs(b).max()


def test_bad_descriptions_are_refused():
    keep = []
    bad = Stf("TAB", tab=(np.array([0.0, 1.0, 1.0]), np.array([0.0, 1.0, 2.0]))).to_c(keep)
    out = np.zeros(1)
    t = np.zeros(1)
    assert lib().sem2d_stf_eval(C.byref(bad), 1, t.ctypes.data_as(P_d), out.ctypes.data_as(P_d)) == abi.SEM2D_E_ARG
    unknown = abi.Stf()
    unknown.kind = 2  # BUTTERWORTH: the reference aborts, not implemented
    assert lib().sem2d_stf_eval(C.byref(unknown), 1, t.ctypes.data_as(P_d), out.ctypes.data_as(P_d)) == abi.SEM2D_E_ARG
    with pytest.raises(ValueError):
        Stf("BUTTERWORTH").to_c(keep)

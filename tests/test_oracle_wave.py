"""The oracle's incident plane wave against its analytic form.

In a homogeneous box with periodic left and right sides and absorbing
bottom and top (the 1-D set-up of EXAMPLES/TestAbso/Par.inp), a wave
entering from below at normal incidence is the whole field: the absorbing
terms act on the diffracted part only (bc_abso.f90:279-306), so the
velocity at height z is P f(t - z/c) (src_wave.f90:4-12), P the
polarisation, f the time function, c the phase speed.  This pins the
restatement of SRC_WAVE_get_VT and BC_ABSO_apply independently of the GPU
comparison."""
import numpy as np
import pytest

import decks
from oracle import pyoracle as po
from sem2dpack_gb300 import Problem
from sem2dpack_gb300.deck import Stf


def ricker(t, f0, t0):
    a = (np.pi * f0 * (t - t0)) ** 2
    return -(1 - 2 * a) * np.exp(-a)


def analytic_case(ndof, phase):
    dk = decks.wave_box(ndof, phase, 0.0, periodic=True, stf=Stf("RICKER", f0=5.0, onset=0.25, ampli=1.0))
    dk.time.total_time = 0.8
    dk.nelem = (20, 20)
    return dk


def compare(dk, sis, dt, isamp):
    ndof = dk.ndof
    c = 5000.0 if dk.sources.wave_phase == "P" and ndof == 2 else 2887.0
    # the velocity recorded after step it is v at (it + 1/2) dt (solve_leapfrog, solver.f90:133-161)
    t = (np.arange(sis.shape[0]) * isamp + 0.5) * dt
    f = ricker(t - 500.0 / c, float(np.float32(5.0)), float(np.float32(0.25)))
    comp = 1 if (ndof == 2 and dk.sources.wave_phase == "P") else 0
    expect = np.zeros_like(sis)
    expect[:, :, comp] = f[:, None]
    return np.linalg.norm(sis - expect) / np.linalg.norm(expect)


@pytest.mark.parametrize("ndof,phase", [(1, "S"), (2, "P"), (2, "S")])
def test_oracle_wave_is_the_analytic_plane_wave(ndof, phase):
    dk = analytic_case(ndof, phase)
    P = Problem(dk)
    d = P.desc()
    o = po.OracleSim(d, owner=P)
    o.run(d.nt)
    err = compare(dk, o.seismograms(), d.dt, d.rec_isamp)
    assert err <= 5e-3, err

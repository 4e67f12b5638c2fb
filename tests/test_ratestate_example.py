"""The reference's rate-and-state example (EXAMPLES/RateState/Par.inp:
SH, one-sided fault on the bottom side, RSF kind 3, ORDER0 initial stress
and state, Neumann sides, Newmark) run as written, against the slip, slip
rate and shear stress change traces the example ships at x = 0, 3, 6 and
9 km ({Ux,Vx,Tau}_{0,3,6,9}km_ascii, every step of 803).

The traces' provenance is not recorded and they carry dt = 4.985e-3 s
(their first slip sample is V dt) where this deck gives 4.98479e-3 s, so
this is a loose pin: relative L2 per station within 1 % for slip, 4 % for
slip rate and 2 % for stress (measured: 0.17-0.78 %, 0.17-3.3 %,
0.01-1.6 %, growing with the distance the rupture has run), and 0.3 % at
the nucleation point for all three.  The oracle runs it on the CPU; the GPU
path runs it in test_gpu_frontend.py against the same bounds.
"""
import numpy as np

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, Problem
from sem2dpack_gb300.parinp import deck_from_parinp

BOUNDS = {"Ux": 0.01, "Vx": 0.04, "Tau": 0.02}


def check_ratestate(P, series, golden):
    x = P.fault_coord()[0]
    idx = [int(np.argmin(np.abs(x - xx))) for xx in (0.0, 3e3, 6e3, 9e3)]
    assert np.allclose(x[idx], [0.0, 3e3, 6e3, 9e3])
    for q, rec in (("Ux", 0), ("Vx", 1), ("Tau", 2)):
        ref = golden["ratestate_" + q]
        ours = series[idx, rec, 1:1 + ref.shape[1]]
        err = [np.linalg.norm(ours[i] - ref[i]) / np.linalg.norm(ref[i]) for i in range(4)]
        assert max(err) <= BOUNDS[q], (q, err)
        assert err[0] <= 3e-3, (q, err)


def test_ratestate_example_oracle(golden):
    dk = deck_from_parinp(str(golden["parinp_RateState"]))
    P = Problem(dk)
    d = P.desc()
    d.precision = PRECISION_FP64
    assert d.nt == 803
    o = po.OracleSim(d, owner=P)
    o.run(d.nt)
    check_ratestate(P, o.fault_series(), golden)

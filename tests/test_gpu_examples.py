"""Every example deck of the reference that the Cartesian front end takes
(16),
run as written through the GPU path for its first 30 steps against the FP64
oracle (FP64 <= 1e-9 for the rate-and-state decks' Newton solves, 1e-10
otherwise; mixed <= 1e-4): seismograms, and slip and slip rate on faults.
The decks are text fixtures (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Problem, Solver
from conftest import example_deck

pytestmark = pytest.mark.gpu

EXAMPLES = ["LambsProblem", "TestSH", "Anisotropic", "InaBox", "TestFlt2D_SCEC_TPV3_inplane", "RateState",
            "TestFlt1D", "Bimaterial_fault", "2.5D_V-shape_rate-and-state", "2.5D_inplane",
            "2D_roughness_drag_approximation", "Kelvin_Visco_FZ", "Velocity_weakening", "TestAbso", "TestLayers",
            "TestLayers_2"]


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("name", EXAMPLES)
def test_example_deck(golden, name, precision, tmp_path):
    dk = example_deck(golden, name, tmp_path)
    P = Problem(dk)
    d = P.desc()
    d.precision = precision
    n = min(30, d.nt)
    g = Solver(d, owner=P)
    g.step(n)
    o = po.OracleSim(d, owner=P)
    o.run(n)
    rsf = dk.fault is not None and dk.fault.friction == "RSF"
    tol = (1e-9 if rsf else 1e-10) if precision == PRECISION_FP64 else 1e-4
    if d.nrec:
        assert rel_l2(g.seismograms(), o.seismograms()) <= tol
    if d.nflt:
        fg, fo = g.fault_series(), o.fault_series()
        for rec in (0, 1):
            assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= tol, rec
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(vg, vo) <= tol

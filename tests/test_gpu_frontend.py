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

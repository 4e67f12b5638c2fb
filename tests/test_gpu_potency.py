"""Fault potency records on the GPU (sem2d_gpu_get_fault_potency) against
the oracle: FP64 <= 1e-10 relative L2 (the GPU sums the node terms in a
different order), mixed <= 1e-4; both kernels of the mixed path."""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Sem2dError, Solver, workloads

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def case(name, nsteps):
    pair = (workloads.sh_rupture(scale=0.1, nsteps=nsteps) if name == "sh"
            else workloads.psv_rsf(scale=0.05, nsteps=nsteps))
    pair[0].fault.potency = True
    return pair


@pytest.mark.parametrize("name", ["sh", "psv"])
@pytest.mark.parametrize("precision,march", [(PRECISION_FP64, "1"), (PRECISION_MIXED, "1"),
                                             (PRECISION_MIXED, "0")])
def test_potency_matches_oracle(name, precision, march, monkeypatch):
    nt = 200
    monkeypatch.setenv("SEM2D_MARCH", march)
    P = workloads.build(case(name, nt))
    d = P.desc()
    d.precision = precision
    g = Solver(d, owner=P)
    monkeypatch.delenv("SEM2D_MARCH")
    g.step(nt)
    o = po.OracleSim(d, owner=P)
    o.run(nt)
    pg, pr = g.fault_potency(), o.fault_potency()
    assert pg.shape == pr.shape == (nt + 1, 2, 3)
    assert np.abs(pr[:, 1]).max() > 0  # the fault slipped
    tol = 1e-10 if precision == PRECISION_FP64 else 1e-4
    assert rel_l2(pg[:, 0], pr[:, 0]) <= tol
    assert rel_l2(pg[:, 1], pr[:, 1]) <= tol


def test_potency_off_by_default():
    P = workloads.build(workloads.sh_rupture(scale=0.1, nsteps=20))
    g = Solver(P.desc(), owner=P)
    g.step(20)
    with pytest.raises(Sem2dError):
        g.fault_potency()

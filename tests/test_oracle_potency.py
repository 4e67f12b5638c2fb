"""Fault potency records of the oracle (BC_DYNFLT_potency,
bc_dynflt.f90:832-855, written every step at :757) against a direct
evaluation from the oracle's fields with numpy."""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, workloads


def direct_potency(desc, d, v):
    nf, nd = desc.nflt, desc.ndof
    n1 = np.ctypeslib.as_array(desc.flt_node1, shape=(nf,)) - 1
    two = bool(desc.flt_node2)
    n2 = np.ctypeslib.as_array(desc.flt_node2, shape=(nf,)) - 1 if two else None
    nrm = np.ctypeslib.as_array(desc.flt_n1, shape=(2 * nf,)).reshape(2, nf)
    B = np.ctypeslib.as_array(desc.flt_B, shape=(nf,))
    out = []
    for x in (d, v):
        x = x.reshape(-1, nd, order="F")
        dl = x[n2] - x[n1] if two else -2.0 * x[n1]
        if nd == 2:
            out.append([np.sum(nrm[0] * dl[:, 0] * B), np.sum(nrm[1] * dl[:, 1] * B),
                        0.5 * np.sum((nrm[0] * dl[:, 1] + nrm[1] * dl[:, 0]) * B)])
        else:
            out.append([0.5 * np.sum(nrm[0] * dl[:, 0] * B), 0.5 * np.sum(nrm[1] * dl[:, 0] * B), 0.0])
    return np.array(out)


@pytest.mark.parametrize("case", ["sh", "psv"])
def test_oracle_potency_matches_direct_sum(case):
    pair = (workloads.sh_rupture(scale=0.05, nsteps=60) if case == "sh"
            else workloads.psv_rsf(scale=0.03, nsteps=60))
    P = workloads.build(pair)
    d = P.desc()
    d.precision = PRECISION_FP64
    o = po.OracleSim(d, owner=P)
    pot = o.fault_potency()
    assert pot.shape == (d.nt + 1, 2, 3)
    assert np.all(pot[0] == 0.0)
    o.run(40)
    dd, vv, _ = o.fields()
    k = 40
    ref = direct_potency(d, dd.reshape(-1, order="F"), vv.reshape(-1, order="F"))
    got = o.fault_potency()[k]
    assert np.abs(ref).max() > 0
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())

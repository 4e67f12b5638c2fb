"""Zero-Dirichlet sides (&BC_DIRNEU h/v = 'D', bc_dirneu.f90:148-169) on the
GPU against the FP64 oracle: FP64 <= 1e-10 (rate-free faults) and mixed
<= 1e-4 relative L2.  At nodes a Dirichlet side shares with a fault the
&BC_DEF order decides whether the zero comes before the fault traction (the
step kernel zeroes the force it hands to the fault update) or after it (the
fault update zeroes the node's force).
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from sem2dpack_gb300 import PRECISION_FP64, PRECISION_MIXED, Solver, workloads
from sem2dpack_gb300.parinp import deck_from_parinp

from test_boundaries import dirneu_box

pytestmark = pytest.mark.gpu

TOL = {PRECISION_FP64: 1e-10, PRECISION_MIXED: 1e-4}


def rel_l2(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def run_both(deck_or_pair, nsteps, precision):
    P = workloads.build(deck_or_pair)
    d = P.desc()
    d.precision = precision
    g = Solver(d, owner=P)
    g.step(nsteps)
    o = po.OracleSim(d, owner=P)
    o.run(nsteps)
    return P, d, g, o


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("hv", [("N", "D"), ("D", "D"), ("D", "N")])
def test_box_side(precision, hv):
    P, d, g, o = run_both(dirneu_box(*hv), 200, precision)
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    dg, vg = g.fields()
    do, vo, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision]
    node = np.ctypeslib.as_array(d.dir_node, shape=(d.ndir,)) - 1
    comp = np.ctypeslib.as_array(d.dir_comp, shape=(d.ndir,))
    assert np.all(dg[node, comp] == 0) and np.all(vg[node, comp] == 0)


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("before", [True, False])
def test_split_fault_reaching_a_dirichlet_side(precision, before):
    """SH rupture on a split fault whose end nodes lie on the left side, held
    by h = 'D' there, before or after the fault in &BC_DEF order."""
    deck, grid = workloads.sh_rupture(scale=0.1, nsteps=300)
    deck.absorbing = [1, 2, 3]
    deck.dirneu = [(4, "D", "N", before)]
    P, d, g, o = run_both((deck, grid), 300, precision)
    assert d.ndir > 0
    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 0, -1].max() > 0.1
    for rec in (0, 1, 2, 4):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= TOL[precision], rec
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
    dg, _ = g.fields()
    do, _, _ = o.fields()
    assert rel_l2(dg, do) <= TOL[precision]


ONE_SIDED = """
&GENERAL ngll=5, fmax=10d0, ndof=2 /
&MESH_DEF method='CARTESIAN' /
&MESH_CART xlim=0d0,4d3, zlim=0d0,2d3, nelem=40,20 /
&MATERIAL tag=1, kind='ELAST' /
&MAT_ELASTIC rho=2670d0, cp=6000d0, cs=3464d0 /
&BC_DEF tag = 1, kind = 'DYNFLT' /
&BC_DYNFLT friction='SWF', Tn=-120d6, Tt=81.6d6 /
&BC_DYNFLT_SWF Dc=0.4d0, MuS=0.677d0, MuD=0.525d0 /
&BC_DEF tag=2, kind='ABSORB' /
&BC_DEF tag=3, kind='ABSORB' /
&BC_DEF tag=4, kind='DIRNEU' /
&BC_DIRNEU h='N', v='D' /
&TIME TotalTime=0.4d0, courant=0.5d0, kind='newmark' /
&REC_LINE number=8, first=250d0,500d0, last=3750d0,500d0 /
"""


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_MIXED])
@pytest.mark.parametrize("before", [False, True])
def test_one_sided_fault_with_symmetry_side(precision, before):
    """The layout of the reference's TestFlt2D_SCEC_TPV3_inplane deck: a
    one-sided fault on the bottom side, v = 'D' on the left side after it
    (the corner node is both), Newmark; and the same with the &BC_DIRNEU
    block first."""
    text = ONE_SIDED
    if before:
        blk = "&BC_DEF tag=4, kind='DIRNEU' /\n&BC_DIRNEU h='N', v='D' /\n"
        text = text.replace(blk, "").replace("&BC_DEF tag = 1", blk + "&BC_DEF tag = 1")
    dk = deck_from_parinp(text)
    assert dk.dirneu[0][3] == before
    P, d, g, o = run_both(dk, 250, precision)
    assert d.nflt == 161 and not d.flt_node2
    fg, fo = g.fault_series(), o.fault_series()
    assert fo[:, 0, :].max() > 0
    for rec in (0, 1, 2, 4):
        assert rel_l2(fg[:, rec, :], fo[:, rec, :]) <= TOL[precision], rec
    assert rel_l2(g.seismograms(), o.seismograms()) <= TOL[precision]
